#!/usr/bin/env bash
# Build the reference's own marching-cubes / dual-contouring code for the host
# CPU (Thrust OpenMP backend) into oracle/_ref/libisoext_ref.so.
#
# The sources are compiled where they lie under the isoext checkout given as $1
# (required); nothing is copied.  src/isoext_ext.cu (nanobind) and
# src/batched_la.cu (cuSOLVER/cuBLAS, GPU only) are left out; ref_la_host.cpp
# stands in for the latter.  TEST INFRASTRUCTURE ONLY.
set -euo pipefail
REF="${1:?usage: build_ref.sh <isoext checkout>}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT/obj"
CUDA="${CUDA_HOME:-/usr/local/cuda}"
FLAGS=(-std=c++17 -O2 -fopenmp -fPIC -ffp-contract=off
       -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP
       -I"$CUDA/include" -I"$CUDA/include/cccl" -I"$REF/include")
SRCS=(utils.cu shared_luts.cu its.cu dc.cu ndarray.cu grid/uniform.cu grid/sparse.cu
      mc/mc.cu mc/base.cu mc/nagae.cu mc/lorensen.cu)
pids=()
objs=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr / _).o"
  objs+=("$o")
  g++ "${FLAGS[@]}" -x c++ -include "$HERE/ref_prelude.h" -c "$REF/src/$s" -o "$o" &
  pids+=($!)
done
for s in ref_driver.cpp ref_la_host.cpp; do
  o="$OUT/obj/${s%.cpp}.o"
  objs+=("$o")
  g++ "${FLAGS[@]}" -include "$HERE/ref_prelude.h" -c "$HERE/$s" -o "$o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libisoext_ref.so" "${objs[@]}" -L"$CUDA/lib64" -lcudart
echo "built $OUT/libisoext_ref.so"
