"""Generate tests/golden/*.npz from the reference's own code.

Runs the isoext sources compiled for the host CPU (oracle/build_ref.sh ->
oracle/_ref/libisoext_ref.so) on small seeded inputs and stores inputs and
outputs.  Run here, where the isoext checkout exists:

    python tests/golden/make_golden.py
    python tests/golden/make_golden.py luts <isoext checkout>   # luts_ref.npz

The GPU machine has no isoext sources; tests there read these files.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from helpers import axis_coords, grid_points, noise, sphere, torus  # noqa: E402
from oracle import Reference  # noqa: E402


def dense_cases():
    out = {}
    out["sphere20"] = dict(values=sphere((20, 20, 20), 0.6), level=0.0)
    out["torus24"] = dict(values=torus((24, 24, 24), 0.5, 0.2), level=0.05)
    out["noise12"] = dict(values=noise((12, 12, 12), seed=1, zero_frac=0.2), level=0.0)
    out["aniso"] = dict(values=sphere((9, 17, 13), 0.7), level=0.0)
    # plane x = 0: exact zeros on a grid plane, vertices weld onto grid points
    v = np.broadcast_to(axis_coords(17)[:, None, None], (17, 17, 17)).astype(np.float32).copy()
    out["plane17"] = dict(values=v, level=0.0)
    # FLT_MAX outside a box: crossings round onto the finite corner
    v = sphere((16, 16, 16), 0.5)
    v[:3] = np.finfo(np.float32).max
    v[:, 12:] = np.finfo(np.float32).max
    out["fltmax16"] = dict(values=v, level=0.0)
    return out


def sparse_case(shape=(16, 16, 16), r=0.55):
    """Cells whose 8 corners straddle the level; values from the sphere SDF."""
    n = np.asarray(shape)
    p = grid_points(shape)
    d = (np.sqrt((p * p).sum(-1)) - np.float32(r)).astype(np.float32)
    cx, cy, cz = np.meshgrid(*[np.arange(k - 1) for k in shape], indexing="ij")
    vals = np.stack([d[cx + (k >> 2), cy + ((k >> 1) & 1), cz + (k & 1)] for k in range(8)], -1)
    neg = (vals < 0).sum(-1)
    keep = (neg > 0) & (neg < 8)
    ids = ((cx * (n[1] - 1) + cy) * (n[2] - 1) + cz)[keep].astype(np.int32)
    order = np.argsort(ids)
    return ids[order], vals[keep][order].astype(np.float32)


def _c_table(path: str, name: str) -> list[int]:
    """The integers of a C array initialiser ``name = { ... }`` in a source file."""
    import re

    s = open(path).read()
    i = s.index(name)
    body = re.sub(r"//.*", "", s[s.index("{", i) + 1: s.index("}", i)])
    return [int(x, 0) for x in re.findall(r"-?0b[01]+|-?\d+", body)]


def write_luts(checkout: str) -> None:
    """Store the reference's MC tables (read from its sources) as luts_ref.npz."""
    j = os.path.join
    rec = {
        "nagae_tri": _c_table(j(checkout, "include/mc/nagae.cuh"), "tri_table[]"),
        "lorensen_tri": _c_table(j(checkout, "include/mc/lorensen.cuh"), "tri_table[]"),
        "edge_status": _c_table(j(checkout, "src/shared_luts.cu"), "edge_status_table[edge_table_size]"),
    }
    np.savez_compressed(j(HERE, "luts_ref.npz"), **{k: np.asarray(v, np.int32) for k, v in rec.items()})
    print("luts_ref", {k: len(v) for k, v in rec.items()})


def main() -> None:
    if len(sys.argv) == 3 and sys.argv[1] == "luts":
        write_luts(sys.argv[2])
        return
    ref = Reference()
    for name, c in dense_cases().items():
        rec = {"values": c["values"], "level": np.float32(c["level"])}
        for m in ["nagae", "lorensen"]:
            v, f = ref.mc_dense(c["values"], level=c["level"], method=m)
            rec[f"mc_{m}_v"], rec[f"mc_{m}_f"] = v, f
        if name in ("sphere20", "torus24", "aniso"):
            v, f = ref.dc_dense(c["values"], level=c["level"])
            rec["dc_v"], rec["dc_f"] = v, f
            its = ref.intersection_dense(c["values"], level=c["level"], normals=True)
            for k, a in its.items():
                rec[f"its_{k}"] = a
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, {k: getattr(a, "shape", ()) for k, a in rec.items() if k.endswith(("_v", "_f"))})
    # dual contouring of a cuboid with sharp edges (QEF solve exercised)
    p = grid_points((24, 24, 24))
    q = np.abs(p) - np.float32(0.5)
    qm = q.max(-1)
    cub = (np.sqrt((np.maximum(q, 0) ** 2).sum(-1)) + np.minimum(qm, 0)).astype(np.float32)
    v, f = ref.dc_dense(cub)
    np.savez_compressed(os.path.join(HERE, "cuboid24.npz"), values=cub, level=np.float32(0),
                        dc_v=v, dc_f=f)
    print("cuboid24", v.shape, f.shape)
    ids, vals = sparse_case()
    rec = {"cell_ids": ids, "values": vals, "shape": np.array([16, 16, 16], np.int32)}
    for m in ["nagae", "lorensen"]:
        v, f = ref.mc_sparse(ids, vals, (16, 16, 16), method=m)
        rec[f"mc_{m}_v"], rec[f"mc_{m}_f"] = v, f
    v, f = ref.dc_sparse(ids, vals, (16, 16, 16))
    rec["dc_v"], rec["dc_f"] = v, f
    np.savez_compressed(os.path.join(HERE, "sparse16.npz"), **rec)
    print("sparse16", len(ids), v.shape, f.shape)


if __name__ == "__main__":
    main()
