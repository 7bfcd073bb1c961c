"""Writes tests/golden/sdf_cases.npz: SDF values and normals of isoext's own sdf
module (src/isoext/sdf.py, imported from the reference checkout given as the
first argument) at seeded points, for the CPU tests of isoext_gb300.sdf.

    python tests/golden/make_sdf_golden.py <path to the isoext checkout>
"""

import importlib.util
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))
from test_sdf import CASES  # noqa: E402  (the same case list the test uses)


def main() -> None:
    src = os.path.join(sys.argv[1], "src", "isoext", "sdf.py")
    spec = importlib.util.spec_from_file_location("isoext_sdf", src)
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    g = torch.Generator().manual_seed(1234)
    p = torch.rand((4096, 3), generator=g) * 2.2 - 1.1
    rec = {"points": p.numpy()}
    for name, make in CASES.items():
        s = make(ref)
        rec[f"{name}_value"] = s(p).numpy()
        rec[f"{name}_normal"] = ref.get_sdf_normal(s, p.clone()).detach().numpy()
    np.savez_compressed(os.path.join(HERE, "sdf_cases.npz"), **rec)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
