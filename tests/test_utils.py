"""write_obj writes isoext's OBJ text (src/isoext/utils.py:42-63): one ``v x y z``
line per vertex with Python's float formatting of each FP32 value, then one
``f a b c`` line per face with 1-based indices; an empty or missing mesh gives
an empty file."""

import numpy as np
import torch

from isoext_gb300.utils import write_obj


def _parse(path):
    v, f = [], []
    with open(path) as fh:
        for line in fh:
            tag, *rest = line.split()
            if tag == "v":
                v.append([float(x) for x in rest])
            elif tag == "f":
                f.append([int(x) for x in rest])
    return np.asarray(v, np.float32).reshape(-1, 3), np.asarray(f, np.int64).reshape(-1, 3)


def test_write_obj_text_and_round_trip(tmp_path):
    g = np.random.default_rng(3)
    v = torch.from_numpy(g.uniform(-1, 1, size=(7, 3)).astype(np.float32))
    v[0] = torch.tensor([0.1, -0.0, 1e-30])  # repr of FP32 values widened to float
    f = torch.from_numpy(g.integers(0, 7, size=(5, 3)).astype(np.int32))
    p = tmp_path / "m.obj"
    write_obj(str(p), v, f)
    text = p.read_text()
    lines = text.splitlines()
    assert len(lines) == 12
    assert lines[0] == f"v {float(np.float32(0.1))} -0.0 {float(np.float32(1e-30))}"
    assert lines[7] == "f " + " ".join(str(int(i) + 1) for i in f[0])
    assert all(line.startswith("v ") for line in lines[:7]) and all(line.startswith("f ") for line in lines[7:])
    vr, fr = _parse(p)
    np.testing.assert_array_equal(vr, v.numpy())  # the decimal text round-trips FP32 exactly
    np.testing.assert_array_equal(fr, f.numpy().astype(np.int64) + 1)


def test_write_obj_empty_and_missing_meshes(tmp_path):
    for v, f in [(None, None), (torch.zeros(0, 3), torch.zeros(0, 3, dtype=torch.int32)),
                 (torch.ones(3, 3), torch.zeros(0, 3, dtype=torch.int32)), (torch.ones(3, 3), None)]:
        p = tmp_path / "e.obj"
        p.write_text("stale")
        write_obj(str(p), v, f)
        assert p.read_text() == ""


def test_make_grid_on_the_host():
    """tests/test_grid_utils.py:11-37 on the CPU: [X, Y, Z, 3] point coordinates,
    corners at the box's corners, per-axis resolutions."""
    from isoext_gb300.utils import make_grid

    grid = make_grid([-1, -1, -1, 1, 1, 1], res=16, device="cpu")
    assert grid.shape == (16, 16, 16, 3) and grid.device.type == "cpu"
    assert torch.equal(grid[0, 0, 0], torch.tensor([-1.0, -1.0, -1.0]))
    assert torch.allclose(grid[-1, -1, -1], torch.tensor([1.0, 1.0, 1.0]), atol=1e-5)
    grid = make_grid([0, -2, 1, 1, 2, 3], res=[4, 5, 6], device="cpu")
    assert grid.shape == (4, 5, 6, 3)
    assert torch.allclose(grid[:, 0, 0, 0], torch.linspace(0, 1, 4))
    assert torch.allclose(grid[0, :, 0, 1], torch.linspace(-2, 2, 5))
    assert torch.allclose(grid[0, 0, :, 2], torch.linspace(1, 3, 6))
