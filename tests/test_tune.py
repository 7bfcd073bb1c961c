"""The autotuner's persistent cache (host logic; the timing itself is tested on
the GPU in test_mc_gpu.py and test_sparse_gpu.py)."""

import json

from isoext_gb300 import tune


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    k1 = tune.cache_key("mc", (512, 512, 512), 0.0, gpu="NVIDIA GB300")
    k2 = tune.cache_key("dc", (256, 256, 256), 0.25, gpu="NVIDIA GB300")
    assert k1 != k2 and "512x512x512" in k1 and "NVIDIA GB300" in k1
    assert tune.cache_lookup(path, k1) is None
    rep = {"best": {"mc.emit_threads": 256}, "ms": {"mc.emit_threads": {"128": 0.2, "256": 0.1}}}
    tune.cache_store(path, k1, rep)
    tune.cache_store(path, k2, {"best": {"dc.cell_threads": 128}, "ms": {}})
    assert tune.cache_lookup(path, k1) == rep
    assert tune.cache_lookup(path, k2)["best"] == {"dc.cell_threads": 128}
    assert set(json.load(open(path))) == {k1, k2}


def test_cache_path_choice(tmp_path, monkeypatch):
    monkeypatch.delenv(tune.CACHE_ENV, raising=False)
    assert tune.cache_path(None) is None
    assert tune.cache_path(str(tmp_path / "a.json")) == str(tmp_path / "a.json")
    assert tune.cache_path(True).endswith("tune.json")
    monkeypatch.setenv(tune.CACHE_ENV, str(tmp_path / "env.json"))
    assert tune.cache_path(None) == str(tmp_path / "env.json")
    assert tune.cache_path(True) == str(tmp_path / "env.json")


def test_unreadable_cache_is_a_miss(tmp_path):
    path = tmp_path / "bad.json"
    path.write_text("{not json")
    assert tune.cache_lookup(str(path), "k") is None
    tune.cache_store(str(path), "k", {"best": {}, "ms": {}})
    assert tune.cache_lookup(str(path), "k") == {"best": {}, "ms": {}}


def test_populate_brick_setting():
    old = tune.populate_brick()
    try:
        tune.set_populate_brick(16)
        assert tune.populate_brick() == 16
    finally:
        tune.set_populate_brick(old)


def test_choose_keeps_the_incumbent_within_the_margin():
    # a value within MARGIN of the fastest does not displace the one in force
    assert tune.choose({128: 1.00, 256: 1.01}, 256) == 256
    assert tune.choose({128: 1.00, 256: 1.00 / (1 - tune.MARGIN) + 0.01}, 256) == 128
    # an incumbent the knob does not offer: the fastest
    assert tune.choose({8: 2.0, 16: 1.5, 32: 1.7}, 64) == 16
    assert tune.choose({8: 2.0, 16: 1.5, 32: 1.7}, 32) == 16
    assert tune.choose({8: 2.0, 16: 1.69, 32: 1.7}, 32) == 32
