"""The committed lookup tables are the generator's output."""

import os
import re
import sys

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "isoext_gb300", "csrc")
sys.path.insert(0, CSRC)
import gen_luts  # noqa: E402


def test_luts_header_is_current():
    with open(os.path.join(CSRC, "luts.h")) as fh:
        assert fh.read() == gen_luts.render()


def test_luts_counts():
    nag = gen_luts.expand(gen_luts.NAGAE, reflect=False)
    lor = gen_luts.expand(gen_luts.LORENSEN, reflect=True)
    assert max(len(t) for t in nag) == 5 and max(len(t) for t in lor) == 4
    st = gen_luts.edge_status(nag)
    assert st[0] == 0 and st[255] == 0 and all(st[i] for i in range(1, 255))


def _ref_table(path, name):
    s = open(path).read()
    i = s.index(name)
    body = re.sub(r"//.*", "", s[s.index("{", i) + 1: s.index("}", i)])
    return [int(x, 0) for x in re.findall(r"-?0b[01]+|-?\d+", body)]


def test_luts_equal_reference_fixture():
    """The generated tables equal the reference's, as stored by make_golden.py luts."""
    import numpy as np

    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "luts_ref.npz"))
    nag = gen_luts.flat(gen_luts.expand(gen_luts.NAGAE, False), 15)
    lor = gen_luts.flat(gen_luts.expand(gen_luts.LORENSEN, True), 12)
    assert nag == ref["nagae_tri"].tolist()
    assert lor == ref["lorensen_tri"].tolist()
    assert gen_luts.edge_status(gen_luts.expand(gen_luts.NAGAE, False)) == ref["edge_status"].tolist()


def test_luts_equal_reference_tables():
    """Same, read live from an isoext checkout named by $ISOEXT_REFERENCE."""
    ref = os.environ.get("ISOEXT_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "include")):
        pytest.skip("ISOEXT_REFERENCE does not name an isoext checkout")
    nag = gen_luts.flat(gen_luts.expand(gen_luts.NAGAE, False), 15)
    lor = gen_luts.flat(gen_luts.expand(gen_luts.LORENSEN, True), 12)
    assert nag == _ref_table(os.path.join(ref, "include/mc/nagae.cuh"), "tri_table[]")
    assert lor == _ref_table(os.path.join(ref, "include/mc/lorensen.cuh"), "tri_table[]")
    st = gen_luts.edge_status(gen_luts.expand(gen_luts.NAGAE, False))
    assert st == _ref_table(os.path.join(ref, "src/shared_luts.cu"), "edge_status_table[edge_table_size]")


def test_packed_triangle_lists_match_tables():
    for method, (table, width) in enumerate([(gen_luts.NAGAE, 15), (gen_luts.LORENSEN, 12)]):
        cases = gen_luts.expand(table, reflect=method == 1)
        flat = gen_luts.flat(cases, width)
        packed = gen_luts.packed(cases)
        for c in range(256):
            v = packed[c]
            n = v >> 60
            edges = [(v >> (4 * i)) & 15 for i in range(3 * n)]
            row = [e for e in flat[c * width:(c + 1) * width] if e >= 0]
            assert edges == row and n == len(cases[c])
