"""Generate the marching-cubes lookup tables as a C header (``luts.h``).

The tables decide the output topology of marching cubes, so they must equal the
tables isoext ships (``include/mc/nagae.cuh``, ``include/mc/lorensen.cuh``,
``src/shared_luts.cu``).  They are produced here the way isoext's offline tool
produces them (``luts/gen_mc_lut.py:10-207``): a small set of base cases is
expanded by the 24 rotations of the cube, visited in a fixed order, optionally
followed by the inside/outside reflection; the first rotation that reaches a
case defines its triangles.  The base cases and the rotation order are data the
result depends on; everything else is computed here.

Case-string convention (as in the offline tool): an 8-character string whose
character ``k`` is the state of vertex ``k``; the table index is the string read
as a binary number, so character ``k`` is bit ``7-k`` of the index.

Run ``python isoext_gb300/csrc/gen_luts.py`` to rewrite ``luts.h``.
"""

from __future__ import annotations

import itertools
import pathlib

# Cube corners in Morton order (v = 4x + 2y + z) and the 12 edges as corner pairs
# (lower corner first).  Edge axis: 0..3 and 4..7 run along z or y, 8..11 along x.
EDGE_PAIRS = [(0, 1), (1, 3), (2, 3), (0, 2), (4, 5), (5, 7), (6, 7), (4, 6),
              (0, 4), (1, 5), (3, 7), (2, 6)]

# The 24 proper rotations of the cube as corner permutations, in the order the
# offline tool visits them (identity; face axes x, y, z; edge axes; vertex axes).
ROTATIONS = [
    [0, 1, 2, 3, 4, 5, 6, 7],
    [2, 0, 3, 1, 6, 4, 7, 5], [3, 2, 1, 0, 7, 6, 5, 4], [1, 3, 0, 2, 5, 7, 4, 6],
    [1, 5, 3, 7, 0, 4, 2, 6], [5, 4, 7, 6, 1, 0, 3, 2], [4, 0, 6, 2, 5, 1, 7, 3],
    [4, 5, 0, 1, 6, 7, 2, 3], [6, 7, 4, 5, 2, 3, 0, 1], [2, 3, 6, 7, 0, 1, 4, 5],
    [1, 0, 5, 4, 3, 2, 7, 6], [7, 3, 5, 1, 6, 2, 4, 0], [7, 6, 3, 2, 5, 4, 1, 0],
    [2, 6, 0, 4, 3, 7, 1, 5], [4, 6, 5, 7, 0, 2, 1, 3], [7, 5, 6, 4, 3, 1, 2, 0],
    [0, 4, 1, 5, 2, 6, 3, 7], [0, 2, 4, 6, 1, 3, 5, 7], [3, 1, 7, 5, 2, 0, 6, 4],
    [5, 1, 4, 0, 7, 3, 6, 2], [6, 4, 2, 0, 7, 5, 3, 1], [3, 7, 2, 6, 1, 5, 0, 4],
    [6, 2, 7, 3, 4, 0, 5, 1], [5, 7, 1, 3, 4, 6, 0, 2],
]

# Base cases: case string -> triangles (edge triples).  Lorensen & Cline (1987)
# uses 15 classes and allows reflection; Nagae's watertight table lists both
# signs explicitly and forbids reflection.
LORENSEN = {
    "00000000": [],
    "00000001": [[0, 8, 3]],
    "00010001": [[0, 7, 3], [0, 4, 7]],
    "00100001": [[0, 8, 3], [4, 9, 5]],
    "10000001": [[0, 8, 3], [5, 10, 6]],
    "01010100": [[3, 8, 4], [3, 4, 2], [2, 4, 6]],
    "10010001": [[0, 7, 3], [0, 4, 7], [5, 10, 6]],
    "10010010": [[4, 7, 8], [0, 1, 9], [5, 10, 6]],
    "01010101": [[0, 4, 6], [0, 6, 2]],
    "01001101": [[0, 10, 1], [0, 8, 10], [6, 10, 8], [6, 8, 7]],
    "11000011": [[1, 9, 3], [3, 9, 8], [5, 10, 11], [5, 11, 7]],
    "11000101": [[0, 8, 2], [2, 8, 5], [5, 8, 7], [2, 5, 10]],
    "01010110": [[0, 1, 9], [3, 8, 4], [3, 4, 2], [2, 4, 6]],
    "01101001": [[0, 8, 3], [1, 2, 10], [4, 9, 5], [6, 11, 7]],
    "01011100": [[1, 3, 8], [1, 6, 10], [1, 8, 6], [4, 6, 8]],
}
NAGAE = {
    "00000000": [],
    "00000001": [[0, 8, 3]],
    "00010001": [[0, 7, 3], [0, 4, 7]],
    "00100001": [[0, 8, 3], [4, 9, 5]],
    "10000001": [[0, 8, 3], [5, 10, 6]],
    "01010100": [[3, 8, 4], [3, 4, 2], [2, 4, 6]],
    "10010001": [[0, 7, 3], [0, 4, 7], [5, 10, 6]],
    "10010010": [[4, 7, 8], [0, 1, 9], [5, 10, 6]],
    "01010101": [[0, 4, 6], [0, 6, 2]],
    "01001101": [[0, 10, 1], [0, 8, 10], [6, 10, 8], [6, 8, 7]],
    "11000011": [[1, 9, 3], [3, 9, 8], [5, 10, 11], [5, 11, 7]],
    "11000101": [[0, 8, 2], [2, 8, 5], [5, 8, 7], [2, 5, 10]],
    "01010110": [[0, 1, 9], [3, 8, 4], [3, 4, 2], [2, 4, 6]],
    "10010110": [[0, 1, 9], [2, 3, 11], [4, 7, 8], [5, 10, 6]],
    "01011100": [[1, 3, 8], [1, 6, 10], [1, 8, 6], [4, 6, 8]],
    "01101101": [[0, 8, 1], [1, 8, 10], [7, 10, 8], [6, 10, 7], [4, 9, 5]],
    "01101110": [[0, 5, 4], [0, 10, 5], [0, 3, 10], [3, 6, 10], [3, 7, 6]],
    "10101011": [[3, 4, 8], [2, 4, 3], [2, 6, 4]],
    "01111110": [[0, 3, 8], [5, 6, 10]],
    "11011110": [[0, 3, 9], [3, 5, 9], [3, 4, 5], [3, 8, 4]],
    "11101110": [[0, 3, 4], [3, 7, 4]],
    "11111110": [[0, 3, 8]],
    "11111111": [],
}


def _edge_map(perm: list[int]) -> list[int]:
    """Edge permutation induced by a corner permutation."""
    index = {pair: i for i, pair in enumerate(EDGE_PAIRS)}
    out = []
    for a, b in EDGE_PAIRS:
        pa, pb = perm[a], perm[b]
        out.append(index[(min(pa, pb), max(pa, pb))])
    return out


def expand(base: dict[str, list[list[int]]], reflect: bool) -> list[list[list[int]]]:
    """All 256 cases, indexed by table index, from base cases."""
    edge_maps = [_edge_map(p) for p in ROTATIONS]
    cases: dict[str, list[list[int]]] = {}
    # The triangles used for a reflected case are those of the most recent
    # rotation that produced a *new* case; when a rotation lands on a case that
    # already exists they are not refreshed.  The shipped Lorensen table depends
    # on this, so it is kept.
    last_new: list[list[int]] = []
    for key, tris in base.items():
        for perm, emap in zip(ROTATIONS, edge_maps):
            # Vertex i of the rotated case takes the state of the corner that the
            # rotation sends to i.
            inv = [perm.index(i) for i in range(8)]
            rkey = "".join(key[inv[i]] for i in range(8))
            if rkey not in cases:
                last_new = [[emap[e] for e in t] for t in tris]
                cases[rkey] = last_new
            if reflect:
                fkey = "".join("1" if c == "0" else "0" for c in rkey)
                if fkey not in cases:
                    cases[fkey] = [t[::-1] for t in last_new]
    assert len(cases) == 256, f"{len(cases)} cases generated"
    return [cases[format(i, "08b")] for i in range(256)]


def edge_status(table: list[list[list[int]]]) -> list[int]:
    out = []
    for tris in table:
        mask = 0
        for e in itertools.chain.from_iterable(tris):
            mask |= 1 << e
        out.append(mask)
    return out


def flat(table: list[list[list[int]]], width: int) -> list[int]:
    out = []
    for tris in table:
        row = [e for t in tris for e in t]
        assert len(row) <= width
        out.extend(row + [-1] * (width - len(row)))
    return out


def packed(table: list[list[list[int]]]) -> list[int]:
    out = []
    for tris in table:
        edges = [e for t in tris for e in t]
        assert len(edges) <= 15
        v = len(tris) << 60
        for i, e in enumerate(edges):
            v |= e << (4 * i)
        out.append(v)
    return out


def ntri(table: list[list[list[int]]]) -> list[int]:
    return [len(row) for row in table]


def render() -> str:
    nag = expand(NAGAE, reflect=False)
    lor = expand(LORENSEN, reflect=True)
    st_n, st_l = edge_status(nag), edge_status(lor)
    assert st_n == st_l, "edge status must not depend on the table"

    def arr(name: str, ctype: str, vals: list[int], per_line: int) -> str:
        lines = []
        for i in range(0, len(vals), per_line):
            lines.append("    " + ", ".join(str(v) for v in vals[i:i + per_line]) + ",")
        return f"ISO_LUT_DECL {ctype} {name}[{len(vals)}] = {{\n" + "\n".join(lines) + "\n};\n"

    parts = [
        "/* Generated by gen_luts.py: do not edit. */\n",
        "#ifndef ISO_LUTS_H\n#define ISO_LUTS_H\n\n",
        "/* Storage class of the tables; CUDA sources define it as static __constant__ const. */\n",
        "#ifndef ISO_LUT_DECL\n#define ISO_LUT_DECL static const\n#endif\n\n",
        "/* Corner v = 4x + 2y + z.  Edge i joins ISO_EDGE_CORNERS[2i] < ISO_EDGE_CORNERS[2i+1]. */\n",
        arr("ISO_EDGE_CORNERS", "signed char", [c for p in EDGE_PAIRS for c in p], 8),
        "\n/* Bit e set when edge e carries a vertex for the case (same for both tables). */\n",
        arr("ISO_EDGE_STATUS", "unsigned short", st_n, 8),
        "\n/* Nagae: up to 5 triangles per case, edge triples, -1 padded. */\n",
        "#define ISO_NAGAE_MAX_TRI 5\n",
        arr("ISO_TRI_NAGAE", "signed char", flat(nag, 15), 15),
        "\n/* Lorensen: up to 4 triangles per case, edge triples, -1 padded. */\n",
        "#define ISO_LORENSEN_MAX_TRI 4\n",
        arr("ISO_TRI_LORENSEN", "signed char", flat(lor, 12), 12),
        "\n/* Triangles per case: [0, 256) Nagae, [256, 512) Lorensen. */\n",
        arr("ISO_NTRI", "unsigned char", ntri(nag) + ntri(lor), 16),
        "\n/* Each case's triangles in one word: edge of slot i in bits 4i .. 4i+3,\n"
        " * triangle count in bits 60 .. 63.  [0, 256) Nagae, [256, 512) Lorensen. */\n",
        arr("ISO_TRI_PACKED", "unsigned long long", [f"{v:#x}ull" for v in packed(nag) + packed(lor)], 4),
        "\n/* ISO_EDGE_CORNERS as a compile-time function, for fully unrolled loops. */\n",
        "#ifdef __cplusplus\n#ifdef __CUDACC__\n#define ISO_LUT_HD __host__ __device__\n#else\n",
        "#define ISO_LUT_HD\n#endif\n",
        "ISO_LUT_HD constexpr int iso_edge_corner(int i) {\n    return ",
        " : ".join(f"i == {i} ? {c}" for i, c in enumerate(c for p in EDGE_PAIRS for c in p)) + " : -1;\n}\n",
        "#endif\n",
        "\n#endif /* ISO_LUTS_H */\n",
    ]
    return "".join(parts)


def main() -> None:
    out = pathlib.Path(__file__).with_name("luts.h")
    out.write_text(render())
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
