"""Writes the MatrixMarket fixtures tests/golden/mtx/*.mtx and, for each, the
CSR the reference's own reader produces (mmio_allinone, src/auxiliary.h:64-232,
compiled from the reference sources into oracle/_ref/) as
tests/golden/mtx/<name>.npz (m, n, nnz, is_symmetric, rowptr, colidx, val).

The files are small hand-made cases covering what the reader must agree on:
every data type and storage scheme, comments and blank lines, CRLF and tab
separators, entries split across lines, tokens past the header's entry
count, duplicates, empty rows, and value spellings whose rounding is hard
(more than 19 digits, halfway cases, subnormals, the extremes of binary64).
Run from the repo root:

    make -C oracle all ref REF_SRC=<checkout>/src && python tests/golden/make_mtx.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, "tests", "golden", "mtx")

HARD_VALUES = [
    "1.5", "-2e-3", "3.", ".25", "1E+2", "-0", "0.1", "0.30000000000000004",
    "9007199254740993",                 # 2^53 + 1: a tie, rounds to even
    "9007199254740995",                 # 2^53 + 3: a tie, rounds up
    "1234567890123456789012",           # 22 digits
    "0.1000000000000000055511151231257827021181583404541015625",  # exactly the double 0.1
    "0.10000000000000000555111512312578270211815834045410156251",  # just above it
    "2.2250738585072011e-308",          # just below the smallest normal
    "2.2250738585072014e-308",          # the smallest normal
    "4.9406564584124654e-324",          # the smallest subnormal
    "2.4703282292062327e-324",          # below half of it: rounds to zero
    "2.4703282292062328e-324",          # above half of it: rounds up
    "1.7976931348623157e308",           # the largest double
    "1.7976931348623158e308",           # still rounds to it
    "1.7976931348623159e308",           # past the midpoint: infinity
    "1e23", "8.589973e9", "123456789e-5", "-7.2057594037927933e16",
    "1e-400", "1e400", "-1e-400", "0.000000000000000000000000000000000000000001e42",
    "1.00000000000000011102230246251565404236316680908203125",  # 1 + half ulp: tie to even (1)
    "1.00000000000000011102230246251565404236316680908203126",  # just above: 1 + ulp
    "inf", "-Infinity", "nan",
]


def fmt_entries(entries, field):
    lines = []
    for e in entries:
        lines.append(" ".join(str(t) for t in e))
    return "\n".join(lines) + "\n"


def cases() -> dict[str, str]:
    c = {}
    # real general: duplicates, empty rows/columns, hard values
    ents = [(1 + (i * 7) % 9, 1 + (i * 5) % 6, HARD_VALUES[i]) for i in range(len(HARD_VALUES))]
    ents += [(2, 3, "1.25"), (2, 3, "-1.25")]  # duplicate position
    c["real_general"] = ("%%MatrixMarket matrix coordinate real general\n% hard value spellings\n%\n"
                         f"9 6 {len(ents)}\n" + fmt_entries(ents, "real"))
    # symmetric real: lower triangle with diagonal, file order not sorted
    ents = [(3, 1, "0.5"), (1, 1, "4"), (5, 2, "-1.5e-1"), (2, 2, "4"), (4, 4, "4"), (5, 5, "2.5"),
            (4, 3, "-3"), (3, 3, "4"), (5, 1, "7e0")]
    c["real_symmetric"] = ("%%MatrixMarket matrix coordinate real symmetric\n"
                           f"5 5 {len(ents)}\n" + fmt_entries(ents, "real"))
    ents = [(2, 1), (3, 1), (3, 2), (4, 4), (6, 1), (6, 5), (5, 5)]
    c["pattern_symmetric"] = ("%%MatrixMarket matrix coordinate pattern symmetric\n"
                              f"6 6 {len(ents)}\n" + fmt_entries(ents, "pattern"))
    ents = [(1, 2, "+5"), (4, 1, "-12"), (2, 2, "0"), (3, 4, "2147483647"), (1, 2, "-2147483648")]
    c["integer_general"] = ("%%MatrixMarket matrix coordinate integer general\n"
                            f"4 4 {len(ents)}\n" + fmt_entries(ents, "integer"))
    ents = [(1, 1, "2.0", "0"), (2, 1, "1.5", "-0.5"), (3, 2, "-1e-3", "2"), (3, 3, "1", "0")]
    c["complex_hermitian"] = ("%%MatrixMarket matrix coordinate complex hermitian\n"
                              f"3 3 {len(ents)}\n" + fmt_entries(ents, "complex"))
    ents = [(2, 1, "1.5"), (3, 1, "-2"), (3, 2, "0.25")]
    c["real_skew"] = ("%%MatrixMarket matrix coordinate real skew-symmetric\n"
                      f"3 3 {len(ents)}\n" + fmt_entries(ents, "real"))
    # whitespace: CRLF, tabs, runs of blanks, a blank line before the size
    # line, entries split across lines, extra tokens after the last entry
    c["whitespace"] = ("%%MatrixMarket Matrix COORDINATE Real General\r\n% comment\r\n\r\n"
                       "  4 5\t3 \r\n"
                       "1\t1  1.0\r\n\r\n  2 3\r\n-2.5e+0\r\n4 5 \t 3.25   \r\n7 7 7 extra tokens\r\n")
    c["empty"] = "%%MatrixMarket matrix coordinate real general\n5 4 0\n"
    ents = [(1, 4, "1"), (6, 1, "2"), (6, 4, "3")]
    c["rect_empty_rows"] = ("%%MatrixMarket matrix coordinate real general\n"
                            f"7 4 {len(ents)}\n" + fmt_entries(ents, "real"))
    # a larger seeded one: 400 x 300, 3000 entries, mixed spellings
    rng = np.random.default_rng(11)
    r = rng.integers(1, 401, 3000)
    cc = rng.integers(1, 301, 3000)
    v = rng.standard_normal(3000) * 10.0 ** rng.integers(-30, 30, 3000)
    spell = []
    for i, x in enumerate(v):
        k = i % 4
        spell.append(repr(float(x)) if k == 0 else f"{x:.6e}" if k == 1 else f"{x:.25e}" if k == 2 else f"{x:.3f}")
    ents = list(zip(r, cc, spell))
    c["seeded_general"] = ("%%MatrixMarket matrix coordinate real general\n"
                           f"400 300 {len(ents)}\n" + fmt_entries(ents, "real"))
    return c


def main() -> None:
    from oracle import ref

    os.makedirs(OUT, exist_ok=True)
    for name, text in cases().items():
        path = os.path.join(OUT, name + ".mtx")
        with open(path, "w", newline="") as f:
            f.write(text)
        m, n, nnz, sym, rp, ci, v = ref.mmio_read(path)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), m=m, n=n, nnz=nnz, is_symmetric=sym, rowptr=rp,
                            colidx=ci, val=v)
        print(f"{name}: {m}x{n} nnz={nnz} symmetric={sym}")


if __name__ == "__main__":
    main()
