"""Seeded MatrixMarket inputs shared by the ingest tests: decimal spellings
whose correct rounding is hard, and random coordinate files."""
from __future__ import annotations

import decimal

import numpy as np


def _random_double(rng) -> float:
    while True:
        x = np.array([rng.integers(0, 1 << 63, dtype=np.uint64)], np.uint64).view(np.float64)[0]
        if np.isfinite(x):
            return float(x)


def _midpoint(a: float) -> str:
    """Exact decimal of the midpoint between a > 0 and the next double."""
    b = float(np.nextafter(a, np.inf))
    with decimal.localcontext() as ctx:
        ctx.prec = 1200
        mid = (decimal.Decimal(a) + decimal.Decimal(b)) / 2
    return format(mid, "E")


def hard_decimals(count: int, seed: int = 5) -> list[str]:
    """count decimal strings mixing every kind of rounding difficulty."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        k = i % 9
        x = _random_double(rng)
        if k == 0:
            s = repr(x)
        elif k == 1:
            s = f"{x:.{int(rng.integers(0, 30))}e}"
        elif k == 2:  # random digit strings of up to 40 digits, any exponent
            nd = int(rng.integers(1, 41))
            digits = "".join(str(d) for d in rng.integers(0, 10, nd))
            p = int(rng.integers(0, nd + 1))
            s = digits[:p] + "." + digits[p:] + f"e{int(rng.integers(-360, 331))}"
            if s.startswith("."):
                s = "0" + s
        elif k == 3:  # exact midpoints: ties to even
            s = _midpoint(abs(x) or 5e-324)
        elif k == 4:  # a hair above or below a midpoint
            m = _midpoint(abs(x) or 5e-324)
            mant, ex = m.split("E")
            if rng.random() < 0.5:
                s = mant + "000001E" + ex if "." in mant else mant + ".000001E" + ex
            else:
                d = decimal.Decimal(m)
                with decimal.localcontext() as ctx:
                    ctx.prec = 1300
                    s = format(d - d.scaleb(-1100), "E")
        elif k == 5:  # subnormals
            sub = float(np.array([rng.integers(1, 1 << 52, dtype=np.uint64)], np.uint64).view(np.float64)[0])
            s = repr(sub) if rng.random() < 0.5 else f"{sub:.{int(rng.integers(0, 25))}e}"
        elif k == 6:  # integers up to 2^64 and beyond
            s = str(int(rng.integers(0, 1 << 62)) * int(rng.integers(1, 9)))
        elif k == 7:  # short everyday spellings
            s = f"{int(rng.integers(0, 1000))}.{int(rng.integers(0, 1000)):03d}e{int(rng.integers(-25, 26))}"
        else:  # powers of ten and their neighbours across the whole range
            e = int(rng.integers(-340, 309))
            s = rng.choice(["1e%d", "9.999999999999999e%d", "1.0000000000000001e%d", "5e%d"]) % e
        if rng.random() < 0.3 and not s.startswith("-"):
            s = "-" + s
        out.append(s)
    return out


def write_value_file(path, values) -> None:
    """One value per row: (i+1, 1, values[i]) in an m x 1 real file."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{len(values)} 1 {len(values)}\n")
        for i, s in enumerate(values):
            f.write(f"{i + 1} 1 {s}\n")


def write_random(path, m, n, nnz, field="real", storage="general", seed=0) -> None:
    """A seeded random coordinate file (lower triangle for symmetric kinds)."""
    rng = np.random.default_rng(seed)
    r = rng.integers(1, m + 1, nnz)
    c = rng.integers(1, n + 1, nnz)
    if storage != "general":
        r, c = np.maximum(r, c), np.minimum(r, c)
        if storage == "skew-symmetric":
            keep = r != c
            r, c = r[keep], c[keep]
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {storage}\n% seeded\n{m} {n} {len(r)}\n")
        for i in range(len(r)):
            if field == "pattern":
                f.write(f"{r[i]} {c[i]}\n")
            elif field == "integer":
                f.write(f"{r[i]} {c[i]} {int(rng.integers(-1000, 1000))}\n")
            elif field == "complex":
                f.write(f"{r[i]} {c[i]} {rng.standard_normal():.17g} {rng.standard_normal():.17g}\n")
            else:
                f.write(f"{r[i]} {c[i]} {rng.standard_normal() * 10.0 ** rng.integers(-5, 6):.17g}\n")
