"""Shared helpers of the test-suite: paths, seeded inputs shaped like the
benchmark configurations, exact decoding of RNS numbers, and error bounds."""
import math
import pathlib
import re
import sys
from fractions import Fraction

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
PKG = ROOT / "mpres-blas_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

LOG2M = {8: 242, 16: 482, 32: 962}
SEED = 0x4D505245  # seed of configuration c is SEED + c


def moduli(nmod):
    text = (PKG / "csrc" / "moduli_sets.h").read_text()
    m = re.search(r"#define MPRES_SET%d_MODULI \{([^}]*)\}" % nmod, text)
    return [int(v) for v in m.group(1).replace("\\", " ").replace("\n", " ").split(",")]


from workloads import csr_to_ell, doubles, power_law_rows, random_csr  # noqa: E402,F401


def crt(digits, mods):
    M = 1
    for m in mods:
        M *= m
    X = 0
    for d, m in zip(digits, mods):
        Mi = M // m
        X += int(d) * Mi * pow(Mi, -1, m)
    return X % M


def mp_value(rec, mods):
    """Exact value of one mp_float_t record as a Fraction."""
    X = crt(rec["digits"], mods)
    v = Fraction(X) * (Fraction(2) ** int(rec["exp"]))
    return -v if int(rec["sign"]) else v


def exact_dot(x, y):
    return sum((Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y)), Fraction(0))


def dot_bound(nmod, n, x, y):
    """The reference's a-priori bound (tests/blas/accuracy/test_dot_accuracy.cu:39-90):
    |r - exact| <= u*n/(1 - u*n) * sum|x_i*y_i| with u = 4/sqrt(M)."""
    M = 1
    for m in moduli(nmod):
        M *= m
    u = Fraction(4, math.isqrt(M))  # >= 4/sqrt(M): the bound only loosens
    s = sum((abs(Fraction(float(a)) * Fraction(float(b))) for a, b in zip(x, y)), Fraction(0))
    return u * n / (1 - u * n) * s
