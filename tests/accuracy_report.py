"""Maximum error of each benchmark configuration against exact rational
arithmetic (stronger than an MPFR run at twice the precision: every input is a
double, so every exact result is a dyadic rational held in Python integers).

    python tests/accuracy_report.py [--quick]

The results come from the oracle, which the parity tests pin bit for bit to
the CUDA path and to the reference, at the benchmark sizes (sampled outputs
for GEMM, GEMV and SpMV).  For each configuration it prints the largest
relative error |r - exact| / |exact| and the largest error relative to the sum
of absolute terms, |r - exact| / sum|terms|, next to the reference's a-priori
bound gamma_n = n u / (1 - n u), u = 4 / sqrt(M)
(tests/blas/accuracy/test_dot_accuracy.cu:39-90 of the reference)."""
import json
import math
import sys
from fractions import Fraction

import numpy as np

import helpers
from oracle import ffi

SEED = helpers.SEED


def exact_double(v):
    return Fraction(float(v))


def value(rec, mods):
    return helpers.mp_value(rec, mods)


def gamma(nmod, n):
    M = 1
    for m in helpers.moduli(nmod):
        M *= m
    u = Fraction(4, math.isqrt(M))
    return u * n / (1 - u * n)


def errors(pairs):
    """pairs of (result, exact, sum of |terms|) -> (max relative, max normalised)"""
    rel = max((abs(r - e) / abs(e) for r, e, s in pairs if e != 0), default=Fraction(0))
    nrm = max((abs(r - e) / s for r, e, s in pairs if s != 0), default=Fraction(0))
    return float(rel), float(nrm)


def dot_report(O, quick):
    n = 8
    count = 1 << (14 if quick else 20)
    rng = np.random.default_rng(SEED + 0)
    xd, yd = helpers.doubles(rng, count, -16, 16), helpers.doubles(rng, count, -16, 16)
    x, y = O.set_d(n, xd), O.set_d(n, yd)
    r = O.dot(n, x, y, g3=256, b3=64)
    terms = [exact_double(a) * exact_double(b) for a, b in zip(xd, yd)]
    ex = sum(terms, Fraction(0))
    s = sum((abs(t) for t in terms), Fraction(0))
    rel, nrm = errors([(value(r[0], helpers.moduli(n)), ex, s)])
    return {"config": "mp_dot n=%d, 8 moduli" % count, "max_rel": rel, "max_err_over_sum_abs": nrm,
            "gamma_n": float(gamma(n, count)), "outputs": 1}


def gemm_report(O, quick):
    n, m = 32, (128 if quick else 1024)
    rng = np.random.default_rng(SEED + 1)
    Ad, Bd, Cd = (helpers.doubles(rng, m * m, -32, 32) for _ in range(3))
    al, be = rng.uniform(-1, 1, 2)
    A, B, C = O.set_d(n, Ad), O.set_d(n, Bd), O.set_d(n, Cd)
    alpha, beta = O.set_d(n, np.array([al])), O.set_d(n, np.array([be]))
    mods = helpers.moduli(n)
    cols = 2 if not quick else 4  # full k = m chains for a few columns of C
    R = O.gemm(n, m, cols, m, alpha, A, m, B, m, beta, C[: m * cols], m)
    a, b = value(alpha[0], mods), value(beta[0], mods)
    pairs = []
    for c in range(cols):
        for r in range(0, m, max(1, m // 64)):
            terms = [a * exact_double(Ad[r + i * m]) * exact_double(Bd[i + c * m]) for i in range(m)]
            terms.append(b * exact_double(Cd[r + c * m]))
            pairs.append((value(R[r + c * m], mods), sum(terms, Fraction(0)), sum((abs(t) for t in terms), Fraction(0))))
    rel, nrm = errors(pairs)
    return {"config": "mp_gemm m=n=k=%d, 32 moduli (sampled C entries)" % m, "max_rel": rel,
            "max_err_over_sum_abs": nrm, "gamma_n": float(gamma(n, m + 3)), "outputs": len(pairs)}


def gemv_report(O, quick):
    n = 16
    sizes = np.clip(np.floor(np.exp(np.random.default_rng(SEED + 3).uniform(np.log(32), np.log(4097), (4096, 2)))),
                    32, 4096).astype(int)
    rng = np.random.default_rng(SEED + 31)
    mods = helpers.moduli(n)
    pairs, worst_n = [], 0
    for m, k in sizes[: (3 if quick else 12)]:
        m, k = int(min(m, 256 if quick else m)), int(k)
        Ad, xd, yd = helpers.doubles(rng, m * k, -32, 32), helpers.doubles(rng, k, -32, 32), helpers.doubles(rng, m, -32, 32)
        al, be = rng.uniform(-1, 1, 2)
        R = O.gemv(n, 111, m, k, O.set_d(n, np.array([al])), O.set_d(n, Ad), m, O.set_d(n, xd),
                   O.set_d(n, np.array([be])), O.set_d(n, yd), b3=32)
        a, b = Fraction(float(al)), Fraction(float(be))
        for r in range(0, m, max(1, m // 16)):
            terms = [a * exact_double(Ad[r + j * m]) * exact_double(xd[j]) for j in range(k)]
            terms.append(b * exact_double(yd[r]))
            pairs.append((value(R[r], mods), sum(terms, Fraction(0)), sum((abs(t) for t in terms), Fraction(0))))
        worst_n = max(worst_n, k)
    rel, nrm = errors(pairs)
    return {"config": "mp_gemv instances of the 4096-GEMV batch, 16 moduli (sampled rows)", "max_rel": rel,
            "max_err_over_sum_abs": nrm, "gamma_n": float(gamma(n, worst_n + 3)), "outputs": len(pairs)}


def spmv_report(O, quick):
    n, m = 8, 1 << (14 if quick else 20)
    rng = np.random.default_rng(SEED + 2)
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    xd = helpers.doubles(rng, m, -16, 16)
    y = O.spmv_csr(n, m, irp, ja, vals, O.set_d(n, xd))
    mods = helpers.moduli(n)
    pairs, longest = [], 0
    rows = list(range(0, m, max(1, m // 400))) + [int(np.argmax(np.diff(irp)))]
    for r in rows:
        terms = [exact_double(vals[i]) * exact_double(xd[ja[i]]) for i in range(irp[r], irp[r + 1])]
        longest = max(longest, len(terms))
        pairs.append((value(y[r], mods), sum(terms, Fraction(0)), sum((abs(t) for t in terms), Fraction(0))))
    rel, nrm = errors(pairs)
    return {"config": "mp_spmv_csr 2^%d rows, power-law, 8 moduli (sampled rows)" % int(math.log2(m)), "max_rel": rel,
            "max_err_over_sum_abs": nrm, "gamma_n": float(gamma(n, longest)), "outputs": len(pairs)}


def report(quick=False):
    O = ffi.oracle()
    return [f(O, quick) for f in (dot_report, gemm_report, gemv_report, spmv_report)]


if __name__ == "__main__":
    for row in report("--quick" in sys.argv[1:]):
        print(json.dumps(row))
