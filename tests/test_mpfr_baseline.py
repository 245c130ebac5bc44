"""The reference's MPFR/OpenMP CPU loops (oracle/mpfr_blas.c), timed as the CPU
baseline: results of mpfr_dot / mpfr_gemm / mpfr_mpspmv_csr restated in C
against exact rational arithmetic, within the error of round-to-nearest MPFR
arithmetic at MP_PRECISION bits."""
from fractions import Fraction

import numpy as np
import pytest

import helpers
from oracle import ffi


@pytest.fixture(scope="module")
def mpfr():
    lib = ffi.mpfr_blas()
    if lib is None:
        pytest.skip("libmpfr.so.6 not available on this host")
    return lib


def close(got, exact, scale, bits, terms):
    # each of the `terms` roundings errs by at most 2^-bits of a partial result,
    # bounded by the sum of magnitudes `scale`; plus the final rounding to double
    err = abs(Fraction(got) - exact)
    return err <= scale * terms * Fraction(1, 2 ** bits) + abs(exact) * Fraction(1, 2 ** 52)


def test_mpfr_dot(mpfr):
    rng = np.random.default_rng(helpers.SEED + 501)
    n = 4000
    x, y = helpers.doubles(rng, n, -16, 16), helpers.doubles(rng, n, -16, 16)
    for threads in (1, 4):
        t, r = mpfr.dot(x, y, 120, threads)
        assert t >= 0
        exact = helpers.exact_dot(x, y)
        scale = sum(abs(Fraction(float(a)) * Fraction(float(b))) for a, b in zip(x, y))
        assert close(r, exact, scale, 120, 2 * n + threads)


def test_mpfr_gemm_block(mpfr):
    rng = np.random.default_rng(helpers.SEED + 502)
    m = k = 40
    A, B, C = (helpers.doubles(rng, m * m, -32, 32) for _ in range(3))
    alpha, beta = 0.75, -0.3125
    rows, cols = 7, 5
    t, out = mpfr.gemm(rows, cols, k, alpha, A, m, B, m, beta, C, m, 480, 3)
    for c in range(cols):
        for r in range(rows):
            terms = [Fraction(float(A[i * m + r])) * Fraction(float(B[c * m + i])) for i in range(k)]
            exact = Fraction(alpha) * sum(terms, Fraction(0)) + Fraction(beta) * Fraction(float(C[c * m + r]))
            scale = sum(abs(v) for v in terms) + abs(Fraction(beta) * Fraction(float(C[c * m + r])))
            assert close(out[c * rows + r], exact, scale, 480, 2 * k + 3)


def test_mpfr_spmv_csr(mpfr):
    rng = np.random.default_rng(helpers.SEED + 503)
    m = 300
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m, kmax=40))
    x = helpers.doubles(rng, m, -16, 16)
    t, y = mpfr.spmv_csr(m, irp, ja, vals, x, 120, 2)
    for r in range(m):
        terms = [Fraction(float(vals[i])) * Fraction(float(x[ja[i]])) for i in range(irp[r], irp[r + 1])]
        exact = sum(terms, Fraction(0))
        assert close(y[r], exact, sum(abs(v) for v in terms), 120, 2 * len(terms) + 1)
