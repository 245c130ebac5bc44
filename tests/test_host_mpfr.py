"""The host division and square roots (restated MPFR arithmetic) against the
reference's own ::mp_div / ::mp_sqrt / ::mp_dsqrt on MPFR, bit for bit, for
every moduli set: converted doubles, long products and sums whose integers
exceed MP_PRECISION bits (so the rounding on input matters), ties, zeros and
negative zeros."""
import numpy as np
import pytest

import helpers
from oracle import ffi


def operands(oracle, n, rng, count):
    a = oracle.set_d(n, helpers.doubles(rng, count, -40, 40))
    b = oracle.set_d(n, helpers.doubles(rng, count, -40, 40))
    big = a.copy()
    for _ in range(6):  # grow the integers past MP_PRECISION bits
        big = oracle.add(n, oracle.mul(n, big, b), a)
    small_ints = oracle.set_d(n, rng.integers(1, 1 << 20, count).astype(float))
    xs = np.concatenate([a, big, small_ints, oracle.set_d(n, np.array([0.0, -0.0, 1.0, 4.0, 2.0, 0.25]))])
    ys = np.concatenate([b, a, small_ints[::-1].copy(), oracle.set_d(n, np.array([3.0, 3.0, 3.0, 1.0, 7.0, 9.0]))])
    return xs, ys


@pytest.mark.skipif(not ffi.ref_available(8), reason="the reference is not built here")
@pytest.mark.parametrize("n", [8, 16, 32])
def test_host_mpfr_ops_match_reference(library, oracle, n):
    rng = np.random.default_rng(helpers.SEED + 70 + n)
    x, y = operands(oracle, n, rng, 300)
    q, r, d = ffi.ref_div_sqrt(n, x, y)
    ax = x.copy()
    ax["sign"] = 0
    mq = library.div(n, x, y)
    assert len(ffi.mismatches(mq, q)) == 0, ffi.mismatches(mq, q)[:5]
    mr = library.sqrt(n, ax)
    assert len(ffi.mismatches(mr, r)) == 0
    md = library.dsqrt(n, ax)
    assert md.tobytes() == d.tobytes()


def test_host_mpfr_errors(library, oracle):
    one, zero = oracle.set_d(8, np.array([1.0])), oracle.set_d(8, np.array([0.0]))
    with pytest.raises(library.MpresError):
        library.div(8, one, zero)
    neg = oracle.set_d(8, np.array([-2.0]))
    with pytest.raises(library.MpresError):
        library.dsqrt(8, neg)
