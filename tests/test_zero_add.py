"""The zero-addition shortcut of the SpMV kernels (mp_device.cuh, zero_add_keeps):
mp_add(x, 0) and mp_add(0, x) return x bit for bit when x.exp <= 0, both
interval bounds are normalised (1 <= |frac| < 2) and x needs no rounding; 0 + 0
is 0.  Checked here on the oracle over the states a chain produces: converted
values with exponents up to +-300 and zeros, then generations of products, sums
(exact cancellations included) and products by doubles."""
import numpy as np
import pytest

import helpers


def mp_h(n):
    log2m = helpers.LOG2M[n]
    return -(log2m // 2) - 1 if log2m % 2 == 0 else -((log2m + 1) // 2)


@pytest.mark.parametrize("n", [8, 16, 32])
def test_zero_addition_identity(oracle, n):
    from oracle import ffi
    rng = np.random.default_rng(helpers.SEED + 2100 + n)
    cnt = 8000
    pools = []
    for lo, hi in ((-16, 16), (-60, 60), (-300, 300), (-2, 2)):
        v = helpers.doubles(rng, cnt, lo, hi)
        v[rng.random(cnt) < 0.02] = 0.0
        pools.append(oracle.set_d(n, v))
    cur = np.concatenate(pools)
    states = [cur]
    for gen in range(6):
        i, j = rng.integers(0, len(cur), cnt), rng.integers(0, len(cur), cnt)
        a, b = cur[i], cur[j]
        if gen % 3 == 0:
            r = oracle.mul(n, a, b)
        elif gen % 3 == 1:
            r = np.concatenate([oracle.add(n, a, b),
                                oracle.add(n, a[:500], oracle.mul_d(n, a[:500], np.full(500, -1.0)))])
        else:
            d = rng.standard_normal(cnt)
            d[rng.random(cnt) < 0.05] = 0.0
            r = oracle.mul_d(n, a, d)
        states.append(r)
        cur = np.concatenate([cur[-20000:], r])
    X = np.concatenate(states)
    zero = np.zeros(len(X), X.dtype)
    f0, f1 = np.abs(X["eval"][:, 0]["frac"]), np.abs(X["eval"][:, 1]["frac"])
    keeps = ((X["exp"] <= 0) & (f0 >= 1) & (f0 < 2) & (f1 >= 1) & (f1 < 2) & (X["eval"][:, 1]["exp"] < mp_h(n)))
    assert keeps.sum() > len(X) // 2
    r1, r2 = oracle.add(n, X, zero), oracle.add(n, zero, X)
    assert len(ffi.mismatches(r1[keeps], X[keeps])) == 0
    assert len(ffi.mismatches(r2[keeps], X[keeps])) == 0
    assert len(ffi.mismatches(oracle.add(n, zero[:4], zero[:4]), zero[:4])) == 0
    # the rejected kinds do change somewhere (the conditions are not vacuous)
    assert len(ffi.mismatches(r1[~keeps], X[~keeps])) > 0
