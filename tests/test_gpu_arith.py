"""The device arithmetic on its own (mp_add, mp_mul, mp_mul_d, power-of-two
scaling, interval evaluation) against the reference's golden vectors and the
oracle, for every moduli set, through the element-wise C entry points."""
import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu
GOLD = helpers.ROOT / "tests" / "golden"


def eq(a, b):
    mm = ffi.mismatches(a, b)
    assert len(mm) == 0, "%d of %d records differ, first at %d" % (len(mm), len(a), mm[0])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_elementwise_golden(gpu, n):
    g = np.load(GOLD / ("elem_%d.npz" % n))
    ew = gpu.elementwise
    eq(ew(n, gpu.OP_MUL, g["mx"], g["my"]), g["prod"])
    eq(ew(n, gpu.OP_ADD, g["mx"], g["my"]), g["sum"])
    eq(ew(n, gpu.OP_MUL_D, g["mx"], g["d"]), g["q"])
    eq(ew(n, gpu.OP_ADD, g["mx"], g["q"]), g["canc"])
    acc = g["prod"].copy()
    for _ in range(6):
        acc = ew(n, gpu.OP_ADD, ew(n, gpu.OP_MUL, acc, g["my"]), g["prod"])
    eq(acc, g["acc"])
    eq(ew(n, gpu.OP_MUL_D, g["acc"], g["dd"]), g["muld"])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_random_chains_vs_oracle(gpu, oracle, n):
    """Mixed products and sums with exponents spread over +-60, so that roundings of
    several 30-bit scaling steps and ambiguous signs occur."""
    rng = np.random.default_rng(helpers.SEED + 900 + n)
    cnt = 20000
    pool = gpu.set_d(n, helpers.doubles(rng, cnt, -60, 60))
    for gen in range(9):
        i, j = rng.integers(0, len(pool), cnt), rng.integers(0, len(pool), cnt)
        a, b = pool[i].copy(), pool[j].copy()
        if gen % 3 == 0:
            got, want = gpu.elementwise(n, gpu.OP_MUL, a, b), oracle.mul(n, a, b)
        elif gen % 3 == 1:
            got, want = gpu.elementwise(n, gpu.OP_ADD, a, b), oracle.add(n, a, b)
        else:
            d = -(1 + np.ldexp(rng.integers(1, 1 << 20, cnt).astype(float), -52 - rng.integers(0, 20, cnt)))
            got, want = gpu.elementwise(n, gpu.OP_MUL_D, a, d), oracle.mul_d(n, a, d)
        eq(got, want)
        pool = np.concatenate([pool, want])[-60000:]


@pytest.mark.parametrize("n", [8, 16, 32])
def test_scale2pow_vs_oracle(gpu, oracle, n):
    rng = np.random.default_rng(helpers.SEED + 910 + n)
    digits = rng.integers(0, 1 << 30, (20000, n)).astype(np.int32)
    D = rng.integers(0, helpers.LOG2M[n], 20000).astype(np.uint32)
    D[:64] = np.arange(64)  # every step split around the 30-bit threshold
    assert gpu.rns_scale2pow(n, digits, D).tobytes() == oracle.scale2pow(n, digits, D).tobytes()


@pytest.mark.parametrize("n", [8, 16, 32])
@pytest.mark.parametrize("fast", [0, 1])
def test_eval_vs_oracle(gpu, oracle, n, fast):
    rng = np.random.default_rng(helpers.SEED + 920 + n)
    big = rng.integers(0, 1 << 30, (20000, n)).astype(np.int32)
    small = gpu.set_d(n, helpers.doubles(rng, 20000, -20, 20))["digits"].copy()
    for digits in (big, small):
        lo1, up1 = gpu.rns_eval(n, digits, fast)
        lo2, up2 = (oracle.eval_fast if fast else oracle.eval)(n, digits)
        assert lo1.tobytes() == lo2.tobytes() and up1.tobytes() == up2.tobytes()
