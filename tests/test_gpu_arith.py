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


def _doubles_all_binades(rng, count):
    """Random doubles over every exponent and both signs, plus edge values."""
    bits = rng.integers(0, 1 << 63, count, dtype=np.int64).astype(np.uint64)
    bits |= rng.integers(0, 2, count).astype(np.uint64) << np.uint64(63)
    x = bits.view(np.float64)
    x = x[np.isfinite(x)]
    edge = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, np.nextafter(1.0, 2.0), np.nextafter(2.0, 0.0), 5e-324,
                     2.0 ** -1022, np.finfo(float).max, -np.finfo(float).max, 3.9999999999999996, 1.0000000000000002])
    return np.concatenate([edge, x])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_directed_division_matches_cuda(gpu, n):
    """er_md's division by the constant RNS_EVAL_UNIT bound (one multiply and FMA
    remainder sign tests) gives the bits of __ddiv_rd / __ddiv_ru."""
    rng = np.random.default_rng(helpers.SEED + 930 + n)
    # the operands er_md sees: products of two significands in [1, 2) (and [0.5, 1)), rounded
    a, b = rng.uniform(1, 2, 400000), rng.uniform(0.5, 2, 400000)
    p = np.concatenate([a * b, np.nextafter(a * b, 0), np.nextafter(a * b, 4), _doubles_all_binades(rng, 400000)])
    out = gpu.probe_check(0, n, p)
    v = out.view(np.int64)
    assert (v[:, 0] == v[:, 1]).all(), p[v[:, 0] != v[:, 1]][:5]
    assert (v[:, 2] == v[:, 3]).all(), p[v[:, 2] != v[:, 3]][:5]


def test_exponent_scaling_matches_scalbn(gpu):
    rng = np.random.default_rng(helpers.SEED + 940)
    x = _doubles_all_binades(rng, 300000)
    k = rng.integers(-2200, 2200, len(x)).astype(np.int32)
    k[: len(x) // 2] = rng.integers(-600, 0, len(x) // 2)  # the er_add range: shifts down
    out = gpu.probe_check(1, 8, x, k).view(np.int64)
    assert (out[:, 0] == out[:, 1]).all()


def test_fixed_point_ceil_log2_matches_cuda(gpu):
    """ceil(log2(x)) from the bits of a fixed-point fraction (with CUDA's log2 at and
    near powers of two) equals ceil(log2(x)) computed with CUDA's log2."""
    rng = np.random.default_rng(helpers.SEED + 950)
    vals = []
    for k in range(0, 83):  # x = F * 2^-83 with F near 2^k
        step = 1 << max(0, k - 52)
        for j in range(-3000, 3001, 1 if k < 20 else 7):
            F = (1 << k) + j * step
            if 0 < F < (1 << 83):
                vals.append(F)
    for _ in range(200000):  # random fractions with at most 53 significant bits
        L = int(rng.integers(1, 84))
        F = int(rng.integers(1 << (L - 1), 1 << L)) if L < 63 else int(rng.integers(1 << 52, 1 << 53)) << (L - 53)
        vals.append(F)
    x = np.array([np.ldexp(float(F), -83) for F in vals])
    assert all(float(xx) * 2.0 ** 83 == float(F) for xx, F in zip(x[:1000], vals[:1000]))
    out = gpu.probe_check(2, 8, x)
    bad = np.nonzero(out[:, 0] != out[:, 1])[0]
    assert len(bad) == 0, [(float.hex(float(x[i])), out[i].tolist()) for i in bad[:5]]


def test_ceil_log2_of_doubles_matches_cuda(gpu):
    """ceil(log2(x)) from the bits of any positive double (normal and subnormal,
    at, just above and just below every power of two) equals CUDA's."""
    rng = np.random.default_rng(helpers.SEED + 951)
    powers = np.ldexp(1.0, np.arange(-1074, 1024))
    near = [powers]
    x = powers
    for k in range(1, 40):
        near.append(np.nextafter(x, np.inf))
        x = near[-1]
    x = powers
    for k in range(1, 40):
        x = np.nextafter(x, 0)
        near.append(x)
    wild = np.abs(_doubles_all_binades(rng, 400000))
    allx = np.concatenate(near + [wild, np.ldexp(1.0 + np.arange(1, 5000) * 2.0 ** -52, -60),
                                  np.ldexp(2.0 - np.arange(1, 5000) * 2.0 ** -52, -61)])
    allx = allx[(allx > 0) & np.isfinite(allx)]
    out = gpu.probe_check(3, 8, allx)
    bad = np.nonzero(out[:, 0] != out[:, 1])[0]
    assert len(bad) == 0, [(float.hex(float(allx[i])), out[i].tolist()) for i in bad[:5]]


@pytest.mark.parametrize("n,kind", [(8, 0), (8, 1), (8, 2), (16, 0), (32, 2), (8, 16), (8, 18), (16, 17)])
def test_chain_probe_computes_the_chains(gpu, oracle, n, kind):
    """The latency probe runs the real reduction step, with the FP64 or (kind +
    16) the fixed-point interval evaluation: each lane's chain sum equals the
    oracle's sequential chain, and it reports at least one cycle per step and
    round counts no larger than the warp."""
    fixed, kind = kind >= 16, kind % 16
    rng = np.random.default_rng(helpers.SEED + 950 + n + kind)
    length = 40
    x = gpu.set_d(n, helpers.doubles(rng, 32 * length, -16, 16))
    y = (helpers.doubles(rng, 32 * length, -8, 8) if kind == 2
         else gpu.set_d(n, helpers.doubles(rng, 32 * length, -16, 16)) if kind == 0 else None)
    cycles, prod_rounds, sum_rounds, res = gpu.probe_chain(n, kind + 16 * fixed, x, y, length)
    acc = np.zeros(32, x.dtype)
    acc["eval"]["frac"] = 0.0
    for t in range(length):
        idx = np.arange(32) * length + t
        a = x[idx].copy()
        if kind == 0:
            p = oracle.mul(n, a, y[idx].copy())
        elif kind == 2:
            p = oracle.mul_d(n, a, np.ascontiguousarray(y[idx]))
        else:
            p = a
        acc = oracle.add(n, acc, p)
    eq(res, acc)
    assert (cycles > 0).all()
    assert (prod_rounds <= 32).all() and (sum_rounds <= 32).all()


@pytest.mark.parametrize("n", [8, 16, 32])
def test_integer_leaves_match_directed_products(gpu, n):
    """The fraction-sum leaves formed on the integer pipes (the exact 84-bit
    product s * R rounded to 53 bits) are the doubles __dmul_ru / __dmul_rd give
    for every residue tried: random ones and the edges 0, 1, 2^k, m_i - 1."""
    rng = np.random.default_rng(helpers.SEED + 970 + n)
    mods = np.array(helpers.moduli(n), dtype=np.int64)
    rows = [rng.integers(0, mods) for _ in range(20000)]
    rows += [np.zeros(n, np.int64), np.ones(n, np.int64), mods - 1, mods // 2]
    rows += [np.minimum(np.full(n, 1 << k, np.int64), mods - 1) for k in range(31)]
    digits = np.array(rows, dtype=np.int64).astype(np.int32)
    r = gpu.probe_int_leaves(n, digits)
    assert (r[:, 0] == r[:, 1]).all(), "upward leaves differ at %s" % np.flatnonzero(r[:, 0] != r[:, 1])[:5]
    assert (r[:, 2] == r[:, 3]).all(), "downward leaves differ at %s" % np.flatnonzero(r[:, 2] != r[:, 3])[:5]
