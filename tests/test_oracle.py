"""The CPU oracle against the reference's golden vectors (tests/golden, produced by
the reference built for the CPU) and, where that build exists, against the
reference directly on fresh random inputs; plus accuracy against exact
rational results."""
from fractions import Fraction

import numpy as np
import pytest

import helpers
from oracle import ffi

GOLD = helpers.ROOT / "tests" / "golden"


def load(name):
    return np.load(GOLD / name)


def eq(a, b):
    mm = ffi.mismatches(a, b)
    assert len(mm) == 0, "%d mismatching records, first at %d" % (len(mm), mm[0])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_elementwise_matches_golden(oracle, n):
    g = load("elem_%d.npz" % n)
    eq(oracle.set_d(n, g["x"]), g["mx"])
    eq(oracle.set_d(n, g["y"]), g["my"])
    eq(oracle.mul(n, g["mx"], g["my"]), g["prod"])
    eq(oracle.add(n, g["mx"], g["my"]), g["sum"])
    eq(oracle.mul_d(n, g["mx"], g["d"]), g["q"])
    eq(oracle.add(n, g["mx"], g["q"]), g["canc"])
    acc = g["prod"].copy()
    for _ in range(6):
        acc = oracle.add(n, oracle.mul(n, acc, g["my"]), g["prod"])
    eq(acc, g["acc"])
    eq(oracle.mul_d(n, g["acc"], g["dd"]), g["muld"])


def test_cancellation_golden_covers_ambiguous_sign(oracle):
    """The near-cancellation case must reach the mixed-radix sign test, which sets one
    bound of the result to +-RNS_EVAL_UNIT.low (src/arith/add.cuh:171-176)."""
    g = load("elem_8.npz")
    u = oracle.tables(8, 242)["units"][0]
    ev = g["canc"]["eval"]
    hit = ((np.abs(ev[:, 0]["frac"]) == u["frac"]) & (ev[:, 0]["exp"] == u["exp"])) | \
          ((np.abs(ev[:, 1]["frac"]) == u["frac"]) & (ev[:, 1]["exp"] == u["exp"]))
    assert hit.sum() > 20


@pytest.mark.parametrize("name,n", [("dot_8.npz", 8), ("dot_16.npz", 16), ("dot_32.npz", 32)])
def test_dot_matches_golden(oracle, name, n):
    g = load(name)
    tags = sorted({k.rsplit("_", 1)[0] for k in g.files})
    for tag in tags:
        count, incx, incy, g1, b1, g2, g3, b3 = [int(v) for v in g[tag + "_meta"]]
        eq(oracle.set_d(n, g[tag + "_x"]), g[tag + "_mx"])
        r = oracle.dot(n, g[tag + "_mx"], g[tag + "_my"], g3=g3, b3=b3, incx=incx, incy=incy, length=count)
        eq(r, g[tag + "_r"])


@pytest.mark.parametrize("name,n", [("gemv_16.npz", 16), ("gemv_8.npz", 8)])
def test_gemv_matches_golden(oracle, name, n):
    g = load(name)
    for tag in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        trans, m, cols, lda, incx, incy, b3 = [int(v) for v in g[tag + "_meta"]]
        r = oracle.gemv(n, trans, m, cols, g[tag + "_alpha"], g[tag + "_A"], lda, g[tag + "_x"], g[tag + "_beta"],
                        g[tag + "_y"], incx=incx, incy=incy, b3=b3)
        eq(r, g[tag + "_r"])


@pytest.mark.parametrize("name,n", [("gemm_32.npz", 32), ("gemm_8.npz", 8)])
def test_gemm_matches_golden(oracle, name, n):
    g = load(name)
    for tag in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        m, cols, k, lda, ldb, ldc = [int(v) for v in g[tag + "_meta"]]
        r = oracle.gemm(n, m, cols, k, g[tag + "_alpha"], g[tag + "_A"], lda, g[tag + "_B"], ldb,
                        g[tag + "_beta"], g[tag + "_C"], ldc)
        eq(r, g[tag + "_r"])


def test_spmv_matches_golden(oracle):
    g = load("spmv_8.npz")
    m = len(g["irp"]) - 1
    eq(oracle.spmv_csr(8, m, g["irp"], g["ja"], g["vals"], g["mx"]), g["csr"])
    for tpr in (1, 2, 4, 8, 16, 32):
        eq(oracle.spmv_csrv(8, m, tpr, g["irp"], g["ja"], g["vals"], g["mx"]), g["csrv%d" % tpr])
    eq(oracle.spmv_ell(8, m, int(g["maxnzr"][0]), g["ell_ja"], g["ell_as"], g["mx"]), g["ell"])


needs_ref = pytest.mark.skipif(not ffi.ref_available(8), reason="reference not built here (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("n", [8, 16, 32])
def test_constant_tables_match_reference(oracle, n):
    a, b = oracle.tables(n, helpers.LOG2M[n]), ffi.reference(n).tables(helpers.LOG2M[n])
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k


@needs_ref
@pytest.mark.parametrize("n", [8, 16, 32])
def test_random_arithmetic_matches_reference(oracle, n):
    R = ffi.reference(n)
    rng = np.random.default_rng(helpers.SEED + 500 + n)
    pool = R.set_d(helpers.doubles(rng, 3000, -40, 40))
    for gen in range(8):
        i, j = rng.integers(0, len(pool), 3000), rng.integers(0, len(pool), 3000)
        a, b = pool[i].copy(), pool[j].copy()
        if gen % 3 == 0:
            ro, rr = oracle.mul(n, a, b), R.mul(a, b)
        elif gen % 3 == 1:
            ro, rr = oracle.add(n, a, b), R.add(a, b)
        else:
            d = rng.standard_normal(3000)
            ro, rr = oracle.mul_d(n, a, d), R.mul_d(a, d)
        eq(ro, rr)
        pool = np.concatenate([pool, rr])[-9000:]
    digits = rng.integers(0, 1 << 30, (4000, n)).astype(np.int32)
    D = rng.integers(0, helpers.LOG2M[n], 4000).astype(np.uint32)
    assert oracle.scale2pow(n, digits, D).tobytes() == R.scale2pow(digits, D).tobytes()
    for f in ("eval", "eval_fast"):
        lo1, up1 = getattr(oracle, f)(n, digits)
        lo2, up2 = getattr(R, f)(digits)
        assert lo1.tobytes() == lo2.tobytes() and up1.tobytes() == up2.tobytes(), f


@needs_ref
def test_random_blas_matches_reference(oracle):
    R = ffi.reference(8)
    rng = np.random.default_rng(helpers.SEED + 600)
    x, y = R.set_d(helpers.doubles(rng, 5000, -16, 16)), R.set_d(helpers.doubles(rng, 5000, -16, 16))
    for g3, b3 in [(256, 64), (13, 17), (3, 1024), (1, 1)]:
        eq(oracle.dot(8, x, y, g3=g3, b3=b3), R.dot(x, y, g3=g3, b3=b3))
    irp, ja, vals = helpers.random_csr(rng, 400, 300, helpers.power_law_rows(rng, 400, kmax=128))
    xv = R.set_d(helpers.doubles(rng, 300, -16, 16))
    eq(oracle.spmv_csr(8, 400, irp, ja, vals, xv), R.spmv_csr(400, irp, ja, vals, xv))
    eq(oracle.spmv_csrv(8, 400, 8, irp, ja, vals, xv), R.spmv_csrv(400, 8, irp, ja, vals, xv))


@needs_ref
@pytest.mark.parametrize("n", [8, 16, 32])
def test_gemm_edge_inputs_match_reference(oracle, n):
    """Two GEMM input classes the GPU parity tests use for the out-of-line steps
    of the lazy-residue chain: exact cancellations (the sum's sign comes from the
    residues) and cubed operands (products and sums round), with zeros.  The
    oracle must equal the reference here too.  Wide or huge exponent ranges are
    compared with the oracle only: at the first step of a chain the running sum
    is zero, and the reference aligns it by indexing RNS_POW2 with the full
    exponent gap, past the end of the table (the CPU build faults there); the
    oracle and the CUDA kernels clamp that row, which gives the same product
    because the zero's digits are all zero."""
    if not ffi.ref_available(n):
        pytest.skip("reference for %d moduli not built here" % n)
    R = ffi.reference(n)
    rng = np.random.default_rng(helpers.SEED + 700 + n)
    m, cols, k = 12, 7, 26
    al, be = R.set_d(rng.uniform(-1, 1, 1)), R.set_d(rng.uniform(-1, 1, 1))
    for case in ("cancel", "cube"):
        a = helpers.doubles(rng, m * k, -30, 30).reshape(k, m)
        b = helpers.doubles(rng, k * cols, -30, 30).reshape(cols, k)
        if case == "cancel":
            a[1::2, :] = a[0::2, :]
            b[:, 1::2] = -b[:, 0::2]
        a[3, :4] = 0.0
        A, B = R.set_d(a.ravel()), R.set_d(b.ravel())
        if case == "cube":
            A = R.mul(A, R.mul(A, A))
            B = R.mul(B, R.mul(B, B))
        C = R.set_d(helpers.doubles(rng, m * cols, -30, 30))
        eq(oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m), R.gemm(m, cols, k, al, A, m, B, k, be, C, m))


def test_dot_accuracy_within_reference_bound(oracle):
    """|r - exact| <= u*n/(1-u*n) * sum|x_i y_i|, u = 4/sqrt(M): the bound of the
    reference's accuracy test (tests/blas/accuracy/test_dot_accuracy.cu:39-90)."""
    g = load("dot_8.npz")
    mods = helpers.moduli(8)
    for tag in ("perf", "odd", "acc"):
        count = int(g[tag + "_meta"][0])
        x, y = g[tag + "_x"][:count], g[tag + "_y"][:count]
        err = abs(helpers.mp_value(g[tag + "_r"][0], mods) - helpers.exact_dot(x, y))
        assert err <= helpers.dot_bound(8, count, x, y)


def test_gemm_accuracy_within_bound(oracle):
    g = load("gemm_32.npz")
    mods = helpers.moduli(32)
    m, cols, k, lda, ldb, ldc = [int(v) for v in g["a_meta"]]
    val = lambda rec: helpers.mp_value(rec, mods)  # noqa: E731
    al, be = val(g["a_alpha"][0]), val(g["a_beta"][0])
    for r in range(0, m, 5):
        for c in range(0, cols, 4):
            exact = sum((val(g["a_A"][r + i * lda]) * val(g["a_B"][i + c * ldb]) for i in range(k)), Fraction(0))
            exact = al * exact + be * val(g["a_C"][r + c * ldc])
            got = val(g["a_r"][r + c * ldc])
            scale = abs(al) * sum(abs(val(g["a_A"][r + i * lda]) * val(g["a_B"][i + c * ldb])) for i in range(k)) \
                + abs(be * val(g["a_C"][r + c * ldc]))
            u = Fraction(4, int(2 ** (helpers.LOG2M[32] / 2)))
            assert abs(got - exact) <= u * (k + 3) * scale * 2


def test_add_abs_and_v2_reductions_match_reference_golden(oracle):
    for n in (8, 16):
        g = np.load(GOLD / ("v2_%d.npz" % n))
        eq(oracle.add_abs(n, g["x"], g["y"]), g["add_abs"])
        for blocks, threads in ((256, 32), (7, 33)):
            eq(oracle.reduce_v2(n, True, g["x"], None, blocks, threads), g["sumsq_%d_%d" % (blocks, threads)])
            eq(oracle.reduce_v2(n, False, g["x"], g["y"], blocks, threads), g["dot_%d_%d" % (blocks, threads)])
