"""Parity of the CUDA library with the reference: every result bit-identical (digits,
sign, exponent and interval evaluation) to the golden vectors made by the
reference itself and to the oracle, from small edge cases up to the benchmark
sizes.  All calls go through the C ABI."""
import ctypes

import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu
GOLD = helpers.ROOT / "tests" / "golden"


def sync():
    import torch
    torch.cuda.synchronize()


def eq(a, b):
    mm = ffi.mismatches(a, b)
    assert len(mm) == 0, "%d of %d records differ, first at %d" % (len(mm), len(a), mm[0])


def run_dot(lib, n, mx, my, count, order, incx=1, incy=1, r0=None):
    x, y = lib.DeviceArray.from_host(n, mx), lib.DeviceArray.from_host(n, my)
    r = lib.DeviceArray(n, 1)
    if r0 is not None:
        r.upload(r0)
    lib.dot(n, count, x, y, r, incx=incx, incy=incy, order=order)
    sync()
    return r.download()


# ------------------------------------------------------------------ DOT ----

@pytest.mark.parametrize("name,n", [("dot_8.npz", 8), ("dot_16.npz", 16), ("dot_32.npz", 32)])
def test_dot_golden(gpu, name, n):
    g = np.load(GOLD / name)
    for tag in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        count, incx, incy, g1, b1, g2, g3, b3 = [int(v) for v in g[tag + "_meta"]]
        r = run_dot(gpu, n, g[tag + "_mx"], g[tag + "_my"], count, (g1, b1, g2, g3, b3), incx, incy)
        eq(r, g[tag + "_r"])


@pytest.mark.parametrize("n,count,order", [
    (8, 1 << 16, (512, 128, 8192, 256, 64)),
    (8, 100003, (1, 1, 1, 64, 64)),
    (8, 50000, (1, 1, 1, 37, 200)),
    (8, 4000, (1, 1, 1, 2, 1024)),
    (8, 20011, (1, 1, 1, 45, 37)),
    (8, 5000, (1, 1, 1, 7, 3)),
    (8, 3001, (1, 1, 1, 1, 1)),
    (16, 30000, (512, 128, 8192, 256, 64)),
    (32, 20000, (512, 128, 8192, 96, 32)),
])
def test_dot_random_vs_oracle(gpu, oracle, n, count, order):
    rng = np.random.default_rng(helpers.SEED + count + n)
    mx = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    my = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    r = run_dot(gpu, n, mx, my, count, order)
    eq(r, oracle.dot(n, mx, my, g3=order[3], b3=order[4]))


@pytest.mark.parametrize("n", [8, 16])
def test_dot_wide_exponents_vs_oracle(gpu, oracle, n):
    """Entries u * 2^e with e in [-300, 300]: alignments by hundreds of bits,
    zeroed negligible operands and roundings by more than one scaling step."""
    rng = np.random.default_rng(helpers.SEED + 21 + n)
    count = 30011
    mx = gpu.set_d(n, helpers.doubles(rng, count, -300, 300))
    my = gpu.set_d(n, helpers.doubles(rng, count, -300, 300))
    r = run_dot(gpu, n, mx, my, count, (512, 128, 8192, 64, 64))
    eq(r, oracle.dot(n, mx, my, g3=64, b3=64))


def test_dot_strides_and_reuse(gpu, oracle):
    rng = np.random.default_rng(helpers.SEED + 11)
    count = 3000
    mx = gpu.set_d(8, helpers.doubles(rng, 1 + (count - 1) * 3, -16, 16))
    my = gpu.set_d(8, helpers.doubles(rng, 1 + (count - 1) * 2, -16, 16))
    for incx, incy in [(3, 2), (-3, 2), (3, -2), (-3, -2)]:
        r = run_dot(gpu, 8, mx, my, count, (1, 1, 1, 48, 64), incx, incy)
        eq(r, oracle.dot(8, mx, my, g3=48, b3=64, incx=incx, incy=incy, length=count))


def test_dot_zero_length_leaves_result(gpu):
    rec = gpu.set_d(8, np.array([1.5]))
    r = run_dot(gpu, 8, rec, rec, 0, (512, 128, 8192, 256, 64), r0=rec)
    eq(r, rec)


def test_dot_full_size(gpu, oracle):
    """n = 2^20, x and y = u*2^e with e in -16..16: the size and distribution of the
    DOT benchmark, bit-identical to the oracle at the reference's launch parameters."""
    rng = np.random.default_rng(helpers.SEED + 0)
    count = 1 << 20
    mx = gpu.set_d(8, helpers.doubles(rng, count, -16, 16))
    my = gpu.set_d(8, helpers.doubles(rng, count, -16, 16))
    r = run_dot(gpu, 8, mx, my, count, (512, 128, 8192, 256, 64))
    eq(r, oracle.dot(8, mx, my, g3=256, b3=64))


# ----------------------------------------------------------------- GEMV ----

def run_gemv(lib, n, trans, m, cols, alpha, A, lda, x, beta, y, incx, incy, b3):
    dA, dx, dy = (lib.DeviceArray.from_host(n, v) for v in (A, x, y))
    da, db = lib.DeviceArray.from_host(n, alpha), lib.DeviceArray.from_host(n, beta)
    lib.gemv(n, trans, m, cols, da, dA, lda, dx, db, dy, incx=incx, incy=incy, order=(256, 128, 256, b3))
    sync()
    return dy.download()


@pytest.mark.parametrize("name,n", [("gemv_16.npz", 16), ("gemv_8.npz", 8)])
def test_gemv_golden(gpu, name, n):
    g = np.load(GOLD / name)
    for tag in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        trans, m, cols, lda, incx, incy, b3 = [int(v) for v in g[tag + "_meta"]]
        r = run_gemv(gpu, n, trans, m, cols, g[tag + "_alpha"], g[tag + "_A"], lda, g[tag + "_x"],
                     g[tag + "_beta"], g[tag + "_y"], incx, incy, b3)
        eq(r, g[tag + "_r"])


@pytest.mark.parametrize("n,trans,m,cols,b3", [
    (16, 111, 300, 200, 32), (16, 112, 260, 190, 32), (16, 111, 33, 1000, 256), (8, 112, 500, 45, 7),
    (32, 111, 64, 130, 32), (16, 111, 1, 1, 32), (16, 112, 100, 3, 600),
])
def test_gemv_random_vs_oracle(gpu, oracle, n, trans, m, cols, b3):
    rng = np.random.default_rng(helpers.SEED + 3 + m + cols)
    lda = m + 2
    lx, ly = (cols, m) if trans == 111 else (m, cols)
    A = gpu.set_d(n, helpers.doubles(rng, lda * cols, -32, 32))
    x = gpu.set_d(n, helpers.doubles(rng, lx, -32, 32))
    y = gpu.set_d(n, helpers.doubles(rng, ly, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    r = run_gemv(gpu, n, trans, m, cols, al, A, lda, x, be, y, 1, 1, b3)
    eq(r, oracle.gemv(n, trans, m, cols, al, A, lda, x, be, y, b3=b3))


# ----------------------------------------------------------------- GEMM ----

def run_gemm(lib, n, m, cols, k, alpha, A, lda, B, ldb, beta, C, ldc):
    dA, dB, dC = (lib.DeviceArray.from_host(n, v) for v in (A, B, C))
    da, db = lib.DeviceArray.from_host(n, alpha), lib.DeviceArray.from_host(n, beta)
    lib.gemm(n, m, cols, k, da, dA, lda, dB, ldb, db, dC, ldc)
    sync()
    return dC.download()


@pytest.mark.parametrize("name,n", [("gemm_32.npz", 32), ("gemm_8.npz", 8)])
def test_gemm_golden(gpu, name, n):
    g = np.load(GOLD / name)
    for tag in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        m, cols, k, lda, ldb, ldc = [int(v) for v in g[tag + "_meta"]]
        r = run_gemm(gpu, n, m, cols, k, g[tag + "_alpha"], g[tag + "_A"], lda, g[tag + "_B"], ldb,
                     g[tag + "_beta"], g[tag + "_C"], ldc)
        eq(r, g[tag + "_r"])


@pytest.mark.parametrize("n,m,cols,k", [(32, 40, 30, 60), (8, 70, 33, 129), (16, 37, 41, 17)])
def test_gemm_random_vs_oracle(gpu, oracle, n, m, cols, k):
    rng = np.random.default_rng(helpers.SEED + 1 + m * cols)
    lda, ldb, ldc = m, k, m
    A = gpu.set_d(n, helpers.doubles(rng, lda * k, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, ldb * cols, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, ldc * cols, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    r = run_gemm(gpu, n, m, cols, k, al, A, lda, B, ldb, be, C, ldc)
    eq(r, oracle.gemm(n, m, cols, k, al, A, lda, B, ldb, be, C, ldc))


@pytest.mark.parametrize("n", [8, 16, 32])
def test_gemm_wide_exponents_vs_oracle(gpu, oracle, n):
    """Entries u * 2^e with e in [-400, 400]: the aligned additions of the k
    chain shift by more than the 256 rows of powers of two that the GEMM kernel
    stages in shared memory, so both the staged and the global table are read."""
    m, cols, k = 24, 16, 40
    rng = np.random.default_rng(helpers.SEED + 7 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -400, 400))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -400, 400))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, -400, 400))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    r = run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m)
    eq(r, oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m))


def _gemm_case(gpu, oracle, n, A, B, m, cols, k, rng):
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    r = run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m)
    eq(r, oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m))


@pytest.mark.parametrize("n", [8, 16, 32])
def test_gemm_exact_cancellation_vs_oracle(gpu, oracle, n):
    """Column pairs of A repeated and row pairs of B negated: every second step
    of each k chain cancels the sum to exactly zero, so the bounds leave the
    sign open and mp_add decides it from the residues (sign_estimate); some
    entries are zero."""
    m, cols, k = 33, 9, 48
    rng = np.random.default_rng(helpers.SEED + 11 + n)
    a = helpers.doubles(rng, m * k, -40, 40).reshape(k, m)
    b = helpers.doubles(rng, k * cols, -40, 40).reshape(cols, k)
    a[1::2, :] = a[0::2, :]
    b[:, 1::2] = -b[:, 0::2]
    a[5, :7] = 0.0
    b[2, 3:] = 0.0
    _gemm_case(gpu, oracle, n, gpu.set_d(n, a.ravel()), gpu.set_d(n, b.ravel()), m, cols, k, rng)


@pytest.mark.parametrize("n", [8, 16, 32])
def test_gemm_big_integer_operands_vs_oracle(gpu, oracle, n):
    """Operands with wide residue integers (cubes of converted doubles, made by
    the oracle's mp_mul): products and sums round inside the k chain."""
    m, cols, k = 20, 12, 30
    rng = np.random.default_rng(helpers.SEED + 13 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -20, 20))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -20, 20))
    A = oracle.mul(n, A, oracle.mul(n, A, A))
    B = oracle.mul(n, B, oracle.mul(n, B, B))
    _gemm_case(gpu, oracle, n, A, B, m, cols, k, rng)


@pytest.mark.parametrize("n", [8, 32])
def test_gemm_huge_exponents_vs_oracle(gpu, oracle, n):
    """Exponents of A raised and those of B lowered by 2^28 + 5 (the products
    keep ordinary exponents): the integer exponent arithmetic of these steps is
    near its range, so the chain runs them step by step."""
    m, cols, k = 16, 8, 24
    rng = np.random.default_rng(helpers.SEED + 17 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -30, 30))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -30, 30))
    A["exp"][::3] += (1 << 28) + 5
    B["exp"][::3] -= (1 << 28) + 5
    _gemm_case(gpu, oracle, n, A, B, m, cols, k, rng)


@pytest.mark.parametrize("n,lo,hi", [(8, -32, 32), (32, -32, 32), (16, -400, 400)])
def test_gemm_without_scratch_vs_oracle(gpu, oracle, monkeypatch, n, lo, hi):
    """MPRES_GEMM_NO_SCRATCH=1 selects the step-by-step k chain, the path mp_gemm
    takes when its workspace cannot grow: the same bits as the lazy-residue chain."""
    m, cols, k = 36, 20, 50
    rng = np.random.default_rng(helpers.SEED + 19 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, lo, hi))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, lo, hi))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, lo, hi))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    want = oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m)
    eq(run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m), want)
    monkeypatch.setenv("MPRES_GEMM_NO_SCRATCH", "1")
    eq(run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m), want)


def test_gemm_long_k_vs_oracle(gpu, oracle):
    """k = 4200 with 32 moduli: the tensor-core modular product folds its 64-bit
    accumulators every 128 stages of 32 k steps, so this chain crosses a fold
    (and ends in a partial stage)."""
    n, m, cols, k = 32, 9, 7, 4200
    rng = np.random.default_rng(helpers.SEED + 29)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    eq(run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m), oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m))


def test_gemm_phase_probe_matches_gemm(gpu, oracle):
    """mpres_probe_gemm_phases runs mp_gemm's split form (32 moduli) with an
    event between its launches: the oracle's bits, and a time for each launch."""
    n, m, cols, k = 32, 70, 45, 90
    rng = np.random.default_rng(helpers.SEED + 23)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    dA, dB, dC = (gpu.DeviceArray.from_host(n, v) for v in (A, B, C))
    da, db = gpu.DeviceArray.from_host(n, al), gpu.DeviceArray.from_host(n, be)
    ms = gpu.probe_gemm_phases(n, m, cols, k, da, dA, m, dB, k, db, dC, m)
    sync()
    eq(dC.download(), oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m))
    assert list(ms) == list(gpu.GEMM_PHASES) and all(v > 0 for v in ms.values())
    with pytest.raises(gpu.MpresError):
        gpu.probe_gemm_phases(8, 2, 2, 2, da, dA, 2, dB, 2, db, dC, 2)


@pytest.mark.parametrize("lo,hi", [(-32, 32), (-400, 400)])
def test_gemm_tiled_form_vs_oracle(gpu, oracle, monkeypatch, lo, hi):
    """MPRES_GEMM_NO_SPLIT=1 selects, for 32 moduli, the tiled lazy-residue chain
    that mp_gemm takes when its workspace can hold W(A), W(B) but not the split
    form's scratch: the same bits as the split form and the oracle."""
    n, m, cols, k = 32, 45, 19, 70
    rng = np.random.default_rng(helpers.SEED + 31 + hi)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, lo, hi))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, lo, hi))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, lo, hi))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    want = oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C, m)
    eq(run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m), want)
    monkeypatch.setenv("MPRES_GEMM_NO_SPLIT", "1")
    eq(run_gemm(gpu, n, m, cols, k, al, A, m, B, k, be, C, m), want)


def test_gemm_transposed_is_not_supported(gpu):
    rec = gpu.set_d(8, np.ones(4))
    d = gpu.DeviceArray.from_host(8, rec)
    a = gpu.DeviceArray.from_host(8, rec[:1])
    with pytest.raises(gpu.MpresError):
        gpu.gemm(8, 2, 2, 2, a, d, 2, d, 2, a, d, 2, transa=gpu.TRANS)


def test_gemm_full_size(gpu, oracle):
    """m = n = k = 1024 with 32 moduli, the GEMM benchmark's inputs: all
    1 048 576 outputs bit-for-bit against the oracle (each a 1024-long k chain)."""
    n, m = 32, 1024
    rng = np.random.default_rng(helpers.SEED + 1)
    A = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    r = run_gemm(gpu, n, m, m, m, al, A, m, B, m, be, C, m)
    eq(r, oracle.gemm(n, m, m, m, al, A, m, B, m, be, C, m))


# ----------------------------------------------------------------- SpMV ----

def run_spmv(lib, n, kind, m, mx, irp=None, ja=None, vals=None, tpr=None, maxnzr=None, ell_ja=None, ell_as=None):
    x = lib.DeviceBytes.from_numpy(mx)
    y = lib.DeviceBytes(m * mx.dtype.itemsize)
    if kind == "ell":
        e = lib.DeviceEll(m, maxnzr, ell_ja, ell_as)
        lib.spmv_ell(n, m, e, x, y)
    else:
        c = lib.DeviceCsr(m, irp, ja, vals)
        if kind == "csr":
            lib.spmv_csr(n, m, c, x, y)
        else:
            lib.spmv_csrv(n, m, c, x, y, tpr)
    sync()
    return y.to_numpy(mx.dtype, m)


def test_spmv_golden(gpu):
    g = np.load(GOLD / "spmv_8.npz")
    m = len(g["irp"]) - 1
    eq(run_spmv(gpu, 8, "csr", m, g["mx"], g["irp"], g["ja"], g["vals"]), g["csr"])
    for tpr in (1, 2, 4, 8, 16, 32):
        eq(run_spmv(gpu, 8, "csrv", m, g["mx"], g["irp"], g["ja"], g["vals"], tpr=tpr), g["csrv%d" % tpr])
    eq(run_spmv(gpu, 8, "ell", m, g["mx"], maxnzr=int(g["maxnzr"][0]), ell_ja=g["ell_ja"], ell_as=g["ell_as"]),
       g["ell"])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_spmv_random_vs_oracle(gpu, oracle, n):
    rng = np.random.default_rng(helpers.SEED + 2 + n)
    m = 20000
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    mx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    eq(run_spmv(gpu, n, "csr", m, mx, irp, ja, vals), oracle.spmv_csr(n, m, irp, ja, vals, mx))
    for tpr in (4, 16, 32):
        eq(run_spmv(gpu, n, "csrv", m, mx, irp, ja, vals, tpr=tpr), oracle.spmv_csrv(n, m, tpr, irp, ja, vals, mx))
    small = 3000
    sirp, sja, svals = helpers.random_csr(rng, small, m, helpers.power_law_rows(rng, small, kmax=200))
    maxnzr, eja, eas = helpers.csr_to_ell(small, sirp, sja, svals)
    eq(run_spmv(gpu, n, "ell", small, mx, maxnzr=maxnzr, ell_ja=eja, ell_as=eas),
       oracle.spmv_ell(n, small, maxnzr, eja, eas, mx))


def test_spmv_short_rows_and_stored_zeros_vs_oracle(gpu, oracle):
    """2^18 rows of 1..8 entries: the longest chain is below a lane's average
    work, so every block of the persistent grid takes rows (the power-law cases
    keep one block per SM).  A fifth of the values are stored zeros, so ELL rows
    hold zeros before later nonzeros: each row's chain must run to its last
    nonzero."""
    n = 8
    rng = np.random.default_rng(helpers.SEED + 31)
    m = 1 << 18
    irp, ja, vals = helpers.random_csr(rng, m, m, rng.integers(1, 9, m))
    vals[rng.random(len(vals)) < 0.2] = 0.0
    mx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    eq(run_spmv(gpu, n, "csr", m, mx, irp, ja, vals), oracle.spmv_csr(n, m, irp, ja, vals, mx))
    eq(run_spmv(gpu, n, "csrv", m, mx, irp, ja, vals, tpr=4), oracle.spmv_csrv(n, m, 4, irp, ja, vals, mx))
    maxnzr, eja, eas = helpers.csr_to_ell(m, irp, ja, vals)
    eq(run_spmv(gpu, n, "ell", m, mx, maxnzr=maxnzr, ell_ja=eja, ell_as=eas),
       oracle.spmv_ell(n, m, maxnzr, eja, eas, mx))


def test_spmv_ell_odd_rows_vs_oracle(gpu, oracle):
    """ELL with an odd row count (the row-end scan then reads one row per thread
    instead of two) and stored zeros."""
    n = 8
    rng = np.random.default_rng(helpers.SEED + 32)
    m = 4999
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m, kmax=64))
    vals[rng.random(len(vals)) < 0.1] = 0.0
    mx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    maxnzr, eja, eas = helpers.csr_to_ell(m, irp, ja, vals)
    # zero slots (padding and stored zeros) carry other, valid columns: never used
    zero = eas == 0.0
    eja[zero] = rng.integers(0, m, int(zero.sum()))
    eq(run_spmv(gpu, n, "ell", m, mx, maxnzr=maxnzr, ell_ja=eja, ell_as=eas),
       oracle.spmv_ell(n, m, maxnzr, eja, eas, mx))


@pytest.fixture(scope="module")
def spmv_bench_matrix(gpu, oracle):
    """The SpMV benchmark's inputs: 2^20 rows, power-law row lengths 1..1024
    (mean 16), 8 moduli; with the oracle's CSR result over every row."""
    rng = np.random.default_rng(helpers.SEED + 2)
    m = 1 << 20
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    mx = gpu.set_d(8, helpers.doubles(rng, m, -16, 16))
    return m, irp, ja, vals, mx, oracle.spmv_csr(8, m, irp, ja, vals, mx)


def test_spmv_full_size_csr(gpu, spmv_bench_matrix):
    m, irp, ja, vals, mx, want = spmv_bench_matrix
    eq(run_spmv(gpu, 8, "csr", m, mx, irp, ja, vals), want)


@pytest.mark.parametrize("tpr", [4, 16, 32])
def test_spmv_full_size_csrv(gpu, oracle, spmv_bench_matrix, tpr):
    """CSR-vector at the tpr values of the reference's SpMV driver
    (tests/sparse/test_spmv.cu:179-181), every row against the oracle."""
    m, irp, ja, vals, mx, _ = spmv_bench_matrix
    eq(run_spmv(gpu, 8, "csrv", m, mx, irp, ja, vals, tpr=tpr), oracle.spmv_csrv(8, m, tpr, irp, ja, vals, mx))


def test_spmv_full_size_ell(gpu, oracle, spmv_bench_matrix):
    """ELLPACK of the benchmark matrix (maxnzr slots per row, about 12.9 GB,
    built on the device): every row equals the CSR chain (ELL keeps a row's entry
    order and skips only stored zeros, and the values are never zero), which
    equals the oracle; a row sample holding every row of the longest bucket and
    rows of every length is also checked against the oracle's own ELL."""
    import torch
    m, irp, ja, vals, mx, want = spmv_bench_matrix
    lens = np.diff(irp).astype(np.int64)
    maxnzr = int(lens.max())
    irp_t = torch.from_numpy(irp.astype(np.int64)).cuda()
    rows = torch.repeat_interleave(torch.arange(m, device="cuda"), torch.from_numpy(lens).cuda())
    slot = (torch.arange(len(ja), device="cuda") - irp_t[:-1][rows]) * m + rows
    del rows
    ell_ja = torch.zeros(maxnzr * m, dtype=torch.int32, device="cuda")
    ell_as = torch.zeros(maxnzr * m, dtype=torch.float64, device="cuda")
    ell_ja[slot] = torch.from_numpy(ja).cuda()
    ell_as[slot] = torch.from_numpy(vals).cuda()
    del slot
    e = gpu.DeviceEll.from_tensors(m, maxnzr, ell_ja, ell_as)
    x = gpu.DeviceBytes.from_numpy(mx)
    y = gpu.DeviceBytes(m * mx.dtype.itemsize)
    gpu.spmv_ell(8, m, e, x, y)
    sync()
    got = y.to_numpy(mx.dtype, m)
    e.free()
    del ell_ja, ell_as
    torch.cuda.empty_cache()
    eq(got, want)
    rng = np.random.default_rng(helpers.SEED + 23)
    sample = set(np.flatnonzero(lens >= maxnzr // 2).tolist())
    for L in np.unique(lens):
        cand = np.flatnonzero(lens == L)
        sample.update(rng.choice(cand, min(3, len(cand)), replace=False).tolist())
    sample = np.array(sorted(sample))
    sirp = np.concatenate([[0], np.cumsum(lens[sample])]).astype(np.int32)
    sja = np.concatenate([ja[irp[r]:irp[r + 1]] for r in sample])
    svals = np.concatenate([vals[irp[r]:irp[r + 1]] for r in sample])
    smax, eja, eas = helpers.csr_to_ell(len(sample), sirp, sja, svals)
    eq(got[sample], oracle.spmv_ell(8, len(sample), smax, eja, eas, mx))


# ---------------------------------------------------------------- errors ----

def test_bad_arguments_are_reported(gpu):
    rec = gpu.set_d(8, np.ones(4))
    d = gpu.DeviceArray.from_host(8, rec)
    with pytest.raises(gpu.MpresError):
        gpu.dot(8, 4, d, d, d, order=(1, 1, 1, 0, 64))
    c = gpu.DeviceCsr(2, np.array([0, 1, 2]), np.array([0, 1]), np.array([1.0, 2.0]))
    x = gpu.DeviceBytes.from_numpy(rec)
    with pytest.raises(gpu.MpresError):
        gpu.spmv_csrv(8, 2, c, x, x, tpr=3)
    assert gpu.lib().mpres_dot(12, 4, d.ref, 1, d.ref, 1, d.ref, None, 1, 1, 1, 1, 1, None) != 0


# ------------------------------------------------------ Matrix Market input ----

def test_spmv_from_matrix_market_file(gpu, oracle, tmp_path):
    """A symmetric file read by the library's reader: CSR, CSR-vector and ELL
    results on the GPU equal the oracle's on the same arrays."""
    import test_mtx
    rng = np.random.default_rng(helpers.SEED + 61)
    ent = test_mtx.random_entries(rng, 5000, 5000, 30000, symmetric=True)
    ent += [(i, i, rng.normal()) for i in range(1, 5001, 2)]
    rng.shuffle(ent)
    path = test_mtx.write_mtx(tmp_path / "sym.mtx", 5000, 5000, ent, symmetric=True)
    st = gpu.mtx_stats(path)
    irp, ja, vals = gpu.mtx_csr(path, st)
    eja, eas = gpu.mtx_ell(path, st)
    m = st["m"]
    mx = gpu.set_d(8, helpers.doubles(rng, m, -16, 16))
    eq(run_spmv(gpu, 8, "csr", m, mx, irp, ja, vals), oracle.spmv_csr(8, m, irp, ja, vals, mx))
    eq(run_spmv(gpu, 8, "csrv", m, mx, irp, ja, vals, tpr=8), oracle.spmv_csrv(8, m, 8, irp, ja, vals, mx))
    eq(run_spmv(gpu, 8, "ell", m, mx, maxnzr=st["maxnzr"], ell_ja=eja, ell_as=eas),
       oracle.spmv_ell(8, m, st["maxnzr"], eja, eas, mx))
