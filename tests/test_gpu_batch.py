"""Batches (one persistent launch for many operations) against the plain entry
points: every GEMV, GEMM, DOT and SpMV (CSR, CSR-vector, ELL) output of a batch
must equal, record for record, what mpres_gemv / mpres_gemm / mpres_dot / mpres_spmv_* give
for the same arguments -- with and without graph replay and autotuning, for
uneven sizes, strides, transposition, odd blockDim3 and skipped operations."""
import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu


def eq(got, want, what):
    mm = ffi.mismatches(got, want)
    assert len(mm) == 0, "%s: %d of %d records differ, first at %d" % (what, len(mm), len(want), mm[0])


def _vec(gpu, n, rng, count, lo=-32, hi=32):
    return gpu.set_d(n, helpers.doubles(rng, max(count, 1), lo, hi))


GEMVS = [  # trans, m, n, incx, incy, b3
    (False, 1, 1, 1, 1, 32), (False, 33, 70, 1, 1, 32), (True, 130, 17, 1, 1, 32), (False, 64, 300, -2, 3, 64),
    (True, 257, 129, 2, -1, 7), (False, 200, 40, 1, 1, 1), (True, 50, 600, 1, 1, 128), (False, 0, 10, 1, 1, 32),
    (False, 10, 10, 0, 1, 32),
]
DOTS = [(1, 1, 1, 256, 64), (1000, 1, 1, 256, 64), (5000, -1, 2, 7, 33), (3000, 1, 1, 64, 128), (0, 1, 1, 256, 64)]


GEMMS = [(1, 1, 1), (33, 7, 50), (100, 64, 129), (64, 65, 3), (130, 40, 257)]  # m, n, k


def _build(gpu, n, rng, small, gemm=False):
    scale = 4 if small else 1
    ops = []
    for trans, m, k, incx, incy, b3 in GEMVS:
        m, k = max(m // scale, min(m, 1)), max(k // scale, min(k, 1))
        lda = max(m, 1) + int(rng.integers(0, 3))
        lx, ly = (m, k) if trans else (k, m)
        ops.append(dict(kind="gemv", trans=gpu.TRANS if trans else gpu.NO_TRANS, m=m, n=k, lda=lda, incx=incx,
                        incy=incy, b3=b3, A=_vec(gpu, n, rng, lda * max(k, 1)),
                        x=_vec(gpu, n, rng, 1 + max(lx - 1, 0) * max(abs(incx), 1)),
                        y=_vec(gpu, n, rng, 1 + max(ly - 1, 0) * abs(incy)),
                        alpha=_vec(gpu, n, rng, 1, -1, 1), beta=_vec(gpu, n, rng, 1, -1, 1)))
    for cnt, incx, incy, g3, b3 in DOTS:
        cnt //= scale
        ops.append(dict(kind="dot", n=cnt, incx=incx, incy=incy, g3=g3, b3=b3,
                        x=_vec(gpu, n, rng, 1 + max(cnt - 1, 0) * abs(incx), -16, 16),
                        y=_vec(gpu, n, rng, 1 + max(cnt - 1, 0) * abs(incy), -16, 16), r=_vec(gpu, n, rng, 1)))
    m = 3000 // scale
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    ops.append(dict(kind="spmv", m=m, csr=gpu.DeviceCsr(m, irp, ja, vals), x=_vec(gpu, n, rng, m, -16, 16)))
    for tpr in (2, 16):
        m = (2000 + 37 * tpr) // scale
        irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m, kmax=300))
        ops.append(dict(kind="csrv", tpr=tpr, m=m, csr=gpu.DeviceCsr(m, irp, ja, vals),
                        x=_vec(gpu, n, rng, m, -16, 16)))
    m = 1500 // scale
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m, kmax=150))
    maxnzr, eja, eas = helpers.csr_to_ell(m, irp, ja, vals)
    ops.append(dict(kind="ell", m=m, ell=gpu.DeviceEll(m, maxnzr, eja, eas), x=_vec(gpu, n, rng, m, -16, 16)))
    if gemm:
        for m, cols, k in GEMMS:
            m, cols, k = max(m // scale, 1), max(cols // scale, 1), max(k // scale, 1)
            lda, ldb, ldc = m + int(rng.integers(0, 3)), k + int(rng.integers(0, 2)), m + int(rng.integers(0, 2))
            ops.append(dict(kind="gemm", m=m, n=cols, k=k, lda=lda, ldb=ldb, ldc=ldc,
                            A=_vec(gpu, n, rng, lda * k), B=_vec(gpu, n, rng, ldb * cols), C=_vec(gpu, n, rng, ldc * cols),
                            alpha=_vec(gpu, n, rng, 1, -1, 1), beta=_vec(gpu, n, rng, 1, -1, 1)))
    return ops


def _plain(gpu, n, ops):
    out = []
    for o in ops:
        if o["kind"] == "gemv":
            A, x = gpu.DeviceArray.from_host(n, o["A"]), gpu.DeviceArray.from_host(n, o["x"])
            al, be = gpu.DeviceArray.from_host(n, o["alpha"]), gpu.DeviceArray.from_host(n, o["beta"])
            y = gpu.DeviceArray.from_host(n, o["y"])
            gpu.gemv(n, o["trans"], o["m"], o["n"], al, A, o["lda"], x, be, y, o["incx"], o["incy"],
                     order=(256, 128, 256, o["b3"]))
            out.append(y.download())
        elif o["kind"] == "dot":
            x, y = gpu.DeviceArray.from_host(n, o["x"]), gpu.DeviceArray.from_host(n, o["y"])
            r = gpu.DeviceArray.from_host(n, o["r"])
            gpu.dot(n, o["n"], x, y, r, o["incx"], o["incy"], order=(512, 128, 8192, o["g3"], o["b3"]))
            out.append(r.download())
        elif o["kind"] == "gemm":
            A, B = gpu.DeviceArray.from_host(n, o["A"]), gpu.DeviceArray.from_host(n, o["B"])
            al, be = gpu.DeviceArray.from_host(n, o["alpha"]), gpu.DeviceArray.from_host(n, o["beta"])
            C = gpu.DeviceArray.from_host(n, o["C"])
            gpu.gemm(n, o["m"], o["n"], o["k"], al, A, o["lda"], B, o["ldb"], be, C, o["ldc"])
            out.append(C.download())
        else:
            x = gpu.DeviceBytes.from_numpy(o["x"])
            y = gpu.DeviceBytes(o["m"] * (4 * n + 40))
            if o["kind"] == "spmv":
                gpu.spmv_csr(n, o["m"], o["csr"], x, y)
            elif o["kind"] == "csrv":
                gpu.spmv_csrv(n, o["m"], o["csr"], x, y, o["tpr"])
            else:
                gpu.spmv_ell(n, o["m"], o["ell"], x, y)
            out.append(y.to_numpy(o["x"].dtype, o["m"]))
    return out


def _batched(gpu, n, ops, flags, runs=1):
    import torch
    b = gpu.Batch(n)
    outs = []
    for o in ops:
        if o["kind"] == "gemv":
            A, x = gpu.DeviceArray.from_host(n, o["A"]), gpu.DeviceArray.from_host(n, o["x"])
            al, be = gpu.DeviceArray.from_host(n, o["alpha"]), gpu.DeviceArray.from_host(n, o["beta"])
            y = gpu.DeviceArray.from_host(n, o["y"])
            b.add_gemv(o["trans"], o["m"], o["n"], al, A, o["lda"], x, be, y, o["incx"], o["incy"], o["b3"])
            outs.append(y)
        elif o["kind"] == "dot":
            x, y = gpu.DeviceArray.from_host(n, o["x"]), gpu.DeviceArray.from_host(n, o["y"])
            r = gpu.DeviceArray.from_host(n, o["r"])
            b.add_dot(o["n"], x, y, r, o["incx"], o["incy"], o["g3"], o["b3"])
            outs.append(r)
        elif o["kind"] == "gemm":
            A, B = gpu.DeviceArray.from_host(n, o["A"]), gpu.DeviceArray.from_host(n, o["B"])
            al, be = gpu.DeviceArray.from_host(n, o["alpha"]), gpu.DeviceArray.from_host(n, o["beta"])
            C = gpu.DeviceArray.from_host(n, o["C"])
            b.add_gemm(o["m"], o["n"], o["k"], al, A, o["lda"], B, o["ldb"], be, C, o["ldc"])
            outs.append(C)
        else:
            x = gpu.DeviceBytes.from_numpy(o["x"])
            y = gpu.DeviceBytes(o["m"] * (4 * n + 40))
            if o["kind"] == "spmv":
                b.add_spmv_csr(o["m"], o["csr"], x, y)
            elif o["kind"] == "csrv":
                b.add_spmv_csrv(o["m"], o["csr"], x, y, o["tpr"])
            else:
                b.add_spmv_ell(o["m"], o["ell"], x, y)
            outs.append((y, o["m"], o["x"].dtype))
    b.commit(flags)
    for _ in range(runs):
        b.run()
    torch.cuda.synchronize()
    res = [v.download() if isinstance(v, gpu.DeviceArray) else v[0].to_numpy(v[2], v[1]) for v in outs]
    return res, b.info()


@pytest.mark.parametrize("n", [8, 16, 32])
@pytest.mark.parametrize("flags", [0, 1, 3])
@pytest.mark.parametrize("gemm", [False, True])
def test_batch_matches_plain_calls(gpu, n, flags, gemm):
    """With GEMMs in the batch, the GEMM variant of the kernel runs every task."""
    rng = np.random.default_rng(helpers.SEED + 980 + n)
    ops = _build(gpu, n, rng, small=(n == 32), gemm=gemm)
    want = _plain(gpu, n, ops)
    got, info = _batched(gpu, n, ops, flags)
    live = [o for o in ops if (o["kind"] == "gemv" and o["m"] > 0 and o["n"] > 0 and o["incx"] and o["incy"])
            or (o["kind"] == "dot" and o["n"] > 0) or o["kind"] in ("spmv", "csrv", "ell", "gemm")]
    assert info["ops"] == len(live)  # the others are quick returns
    assert info["graph"] == (flags & 1)
    assert info["autotuned"] == (1 if flags & 2 else 0)
    for o, g, w in zip(ops, got, want):
        eq(g, w, "%s %s" % (o["kind"], {k: o[k] for k in o if isinstance(o[k], int)}))


def test_batch_replay_reads_current_operands(gpu):
    """A committed batch reads its operands at run time: a second run continues
    from the GEMV outputs of the first, like a second plain call."""
    n = 8
    rng = np.random.default_rng(helpers.SEED + 990)
    ops = [o for o in _build(gpu, n, rng, small=True) if o["kind"] == "gemv"]
    first = _plain(gpu, n, ops)
    second = _plain(gpu, n, [dict(o, y=w) for o, w in zip(ops, first)])
    got, _ = _batched(gpu, n, ops, gpu.BATCH_GRAPH, runs=2)
    for g, w in zip(got, second):
        eq(g, w, "second run")


def test_batch_of_uneven_gemms_autotuned(gpu):
    """Only GEMMs, 32 moduli, m, n, k from 3 to 150: autotuned and replayed from
    the graph, every C equals the plain mpres_gemm's."""
    n = 32
    rng = np.random.default_rng(helpers.SEED + 995)
    ops = []
    for m, cols, k in rng.integers(3, 151, (12, 3)):
        m, cols, k = int(m), int(cols), int(k)
        ops.append(dict(kind="gemm", m=m, n=cols, k=k, lda=m, ldb=k, ldc=m, A=_vec(gpu, n, rng, m * k),
                        B=_vec(gpu, n, rng, k * cols), C=_vec(gpu, n, rng, m * cols),
                        alpha=_vec(gpu, n, rng, 1, -1, 1), beta=_vec(gpu, n, rng, 1, -1, 1)))
    want = _plain(gpu, n, ops)
    got, info = _batched(gpu, n, ops, gpu.BATCH_GRAPH | gpu.BATCH_AUTOTUNE)
    assert info["threads"] in (128, 256)
    for o, g, w in zip(ops, got, want):
        eq(g, w, "gemm %dx%dx%d" % (o["m"], o["n"], o["k"]))


def test_batch_gemm_rejects_transposition(gpu):
    n = 8
    a = gpu.DeviceArray.from_host(n, gpu.set_d(n, np.ones(4)))
    b = gpu.Batch(n)
    with pytest.raises(gpu.MpresError):
        b.add_gemm(2, 2, 2, a, a, 2, a, 2, a, a, 2, transa=gpu.TRANS)
