"""The library against the reference's OWN device code running on the same GPU:
the reference headers compiled unmodified for sm_103a (oracle/_ref/ref_kernels_<N>.cubin,
built with the reference checkout by oracle/ref/build_ref.sh) with the constant
tables its rns_const_init / mp_const_init compute.  Bit-identical results for the
device arithmetic (cuda::mp_add, mp_mul, mp_mul_d, which carry the rounding, the
interval evaluation and the power-of-two scaling), for mp_dot, mp_gemm and
mp_spmv_csr at the reference's launch configurations.  Skipped where the cubin
was not built (no reference checkout)."""
import numpy as np
import pytest

import helpers
from oracle import ffi, ref_gpu

pytestmark = pytest.mark.gpu


def need(n):
    if not ref_gpu.available(n):
        pytest.skip("reference cubin for %d moduli not built (no reference checkout)" % n)
    return ref_gpu.ref_gpu(n)


def eq(a, b, what):
    mm = ffi.mismatches(a, b)
    assert len(mm) == 0, "%s: %d of %d records differ, first at %d" % (what, len(mm), len(a), mm[0])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_device_arithmetic_matches_reference_gpu(gpu, n):
    """Chains of products, sums and products by doubles with exponents over
    +-60 (roundings of several scaling steps, ambiguous signs), each generation
    computed by the reference's device functions and by the library from the
    same operands."""
    ref = need(n)
    rng = np.random.default_rng(helpers.SEED + 1900 + n)
    cnt = 20000
    pool = gpu.set_d(n, helpers.doubles(rng, cnt, -60, 60))
    for gen in range(9):
        i, j = rng.integers(0, len(pool), cnt), rng.integers(0, len(pool), cnt)
        a, b = pool[i].copy(), pool[j].copy()
        if gen % 3 == 0:
            want, got = ref.elementwise("mul", a, b), gpu.elementwise(n, gpu.OP_MUL, a, b)
        elif gen % 3 == 1:
            want, got = ref.elementwise("add", a, b), gpu.elementwise(n, gpu.OP_ADD, a, b)
        else:
            d = -(1 + np.ldexp(rng.integers(1, 1 << 20, cnt).astype(float), -52 - rng.integers(0, 20, cnt)))
            want, got = ref.elementwise("mul_d", a, d), gpu.elementwise(n, gpu.OP_MUL_D, a, d)
        eq(got, want, "generation %d" % gen)
        pool = np.concatenate([pool, want])[-60000:]


@pytest.mark.parametrize("n,count", [(8, 1 << 20), (16, 100003), (32, 30011)])
def test_dot_matches_reference_gpu(gpu, n, count):
    """mp_dot at the reference benchmark's order <512,128,8192,256,64>; 2^20
    elements with 8 moduli is the DOT benchmark."""
    ref = need(n)
    import torch
    rng = np.random.default_rng(helpers.SEED + count + n)
    mx = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    my = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    x, y = ref_gpu.RefArray(n, count).upload(mx), ref_gpu.RefArray(n, count).upload(my)
    r, buf = ref_gpu.RefArray(n, 1), ref_gpu.RefArray(n, count)
    ref.dot(count, x, y, r, buf)
    ref.sync()
    want = r.download(mx.dtype)
    dx, dy, dr = gpu.DeviceArray.from_host(n, mx), gpu.DeviceArray.from_host(n, my), gpu.DeviceArray(n, 1)
    gpu.dot(n, count, dx, dy, dr, order=(512, 128, 8192, 256, 64))
    torch.cuda.synchronize()
    eq(dr.download(), want, "dot")


@pytest.mark.parametrize("n,m,cols,k,lo", [(32, 256, 128, 256, -32), (8, 100, 70, 300, -32), (16, 64, 64, 130, -300)])
def test_gemm_matches_reference_gpu(gpu, n, m, cols, k, lo):
    ref = need(n)
    import torch
    rng = np.random.default_rng(helpers.SEED + 1950 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * k, lo, -lo))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, lo, -lo))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, lo, -lo))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    rA, rB, rC = (ref_gpu.RefArray(n, len(v)).upload(v) for v in (A, B, C))
    ral, rbe = ref_gpu.RefArray(n, 1).upload(al), ref_gpu.RefArray(n, 1).upload(be)
    ref.gemm(m, cols, k, ral, rA, m, rB, k, rbe, rC, m, ref_gpu.RefArray(n, m * cols))
    ref.sync()
    want = rC.download(C.dtype)
    dA, dB, dC = (gpu.DeviceArray.from_host(n, v) for v in (A, B, C))
    dal, dbe = gpu.DeviceArray.from_host(n, al), gpu.DeviceArray.from_host(n, be)
    gpu.gemm(n, m, cols, k, dal, dA, m, dB, k, dbe, dC, m)
    torch.cuda.synchronize()
    eq(dC.download(), want, "gemm")


def test_spmv_csr_matches_reference_gpu(gpu):
    """2^18 power-law rows (1..1024), 8 moduli."""
    n = 8
    ref = need(n)
    import torch
    rng = np.random.default_rng(helpers.SEED + 1960)
    m = 1 << 18
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    mx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    x = gpu.DeviceBytes.from_numpy(mx)
    y_ref, y_lib = gpu.DeviceBytes(m * mx.dtype.itemsize), gpu.DeviceBytes(m * mx.dtype.itemsize)
    csr = gpu.DeviceCsr(m, irp, ja, vals)
    ref.spmv_csr(m, csr.c.irp, csr.c.ja, csr.c.as_, x.ptr, y_ref.ptr)
    ref.sync()
    gpu.spmv_csr(n, m, csr, x, y_lib)
    torch.cuda.synchronize()
    eq(y_lib.to_numpy(mx.dtype, m), y_ref.to_numpy(mx.dtype, m), "spmv_csr")


def _timed(fn, reps):
    import time
    import torch
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    return best * 1e3


def test_benchmark_sizes_against_reference_gpu(gpu, oracle, capsys):
    """The three benchmark workloads run by the reference's own kernels and by the
    library on the same GPU, same inputs: bit-identical results, and the times of
    both (best of a few runs, host clock around a synchronised pipeline) printed as
    one JSON line.  GEMM 1024^3 with 32 moduli, DOT 2^20 with 8, CSR SpMV over
    2^20 power-law rows with 8."""
    import json
    import torch
    if not all(ref_gpu.available(n) for n in (8, 32)):
        pytest.skip("reference cubins not built (no reference checkout)")
    out = {}
    rng = np.random.default_rng(helpers.SEED + 1)
    # GEMM
    n, m = 32, 1024
    ref = ref_gpu.ref_gpu(n)
    A = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, m * m, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    rA, rB = ref_gpu.RefArray(n, m * m).upload(A), ref_gpu.RefArray(n, m * m).upload(B)
    rC, rbuf = ref_gpu.RefArray(n, m * m), ref_gpu.RefArray(n, m * m)
    ral, rbe = ref_gpu.RefArray(n, 1).upload(al), ref_gpu.RefArray(n, 1).upload(be)
    rC.upload(C)
    ref.gemm(m, m, m, ral, rA, m, rB, m, rbe, rC, m, rbuf)
    ref.sync()
    want = rC.download(C.dtype)
    dA, dB, dC = (gpu.DeviceArray.from_host(n, v) for v in (A, B, C))
    dal, dbe = gpu.DeviceArray.from_host(n, al), gpu.DeviceArray.from_host(n, be)
    gpu.gemm(n, m, m, m, dal, dA, m, dB, m, dbe, dC, m)
    torch.cuda.synchronize()
    eq(dC.download(), want, "gemm 1024^3")
    out["gemm_1024_32moduli_ms"] = {
        "reference": _timed(lambda: ref.gemm(m, m, m, ral, rA, m, rB, m, rbe, rC, m, rbuf), 2),
        "library": _timed(lambda: gpu.gemm(n, m, m, m, dal, dA, m, dB, m, dbe, dC, m), 5)}
    del rA, rB, rC, rbuf, dA, dB, dC
    # DOT
    n, count = 8, 1 << 20
    ref = ref_gpu.ref_gpu(n)
    mx = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    my = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
    x, y = ref_gpu.RefArray(n, count).upload(mx), ref_gpu.RefArray(n, count).upload(my)
    r, buf = ref_gpu.RefArray(n, 1), ref_gpu.RefArray(n, count)
    ref.dot(count, x, y, r, buf)
    ref.sync()
    dx, dy, dr = gpu.DeviceArray.from_host(n, mx), gpu.DeviceArray.from_host(n, my), gpu.DeviceArray(n, 1)
    gpu.dot(n, count, dx, dy, dr)
    torch.cuda.synchronize()
    eq(dr.download(), r.download(mx.dtype), "dot 2^20")
    out["dot_2^20_8moduli_ms"] = {"reference": _timed(lambda: ref.dot(count, x, y, r, buf), 10),
                                  "library": _timed(lambda: gpu.dot(n, count, dx, dy, dr), 10)}
    # SpMV
    rows = 1 << 20
    irp, ja, vals = helpers.random_csr(rng, rows, rows, helpers.power_law_rows(rng, rows))
    mxs = gpu.set_d(n, helpers.doubles(rng, rows, -16, 16))
    xs = gpu.DeviceBytes.from_numpy(mxs)
    ys_ref, ys_lib = gpu.DeviceBytes(rows * mxs.dtype.itemsize), gpu.DeviceBytes(rows * mxs.dtype.itemsize)
    csr = gpu.DeviceCsr(rows, irp, ja, vals)
    run_ref = lambda: ref.spmv_csr(rows, csr.c.irp, csr.c.ja, csr.c.as_, xs.ptr, ys_ref.ptr)  # noqa: E731
    run_lib = lambda: gpu.spmv_csr(n, rows, csr, xs, ys_lib)  # noqa: E731
    run_ref()
    ref.sync()
    run_lib()
    torch.cuda.synchronize()
    eq(ys_lib.to_numpy(mxs.dtype, rows), ys_ref.to_numpy(mxs.dtype, rows), "spmv_csr 2^20 rows")
    out["spmv_csr_2^20rows_8moduli_ms"] = {"reference": _timed(run_ref, 5), "library": _timed(run_lib, 5)}
    for v in out.values():
        v["speedup"] = v["reference"] / v["library"]
    with capsys.disabled():
        print("\nREFERENCE_GPU " + json.dumps(out))


def test_spmv_forms_against_reference_gpu(gpu, capsys):
    """CSR-vector (tpr 4, 16, 32) and ELL over the SpMV benchmark matrix (2^20
    power-law rows, 8 moduli) by the reference's own kernels at its drivers'
    launch shapes and by the library: bit-identical, and both times printed.
    The ELL slots (12.9 GB) are built on the device from the CSR arrays."""
    import json
    import torch
    n = 8
    ref = need(n)
    rng = np.random.default_rng(helpers.SEED + 2)
    m = 1 << 20
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
    mx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    rec = mx.dtype.itemsize
    x = gpu.DeviceBytes.from_numpy(mx)
    y_ref, y_lib = gpu.DeviceBytes(m * rec), gpu.DeviceBytes(m * rec)
    csr = gpu.DeviceCsr(m, irp, ja, vals)
    out = {}
    for tpr in (4, 16, 32):
        run_ref = lambda: ref.spmv_csrv(m, tpr, csr.c.irp, csr.c.ja, csr.c.as_, x.ptr, y_ref.ptr)  # noqa: E731
        run_lib = lambda: gpu.spmv_csrv(n, m, csr, x, y_lib, tpr)  # noqa: E731
        run_ref()
        ref.sync()
        run_lib()
        torch.cuda.synchronize()
        eq(y_lib.to_numpy(mx.dtype, m), y_ref.to_numpy(mx.dtype, m), "spmv_csrv tpr %d" % tpr)
        out["spmv_csrv%d_ms" % tpr] = {"reference": _timed(run_ref, 3), "library": _timed(run_lib, 3)}
    lens = np.diff(irp).astype(np.int64)
    maxnzr = int(lens.max())
    irp_t = torch.from_numpy(irp.astype(np.int64)).cuda()
    rows = torch.repeat_interleave(torch.arange(m, device="cuda"), torch.from_numpy(lens).cuda())
    slot = (torch.arange(len(ja), device="cuda") - irp_t[:-1][rows]) * m + rows
    del rows
    ell_ja = torch.zeros(maxnzr * m, dtype=torch.int32, device="cuda")
    ell_as = torch.zeros(maxnzr * m, dtype=torch.float64, device="cuda")
    ell_ja[slot] = torch.from_numpy(ja.astype(np.int32)).cuda()
    ell_as[slot] = torch.from_numpy(vals).cuda()
    del slot, irp_t
    csr.free()
    ell = gpu.DeviceEll.from_tensors(m, maxnzr, ell_ja, ell_as)
    run_ref = lambda: ref.spmv_ell(m, maxnzr, ell_ja.data_ptr(), ell_as.data_ptr(), x.ptr, y_ref.ptr)  # noqa: E731
    run_lib = lambda: gpu.spmv_ell(n, m, ell, x, y_lib)  # noqa: E731
    run_ref()
    ref.sync()
    run_lib()
    torch.cuda.synchronize()
    eq(y_lib.to_numpy(mx.dtype, m), y_ref.to_numpy(mx.dtype, m), "spmv_ell")
    out["spmv_ell_ms"] = {"reference": _timed(run_ref, 3), "library": _timed(run_lib, 3)}
    for v in out.values():
        v["speedup"] = v["reference"] / v["library"]
    with capsys.disabled():
        print("\nREFERENCE_GPU_SPMV " + json.dumps(out))


@pytest.mark.parametrize("n,m,cols", [(16, 1024, 1024), (8, 300, 77), (32, 64, 200)])
def test_gemv_matches_reference_gpu(gpu, n, m, cols):
    """mp_gemv without transposition at the reference benchmark's <256,128,256,32>."""
    ref = need(n)
    import torch
    rng = np.random.default_rng(helpers.SEED + 1970 + n)
    A = gpu.set_d(n, helpers.doubles(rng, m * cols, -32, 32))
    x = gpu.set_d(n, helpers.doubles(rng, cols, -32, 32))
    y = gpu.set_d(n, helpers.doubles(rng, m, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    rA, rx, ry = (ref_gpu.RefArray(n, len(v)).upload(v) for v in (A, x, y))
    ral, rbe = ref_gpu.RefArray(n, 1).upload(al), ref_gpu.RefArray(n, 1).upload(be)
    ref.gemv(m, cols, ral, rA, m, rx, rbe, ry, ref_gpu.RefArray(n, cols), ref_gpu.RefArray(n, m * cols))
    ref.sync()
    dA, dx, dy = (gpu.DeviceArray.from_host(n, v) for v in (A, x, y))
    dal, dbe = gpu.DeviceArray.from_host(n, al), gpu.DeviceArray.from_host(n, be)
    gpu.gemv(n, gpu.NO_TRANS, m, cols, dal, dA, m, dx, dbe, dy, order=(256, 128, 256, 32))
    torch.cuda.synchronize()
    eq(dy.download(), ry.download(y.dtype), "gemv")


def test_gemv_batch_sample_against_reference_gpu(gpu, capsys):
    """64 GEMVs of the batched configuration (m, n log-uniform in [32, 4096],
    entries u*2^e with e in [-32, 32], 16 moduli, NO_TRANS, blockDim3 32): the
    reference's mp_gemv called once per instance, the library's plain calls and
    one batched launch, all bit-identical; the three times printed.  Each
    reference call gets its operands as arrays of their own (copies made outside
    the timed calls): its kernels read a scalar's upper bound at eval[1]."""
    import json
    import time
    import torch
    n, count, b3 = 16, 64, 32
    ref = need(n)
    sizes = np.exp(np.random.default_rng(helpers.SEED + 1980).uniform(np.log(32), np.log(4096 + 1), (count, 2)))
    sizes = np.minimum(sizes.astype(np.int64), 4096)
    M, K = sizes[:, 0], sizes[:, 1]
    a_off = np.concatenate([[0], np.cumsum(M * K)])
    x_off = np.concatenate([[0], np.cumsum(K)])
    y_off = np.concatenate([[0], np.cumsum(M)])
    gen = torch.Generator(device="cuda")
    gen.manual_seed(helpers.SEED + 1981)

    def fill(arr):
        u = torch.rand(arr.size, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
        e = torch.randint(-32, 33, (arr.size,), generator=gen, device="cuda", dtype=torch.int64)
        arr.set_d(torch.ldexp(u, e))

    A, X, Y = gpu.TensorArray(n, int(a_off[-1])), gpu.TensorArray(n, int(x_off[-1])), gpu.TensorArray(n, int(y_off[-1]))
    AB = gpu.TensorArray(n, 2 * count)
    for arr in (A, X, Y):
        fill(arr)
    AB.set_d(torch.rand(2 * count, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
    ops = [(int(M[j]), int(K[j]), AB.view(2 * j, 1), A.view(int(a_off[j]), int(M[j] * K[j])),
            X.view(int(x_off[j]), int(K[j])), AB.view(2 * j + 1, 1), Y.view(int(y_off[j]), int(M[j])))
           for j in range(count)]
    torch.cuda.synchronize()
    y0 = Y.download()

    # the reference, one call at a time on arrays of their own
    buf1 = ref_gpu.RefArray(n, int(K.max()))
    buf2 = ref_gpu.RefArray(n, int((M * K).max()))
    t_ref = 0.0
    for j in range(count):
        m, k = int(M[j]), int(K[j])
        rA = ref_gpu.RefArray.copy_of(A, int(a_off[j]), m * k)
        rx = ref_gpu.RefArray.copy_of(X, int(x_off[j]), k)
        ry = ref_gpu.RefArray.copy_of(Y, int(y_off[j]), m)
        ral, rbe = ref_gpu.RefArray.copy_of(AB, 2 * j, 1), ref_gpu.RefArray.copy_of(AB, 2 * j + 1, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref.gemv(m, k, ral, rA, m, rx, rbe, ry, buf1, buf2)
        ref.sync()
        t_ref += time.perf_counter() - t0
        ry.copy_into(Y, int(y_off[j]))
        del rA
    torch.cuda.synchronize()
    y_ref = Y.download()

    def run_plain():
        for m, k, al, Av, xv, be, yv in ops:
            gpu.gemv(n, gpu.NO_TRANS, m, k, al, Av, m, xv, be, yv, order=(256, 128, 256, b3))

    batch = gpu.Batch(n)
    for m, k, al, Av, xv, be, yv in ops:
        batch.add_gemv(gpu.NO_TRANS, m, k, al, Av, m, xv, be, yv, b3=b3)
    Y.upload(y0)
    batch.commit(gpu.BATCH_GRAPH | gpu.BATCH_AUTOTUNE)
    torch.cuda.synchronize()

    def timed_once(fn):
        Y.upload(y0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, Y.download()

    timed_once(run_plain)
    t_plain, y_plain = timed_once(run_plain)
    timed_once(batch.run)
    t_batch, y_batch = timed_once(batch.run)
    eq(y_plain, y_ref, "plain calls against the reference")
    eq(y_batch, y_ref, "batched launch against the reference")
    batch.destroy()
    out = {"gemv_x64_16moduli_ms": {"reference": t_ref * 1e3, "library_plain": t_plain, "library_batched": t_batch,
                                    "speedup_plain": t_ref * 1e3 / t_plain, "speedup_batched": t_ref * 1e3 / t_batch,
                                    "mp_elements_of_A": int(a_off[-1])}}
    with capsys.disabled():
        print("\nREFERENCE_GPU_GEMV " + json.dumps(out))
