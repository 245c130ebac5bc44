#!/usr/bin/env python3
"""Generates the golden vectors of tests/golden/*.npz from the REFERENCE itself.

The reference library's headers are compiled for the CPU by
oracle/ref/build_ref.sh (oracle/_ref/libmpres_ref_<N>.so): its device
arithmetic runs unmodified, its kernels run under a coroutine emulation of CUDA
blocks, and its directed-rounding intrinsics are IEEE operations under
fesetround().  This script feeds it seeded inputs and stores inputs and outputs
(mp_float_t records, bit for bit).  The reference checkout is needed only here;
the committed .npz files are what the tests read.

    bash oracle/ref/build_ref.sh && python tests/golden/make_golden.py [v2] [cg]

(with group names, only those files are regenerated)
"""
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import helpers  # noqa: E402
from oracle import ffi  # noqa: E402

EDGE = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 3.0, 2.0 ** -1022, 5e-324, 1.7976931348623157e308, -2.5e-300,
                 1.0 / 3.0, 2.0 ** 52 + 1, -(2.0 ** 60), 7.0 * 2.0 ** -40])


def elem_case(n, seed):
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    x = np.concatenate([EDGE, helpers.doubles(rng, 400, -60, 60)])
    y = np.concatenate([EDGE[::-1], helpers.doubles(rng, 400, -60, 60)])
    mx, my = R.set_d(x), R.set_d(y)
    prod = R.mul(mx, my)
    s = R.add(mx, my)
    # near cancellation: x + x*(-(1 + tiny)) exercises the ambiguous-sign path
    d = -(1 + np.ldexp(rng.integers(1, 1 << 20, len(x)).astype(float), -52 - rng.integers(0, 20, len(x))))
    q = R.mul_d(mx, d)
    canc = R.add(mx, q)
    # chains of products and sums exercise rounding (power-of-two scaling)
    acc = prod.copy()
    for _ in range(6):
        acc = R.add(R.mul(acc, my), prod)
    dd = rng.standard_normal(len(x))
    muld = R.mul_d(acc, dd)
    return dict(x=x, y=y, mx=mx, my=my, prod=prod, sum=s, d=d, q=q, canc=canc, acc=acc, dd=dd, muld=muld)


def dot_case(n, seed, sizes):
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    out = {}
    for tag, (count, order, incx, incy) in sizes.items():
        lx = 1 + (count - 1) * abs(incx)
        ly = 1 + (count - 1) * abs(incy)
        x = helpers.doubles(rng, lx, -16, 16)
        y = helpers.doubles(rng, ly, -16, 16)
        mx, my = R.set_d(x), R.set_d(y)
        g1, b1, g2, g3, b3 = order
        r = R.dot(mx, my, g1, b1, g2, g3, b3, incx=incx, incy=incy, length=count)
        out.update({tag + "_x": x, tag + "_y": y, tag + "_mx": mx, tag + "_my": my, tag + "_r": r,
                    tag + "_meta": np.array([count, incx, incy] + list(order), np.int64)})
    return out


def gemv_case(n, seed, shapes):
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    out = {}
    for tag, (trans, m, cols, incx, incy, b3) in shapes.items():
        lda = m + 3
        lx = cols if trans == ffi.MBLAS_NO_TRANS else m
        ly = m if trans == ffi.MBLAS_NO_TRANS else cols
        A = helpers.doubles(rng, lda * cols, -32, 32)
        x = helpers.doubles(rng, 1 + (lx - 1) * abs(incx), -32, 32)
        y = helpers.doubles(rng, 1 + (ly - 1) * abs(incy), -32, 32)
        ab = rng.uniform(-1, 1, 2)
        mA, mx, my, ma, mb = R.set_d(A), R.set_d(x), R.set_d(y), R.set_d(ab[:1]), R.set_d(ab[1:])
        r = R.gemv(trans, m, cols, ma, mA, lda, mx, mb, my, incx=incx, incy=incy, b3=b3)
        out.update({tag + "_A": mA, tag + "_x": mx, tag + "_y": my, tag + "_alpha": ma, tag + "_beta": mb,
                    tag + "_r": r, tag + "_meta": np.array([trans, m, cols, lda, incx, incy, b3], np.int64)})
    return out


def gemm_case(n, seed, shapes):
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    out = {}
    for tag, (m, cols, k) in shapes.items():
        lda, ldb, ldc = m + 1, k + 2, m + 3
        A = helpers.doubles(rng, lda * k, -32, 32)
        B = helpers.doubles(rng, ldb * cols, -32, 32)
        C = helpers.doubles(rng, ldc * cols, -32, 32)
        ab = rng.uniform(-1, 1, 2)
        mA, mB, mC, ma, mb = R.set_d(A), R.set_d(B), R.set_d(C), R.set_d(ab[:1]), R.set_d(ab[1:])
        r = R.gemm(m, cols, k, ma, mA, lda, mB, ldb, mb, mC, ldc)
        out.update({tag + "_A": mA, tag + "_B": mB, tag + "_C": mC, tag + "_alpha": ma, tag + "_beta": mb,
                    tag + "_r": r, tag + "_meta": np.array([m, cols, k, lda, ldb, ldc], np.int64)})
    return out


def spmv_case(n, seed, m, kmax):
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    lengths = helpers.power_law_rows(rng, m, kmax=kmax)
    lengths[:3] = [0, 1, kmax]  # an empty row, a single entry, a full-length row
    irp, ja, vals = helpers.random_csr(rng, m, m, lengths)
    vals[::37] = 0.0  # explicit zeros (the ELL kernel skips them, CSR does not)
    x = helpers.doubles(rng, m, -16, 16)
    mx = R.set_d(x)
    out = dict(irp=irp, ja=ja, vals=vals, x=x, mx=mx, csr=R.spmv_csr(m, irp, ja, vals, mx))
    for tpr in (1, 2, 4, 8, 16, 32):
        out["csrv%d" % tpr] = R.spmv_csrv(m, tpr, irp, ja, vals, mx)
    maxnzr, ell_ja, ell_as = helpers.csr_to_ell(m, irp, ja, vals)
    out.update(ell_ja=ell_ja, ell_as=ell_as, maxnzr=np.array([maxnzr]), ell=R.spmv_ell(m, maxnzr, ell_ja, ell_as, mx))
    return out


def spd_csr(rng, m, per_row):
    """A symmetric, strictly diagonally dominant (so positive definite) sparse
    matrix in CSR: random off-diagonal N(0,1) entries mirrored, diagonal = sum
    of |row| + 1."""
    rows = {i: {} for i in range(m)}
    for i in range(m):
        for j in rng.choice(m, size=per_row, replace=False):
            if j != i:
                v = float(rng.standard_normal())
                rows[i][int(j)] = v
                rows[int(j)][i] = v
    irp, ja, vals = [0], [], []
    for i in range(m):
        rows[i][i] = sum(abs(v) for v in rows[i].values()) + 1.0
        for j in sorted(rows[i]):
            ja.append(j)
            vals.append(rows[i][j])
        irp.append(len(ja))
    return np.array(irp, np.int32), np.array(ja, np.int32), np.array(vals)


def cg_case(n, seed, m):
    """mp_cg_csr<32, 256> and mp_pcg_csr<64, 256> (Jacobi) on an SPD matrix."""
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    irp, ja, vals = spd_csr(rng, m, 3)
    b = R.set_d(helpers.doubles(rng, m, -4, 4))
    x0 = R.set_d(np.zeros(m))
    diag = np.array([vals[irp[i] + list(ja[irp[i]:irp[i + 1]]).index(i)] for i in range(m)])
    M = 1.0 / diag
    out = dict(irp=irp, ja=ja, vals=vals, b=b, x0=x0, M=M)
    for tag, kw in (("cg", dict(threads=32, blocks=256)), ("pcg", dict(M=M, threads=64, blocks=256))):
        k, x, res = ffi.ref_cg(n, irp, ja, vals, b, 1e-30, 40, x0, **kw)
        out.update({tag + "_x": x, tag + "_res": res, tag + "_iters": np.array([k])})
    return out


def v2_case(n, seed):
    """mp_add_abs and the v2 dot / sum of squares."""
    R = ffi.reference(n)
    rng = np.random.default_rng(seed)
    x = R.set_d(helpers.doubles(rng, 3000, -30, 30))
    y = R.set_d(helpers.doubles(rng, 3000, -30, 30))
    out = dict(x=x, y=y, add_abs=ffi.ref_add_abs(n, x, y))
    for blocks, threads in ((256, 32), (256, 64), (7, 33)):
        out["dot_%d_%d" % (blocks, threads)] = ffi.ref_reduce_v2(n, False, x, y, blocks, threads)
        out["sumsq_%d_%d" % (blocks, threads)] = ffi.ref_reduce_v2(n, True, x, None, blocks, threads)
    return out


def main():
    if not ffi.ref_available(8):
        raise SystemExit("build the reference first: bash oracle/ref/build_ref.sh")
    base = helpers.SEED
    only = set(sys.argv[1:])
    if only:  # regenerate the named groups only: v2, cg
        if "v2" in only:
            for n in (8, 16):
                np.savez_compressed(HERE / ("v2_%d.npz" % n), **v2_case(n, base + 200 + n))
        if "cg" in only:
            np.savez_compressed(HERE / "cg_8.npz", **cg_case(8, base + 210, 300))
        return
    for n in (8, 16, 32):
        np.savez_compressed(HERE / ("elem_%d.npz" % n), **elem_case(n, base + 100 + n))
    np.savez_compressed(HERE / "dot_8.npz", **dot_case(8, base + 0, {
        "perf": (1500, (512, 128, 8192, 256, 64), 1, 1),
        "acc": (1200, (512, 128, 8192, 64, 64), 1, 1),
        "odd": (777, (32, 64, 64, 7, 33), 1, 1),
        "strided": (500, (64, 32, 128, 5, 16), 2, -3),
        "one": (1, (512, 128, 8192, 256, 64), 1, 1),
    }))
    np.savez_compressed(HERE / "dot_16.npz", **dot_case(16, base + 16, {
        "perf": (1500, (512, 128, 8192, 256, 64), 1, 1)}))
    np.savez_compressed(HERE / "dot_32.npz", **dot_case(32, base + 32, {
        "perf": (800, (512, 128, 8192, 256, 64), 1, 1)}))
    np.savez_compressed(HERE / "gemv_16.npz", **gemv_case(16, base + 3, {
        "n32": (ffi.MBLAS_NO_TRANS, 40, 24, 1, 1, 32),
        "t32": (ffi.MBLAS_TRANS, 24, 36, 1, 1, 32),
        "n5": (ffi.MBLAS_NO_TRANS, 21, 40, -2, 3, 5),
        "t64": (ffi.MBLAS_TRANS, 70, 10, 2, -1, 64),
    }))
    np.savez_compressed(HERE / "gemv_8.npz", **gemv_case(8, base + 30, {
        "n32": (ffi.MBLAS_NO_TRANS, 48, 40, 1, 1, 32)}))
    np.savez_compressed(HERE / "gemm_32.npz", **gemm_case(32, base + 1, {"a": (24, 20, 28)}))
    np.savez_compressed(HERE / "gemm_8.npz", **gemm_case(8, base + 10, {"a": (17, 9, 33), "b": (5, 31, 1)}))
    np.savez_compressed(HERE / "spmv_8.npz", **spmv_case(8, base + 2, 600, 64))
    for n in (8, 16):
        np.savez_compressed(HERE / ("v2_%d.npz" % n), **v2_case(n, base + 200 + n))
    np.savez_compressed(HERE / "cg_8.npz", **cg_case(8, base + 210, 300))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
