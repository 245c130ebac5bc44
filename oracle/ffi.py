"""ctypes access to the CPU oracle and to the reference built for the CPU.

TEST INFRASTRUCTURE ONLY.  Loads
  oracle/_build/libmpres_oracle.so   the C restatement (builds with `make -C oracle`)
  oracle/_ref/libmpres_ref_<N>.so    the reference compiled here (oracle/ref/build_ref.sh),
                                     present only where the reference checkout exists.
Numbers travel as numpy structured arrays in the reference's mp_float_t layout.
"""
import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libmpres_oracle.so"
REF_DIR = HERE / "_ref"

ER = np.dtype([("frac", "<f8"), ("exp", "<i8")])
P = ctypes.c_void_p
MBLAS_NO_TRANS, MBLAS_TRANS = 111, 112


def mp_dtype(n):
    """mp_float_t of the reference (src/types.cuh:69-74) for n moduli: 4n + 40 bytes."""
    dt = np.dtype([("digits", "<i4", (n,)), ("sign", "<i4"), ("exp", "<i4"), ("eval", ER, (2,))])
    assert dt.itemsize == 4 * n + 40
    return dt


def ptr(a):
    return a.ctypes.data_as(P)


def build_oracle():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def reference_root():
    """The reference checkout's root directory, or None where it is absent (the
    location is named by the recipe oracle/ref/build_ref.sh alone)."""
    r = subprocess.run(["bash", str(HERE / "ref" / "build_ref.sh"), "--where"], capture_output=True, text=True)
    root = r.stdout.strip()
    return pathlib.Path(root) if r.returncode == 0 and root else None


_oracle = None
_mpfr = None
MPFR_SO = HERE / "_build" / "libmpres_mpfr.so"


class MpfrBlas:
    """The reference's MPFR/OpenMP loops (oracle/mpfr_blas.c).  Each call
    returns (seconds of the timed loop, results rounded to double)."""

    D = ctypes.POINTER(ctypes.c_double)

    def __init__(self, lib):
        self.lib = lib
        for name in ("mpb_dot", "mpb_gemm", "mpb_spmv_csr"):
            getattr(lib, name).restype = ctypes.c_double

    def threads(self):
        return int(self.lib.mpb_max_threads())

    def dot(self, x, y, prec, threads=None):
        x, y = np.ascontiguousarray(x, np.float64), np.ascontiguousarray(y, np.float64)
        out = np.zeros(1)
        t = self.lib.mpb_dot(len(x), ptr(x), ptr(y), ctypes.c_long(prec), threads or self.threads(), ptr(out))
        return t, out[0]

    def gemm(self, rows, cols, k, alpha, A, lda, B, ldb, beta, C, ldc, prec, threads=None):
        A, B, C = (np.ascontiguousarray(v, np.float64) for v in (A, B, C))
        out = np.zeros(rows * cols)
        t = self.lib.mpb_gemm(rows, cols, k, ctypes.c_double(alpha), ptr(A), lda, ptr(B), ldb, ctypes.c_double(beta),
                              ptr(C), ldc, ctypes.c_long(prec), threads or self.threads(), ptr(out))
        if t < 0:
            raise MemoryError("mpb_gemm: allocation failed")
        return t, out

    def spmv_csr(self, m, irp, ja, vals, x, prec, threads=None):
        irp, ja = np.ascontiguousarray(irp, np.int32), np.ascontiguousarray(ja, np.int32)
        vals, x = np.ascontiguousarray(vals, np.float64), np.ascontiguousarray(x, np.float64)
        out = np.zeros(m)
        t = self.lib.mpb_spmv_csr(m, len(x), ptr(irp), ptr(ja), ptr(vals), ptr(x), ctypes.c_long(prec),
                                  threads or self.threads(), ptr(out))
        return t, out


def mpfr_blas():
    """The MPFR baseline library, or None where the host has no libmpfr.so.6."""
    global _mpfr
    if _mpfr is None:
        if not MPFR_SO.exists():
            build_oracle()
        if not MPFR_SO.exists():
            return None
        _mpfr = MpfrBlas(ctypes.CDLL(str(MPFR_SO)))
    return _mpfr


def mp_precision(n):
    """MP_PRECISION of the predefined set of n moduli (src/arith/arith_utils.cuh:50)."""
    return {8: 120, 16: 240, 32: 480}[n]


def oracle():
    """The C oracle (built on first use)."""
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build_oracle()
        lib = ctypes.CDLL(str(ORACLE_SO))
        lib.ora_init.restype = P
        _oracle = Oracle(lib)
    return _oracle


class _Common:
    """Wrappers shared by the oracle and the reference library."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.p = prefix

    def _f(self, name):
        return getattr(self.lib, self.p + name)


class Oracle(_Common):
    def __init__(self, lib):
        super().__init__(lib, "ora_")

    def threads(self):
        return self.lib.ora_threads()

    def set_d(self, n, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(x.size, mp_dtype(n))
        self.lib.ora_set_d(n, ptr(x), ctypes.c_long(x.size), ptr(out))
        return out

    def tables(self, n, log2m):
        return _tables(lambda *a: self.lib.ora_tables(n, *a), n, log2m)

    def add(self, n, x, y):
        r = np.zeros(len(x), mp_dtype(n))
        self.lib.ora_add(n, ptr(x), ptr(y), ptr(r), ctypes.c_long(len(x)))
        return r

    def mul(self, n, x, y):
        r = np.zeros(len(x), mp_dtype(n))
        self.lib.ora_mul(n, ptr(x), ptr(y), ptr(r), ctypes.c_long(len(x)))
        return r

    def mul_d(self, n, x, d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        r = np.zeros(len(x), mp_dtype(n))
        self.lib.ora_mul_d(n, ptr(x), ptr(d), ptr(r), ctypes.c_long(len(x)))
        return r

    def eval_fast(self, n, digits):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        cnt = digits.size // n
        lo, up = np.zeros(cnt, ER), np.zeros(cnt, ER)
        self.lib.ora_eval_fast(n, ptr(digits), ptr(lo), ptr(up), ctypes.c_long(cnt))
        return lo, up

    def eval(self, n, digits):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        cnt = digits.size // n
        lo, up = np.zeros(cnt, ER), np.zeros(cnt, ER)
        self.lib.ora_eval(n, ptr(digits), ptr(lo), ptr(up), ctypes.c_long(cnt))
        return lo, up

    def scale2pow(self, n, digits, D):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        D = np.ascontiguousarray(D, dtype=np.uint32)
        out = np.zeros_like(digits)
        self.lib.ora_scale2pow(n, ptr(digits), ptr(D), ptr(out), ctypes.c_long(D.size))
        return out

    def add_abs(self, n, x, y):
        r = np.zeros(len(x), mp_dtype(n))
        self.lib.ora_add_abs(n, ptr(x), ptr(y), ptr(r), ctypes.c_long(len(x)))
        return r

    def reduce_v2(self, n, sumsq, x, y, blocks, threads):
        r = np.zeros(1, mp_dtype(n))
        self.lib.ora_reduce_v2(n, int(sumsq), len(x), ptr(x), ptr(y if y is not None else x), ptr(r), blocks, threads)
        return r

    def dot(self, n, x, y, g3=256, b3=64, incx=1, incy=1, length=None):
        length = len(x) if length is None else length
        r = np.zeros(1, mp_dtype(n))
        self.lib.ora_dot(n, length, ptr(x), incx, ptr(y), incy, ptr(r), g3, b3)
        return r

    def gemv(self, n, trans, m, cols, alpha, A, lda, x, beta, y, incx=1, incy=1, b3=32):
        y = y.copy()
        self.lib.ora_gemv(n, trans, m, cols, ptr(alpha), ptr(A), lda, ptr(x), incx, ptr(beta), ptr(y), incy, b3)
        return y

    def gemm(self, n, m, cols, k, alpha, A, lda, B, ldb, beta, C, ldc):
        C = C.copy()
        self.lib.ora_gemm(n, m, cols, k, ptr(alpha), ptr(A), lda, ptr(B), ldb, ptr(beta), ptr(C), ldc)
        return C

    def spmv_csr(self, n, m, irp, ja, vals, x):
        y = np.zeros(m, mp_dtype(n))
        self.lib.ora_spmv_csr(n, m, ptr(irp), ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y

    def spmv_csrv(self, n, m, tpr, irp, ja, vals, x):
        y = np.zeros(m, mp_dtype(n))
        self.lib.ora_spmv_csrv(n, m, tpr, ptr(irp), ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y

    def spmv_ell(self, n, m, maxnzr, ja, vals, x):
        y = np.zeros(m, mp_dtype(n))
        self.lib.ora_spmv_ell(n, m, maxnzr, ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y


def _tables(fn, n, log2m):
    t = dict(
        part_inv=np.zeros(n, np.int32),
        pow2=np.zeros((log2m + 1) * n, np.int32),
        m_pow2_res=np.zeros(30, np.int32),
        part_pow2_res=np.zeros(30 * n, np.int32),
        pow2_inv=np.zeros(30 * n, np.int32),
        recip_rd=np.zeros(n, np.float64),
        recip_ru=np.zeros(n, np.float64),
        mrc_inv=np.zeros(n * n, np.int32),
        eval_acc=np.zeros(1, np.float64),
        ref_factor=np.zeros(1, np.int32),
        units=np.zeros(4, ER),
        mp_consts=np.zeros(3, np.int32),
    )
    fn(*[ptr(v) for v in t.values()])
    return t


def ref_add_abs(n, x, y):
    r = np.zeros(len(x), mp_dtype(n))
    reference(n).lib.ref_add_abs(ptr(x), ptr(y), ptr(r), ctypes.c_long(len(x)))
    return r


def ref_reduce_v2(n, sumsq, x, y, blocks, threads):
    r = np.zeros(1, mp_dtype(n))
    reference(n).lib.ref_reduce_v2(int(sumsq), len(x), ptr(x), ptr(y if y is not None else x), ptr(r), blocks, threads)
    return r


def ref_cg(n, irp, ja, vals, b, tol, maxit, x0, M=None, threads=32, blocks=256):
    """The reference's mp_cg_csr (M None) or mp_pcg_csr (M = inverse diagonal):
    (iterations, x, resvec)."""
    x = x0.copy()
    res = np.zeros(maxit + 2)
    irp, ja = np.ascontiguousarray(irp, np.int32), np.ascontiguousarray(ja, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    Mp = ptr(np.ascontiguousarray(M, np.float64)) if M is not None else None
    lib = reference(n).lib
    lib.ref_cg_csr.restype = ctypes.c_int
    k = lib.ref_cg_csr(len(b), ptr(irp), ptr(ja), ptr(vals), ptr(b), ctypes.c_double(tol), maxit, Mp, ptr(x),
                       ptr(res), len(res), threads, blocks)
    return k, x, res[: k + 1]


def ref_div_sqrt(n, x, y):
    """The reference's host ::mp_div(x, y), ::mp_sqrt(|x|) and ::mp_dsqrt(|x|) (MPFR)."""
    lib = reference(n).lib
    cnt = len(x)
    q, r, d = np.zeros(cnt, mp_dtype(n)), np.zeros(cnt, mp_dtype(n)), np.zeros(cnt)
    ax = x.copy()
    ax["sign"] = 0
    lib.ref_div(ptr(x), ptr(y), ptr(q), ctypes.c_long(cnt))
    lib.ref_sqrt(ptr(ax), ptr(r), ctypes.c_long(cnt))
    lib.ref_dsqrt(ptr(ax), ptr(d), ctypes.c_long(cnt))
    return q, r, d


def ref_mtx(n, path):
    """The reference's Matrix Market reader (collect_mtx_stats, build_csr,
    build_ell) on a file: stats, (irp, ja, as), (ell ja, ell as)."""
    lib = reference(n).lib
    st = np.zeros(6, np.int32)
    b = str(path).encode()
    lib.ref_mtx_stats(b, ptr(st))
    m, cols, lines, maxnzr, nzmd, sym = (int(v) for v in st)
    nnz = 2 * (lines - nzmd) + nzmd if sym else lines
    irp, ja, vals = np.zeros(m + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz, np.float64)
    lib.ref_mtx_csr(b, m, nnz, lines, sym, ptr(vals), ptr(ja), ptr(irp))
    eja, eas = np.zeros(m * maxnzr, np.int32), np.zeros(m * maxnzr, np.float64)
    lib.ref_mtx_ell(b, m, maxnzr, lines, sym, ptr(eas), ptr(eja))
    return dict(m=m, n=cols, lines=lines, maxnzr=maxnzr, nzmd=nzmd, symmetric=sym), (irp, ja, vals), (eja, eas)


_refs = {}


def ref_available(n=8):
    return (REF_DIR / ("libmpres_ref_%d.so" % n)).exists()


class Reference(_Common):
    """The reference library compiled for the CPU (one moduli set per library)."""

    def __init__(self, n):
        lib = ctypes.CDLL(str(REF_DIR / ("libmpres_ref_%d.so" % n)))
        super().__init__(lib, "ref_")
        assert lib.ref_moduli_size() == n
        self.n = n
        lib.ref_init()

    def set_d(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(x.size, mp_dtype(self.n))
        self.lib.ref_set_d(ptr(x), ctypes.c_long(x.size), ptr(out))
        return out

    def tables(self, log2m):
        return _tables(self.lib.ref_tables, self.n, log2m)

    def _elem(self, name, x, y):
        r = np.zeros(len(x), mp_dtype(self.n))
        getattr(self.lib, name)(ptr(x), ptr(y), ptr(r), ctypes.c_long(len(x)))
        return r

    def add(self, x, y):
        return self._elem("ref_dev_add", x, y)

    def mul(self, x, y):
        return self._elem("ref_dev_mul", x, y)

    def mul_d(self, x, d):
        return self._elem("ref_dev_mul_d", x, np.ascontiguousarray(d, dtype=np.float64))

    def eval_fast(self, digits):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        cnt = digits.size // self.n
        lo, up = np.zeros(cnt, ER), np.zeros(cnt, ER)
        self.lib.ref_dev_eval_fast(ptr(digits), ptr(lo), ptr(up), ctypes.c_long(cnt))
        return lo, up

    def eval(self, digits):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        cnt = digits.size // self.n
        lo, up = np.zeros(cnt, ER), np.zeros(cnt, ER)
        self.lib.ref_dev_eval(ptr(digits), ptr(lo), ptr(up), ctypes.c_long(cnt))
        return lo, up

    def scale2pow(self, digits, D):
        digits = np.ascontiguousarray(digits, dtype=np.int32)
        D = np.ascontiguousarray(D, dtype=np.uint32)
        out = np.zeros_like(digits)
        self.lib.ref_dev_scale2pow(ptr(digits), ptr(D), ptr(out), ctypes.c_long(D.size))
        return out

    def dot(self, x, y, g1=512, b1=128, g2=8192, g3=256, b3=64, incx=1, incy=1, length=None):
        length = len(x) if length is None else length
        r = np.zeros(1, mp_dtype(self.n))
        self.lib.ref_dot(length, ptr(x), incx, ptr(y), incy, ptr(r), g1, b1, g2, g3, b3)
        return r

    def gemv(self, trans, m, cols, alpha, A, lda, x, beta, y, incx=1, incy=1, g1=256, b1=128, g2=256, b3=32):
        y = y.copy()
        self.lib.ref_gemv(trans, m, cols, ptr(alpha), ptr(A), lda, ptr(x), incx, ptr(beta), ptr(y), incy,
                          g1, b1, g2, b3)
        return y

    def gemm(self, m, cols, k, alpha, A, lda, B, ldb, beta, C, ldc, b1x=32, b1y=1, g2x=128, g2y=64, b3=16):
        C = C.copy()
        self.lib.ref_gemm(m, cols, k, ptr(alpha), ptr(A), lda, ptr(B), ldb, ptr(beta), ptr(C), ldc,
                          b1x, b1y, g2x, g2y, b3)
        return C

    def spmv_csr(self, m, irp, ja, vals, x):
        y = np.zeros(m, mp_dtype(self.n))
        self.lib.ref_spmv_csr(m, ptr(irp), ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y

    def spmv_csrv(self, m, tpr, irp, ja, vals, x):
        y = np.zeros(m, mp_dtype(self.n))
        self.lib.ref_spmv_csrv(m, tpr, ptr(irp), ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y

    def spmv_ell(self, m, maxnzr, ja, vals, x):
        y = np.zeros(m, mp_dtype(self.n))
        self.lib.ref_spmv_ell(m, maxnzr, ptr(ja), ptr(vals), ptr(x), ptr(y))
        return y


def reference(n):
    if n not in _refs:
        _refs[n] = Reference(n)
    return _refs[n]


def same_bits(a, b):
    """Bitwise equality of two mp_float_t arrays (digits, sign, exp and eval)."""
    return a.tobytes() == b.tobytes()


def mismatches(a, b):
    """Indices where two mp_float_t arrays differ in any byte."""
    av = a.view(np.uint8).reshape(len(a), -1)
    bv = b.view(np.uint8).reshape(len(b), -1)
    return np.nonzero((av != bv).any(axis=1))[0]
