"""Python access to libmpres_gb300.so through its C ABI (include/mpres_gb300.h).

This is plumbing for tests and benchmarks: it loads the in-tree CUDA library,
raises on any error status, and moves numpy arrays in the reference's
mp_float_t layout to and from device memory.  There is no CPU fallback: if the
library or a GPU is missing, the calls fail loudly.
"""
import ctypes
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmpres_gb300.so"

P = ctypes.c_void_p
I = ctypes.c_int
SZ = ctypes.c_size_t

NO_TRANS, TRANS = 111, 112
ER = np.dtype([("frac", "<f8"), ("exp", "<i8")])


def mp_dtype(n):
    """mp_float_t for n moduli (src/types.cuh:69-74), 4n + 40 bytes."""
    return np.dtype([("digits", "<i4", (n,)), ("sign", "<i4"), ("exp", "<i4"), ("eval", ER, (2,))])


class MpArrayT(ctypes.Structure):
    _fields_ = [("digits", P), ("sign", P), ("exp", P), ("eval", P), ("buf", P), ("len", P)]


class CsrT(ctypes.Structure):
    _fields_ = [("as_", P), ("ja", P), ("irp", P)]


class EllT(ctypes.Structure):
    _fields_ = [("as_", P), ("ja", P)]


class MpresError(RuntimeError):
    pass


_SIGS = {
    "mpres_last_error": (ctypes.c_char_p, []),
    "mpres_mp_float_size": (SZ, [I]),
    "mpres_init": (I, [I]),
    "mpres_get_int_constants": (I, [I, P]),
    "mpres_array_init": (I, [I, P, SZ]),
    "mpres_array_clear": (I, [P]),
    "mpres_array_host2device": (I, [I, P, P, SZ]),
    "mpres_array_device2host": (I, [I, P, P, SZ]),
    "mpres_csr_init": (I, [P, I, I]),
    "mpres_csr_host2device": (I, [P, P, I, I]),
    "mpres_csr_clear": (I, [P]),
    "mpres_ell_init": (I, [P, I, I]),
    "mpres_ell_host2device": (I, [P, P, I, I]),
    "mpres_ell_clear": (I, [P]),
    "mpres_set_d": (I, [I, P, SZ, P]),
    "mpres_v2_diff": (I, [I, I, P, P, P, I, P]),
    "mpres_v2_axpy": (I, [I, I, P, P, P, P, I, P]),
    "mpres_v2_maxpy": (I, [I, I, P, P, P, P, I, P]),
    "mpres_v2_dot": (I, [I, I, P, P, P, I, I, P]),
    "mpres_v2_norm2": (I, [I, I, P, P, I, I, P]),
    "mpres_cg_csr": (I, [I, I, P, P, ctypes.c_double, I, P, P, I, P, I, I, P]),
    "mpres_pcg_csr": (I, [I, I, P, P, ctypes.c_double, I, I, P, P, P, I, P, I, I, P]),
    "mpres_div": (I, [I, P, P, P]),
    "mpres_sqrt": (I, [I, P, P]),
    "mpres_dsqrt": (I, [I, P, P]),
    "mpres_div_device": (I, [I, P, P, P]),
    "mpres_dsqrt_device": (I, [I, P, P]),
    "mpres_mtx_stats": (I, [ctypes.c_char_p, P, P, P, P, P, P, P]),
    "mpres_mtx_build_csr": (I, [ctypes.c_char_p, I, I, I, I, P, P, P]),
    "mpres_mtx_build_ell": (I, [ctypes.c_char_p, I, I, I, I, P, P]),
    "mpres_set_d_device": (I, [I, P, SZ, P, P]),
    "mpres_array_set_d": (I, [I, P, SZ, P, SZ, P]),
    "mpres_dot": (I, [I, I, P, I, P, I, P, P, I, I, I, I, I, P]),
    "mpres_dot_noalloc": (I, [I, I, P, I, P, I, P, I, I, P]),
    "mpres_gemv": (I, [I, I, I, I, P, P, I, P, I, P, P, I, P, P, I, I, I, I, P]),
    "mpres_gemm": (I, [I, I, I, I, I, I, P, P, I, P, I, P, P, I, P, I, I, I, I, I, P]),
    "mpres_spmv_csr": (I, [I, I, P, P, P, I, P]),
    "mpres_spmv_csrv": (I, [I, I, P, P, P, I, I, P]),
    "mpres_spmv_ell": (I, [I, I, I, P, P, P, I, P]),
    "mpres_batch_create": (I, [I, P]),
    "mpres_batch_destroy": (I, [P]),
    "mpres_batch_add_gemv": (I, [P, I, I, I, P, P, I, P, I, P, P, I, I]),
    "mpres_batch_add_dot": (I, [P, I, P, I, P, I, P, I, I]),
    "mpres_batch_add_spmv_csr": (I, [P, I, P, P, P]),
    "mpres_batch_add_spmv_csrv": (I, [P, I, P, P, P, I]),
    "mpres_batch_add_spmv_ell": (I, [P, I, I, P, P, P]),
    "mpres_batch_add_gemm": (I, [P, I, I, I, I, I, P, P, I, P, I, P, P, I]),
    "mpres_batch_commit": (I, [P, ctypes.c_uint, P]),
    "mpres_batch_run": (I, [P, P]),
    "mpres_batch_info": (I, [P, P]),
    "mpres_server_create": (I, [I, SZ, I, I, P]),
    "mpres_server_destroy": (I, [P]),
    "mpres_server_submit_gemv": (I, [P, I, I, I, P, P, I, P, I, P, P, I, I, P]),
    "mpres_server_submit_dot": (I, [P, I, P, I, P, I, P, I, I, P]),
    "mpres_server_submit_spmv_csr": (I, [P, I, I, ctypes.c_longlong, P, P, P, P]),
    "mpres_server_wait": (I, [P, ctypes.c_longlong, ctypes.c_double]),
    "mpres_server_drain": (I, [P]),
    "mpres_server_cancel": (I, [P, ctypes.c_longlong]),
    "mpres_server_times": (I, [P, ctypes.c_longlong, ctypes.c_longlong, P]),
    "mpres_server_stats": (I, [P, P]),
    "mpres_probe_mulmod": (I, [I, I, ctypes.c_longlong, P, P]),
    "mpres_probe_dadd": (I, [I, I, ctypes.c_longlong, P, P]),
    "mpres_probe_latency": (I, [I, ctypes.c_longlong, P, P]),
    "mpres_elementwise": (I, [I, I, P, P, P, SZ, P]),
    "mpres_probe_ceil_log2": (I, [P, P, SZ, P]),
    "mpres_probe_check": (I, [I, I, P, P, P, SZ, P]),
    "mpres_probe_chain": (I, [I, I, P, P, I, P, P, P, P]),
    "mpres_probe_rounding": (I, [I, P, P, I, P, P, P]),
    "mpres_probe_eval_phases": (I, [I, P, I, P, P, P]),
    "mpres_probe_gemm_phases": (I, [I, I, I, I, P, P, I, P, I, P, P, I, P, P]),
    "mpres_probe_fraction_sum": (I, [I, I, P, ctypes.c_longlong, P, P, P]),
    "mpres_rns_scale2pow": (I, [I, P, P, P, SZ, P]),
    "mpres_rns_eval": (I, [I, I, P, P, P, SZ, P]),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise MpresError("libmpres_gb300.so not built: run __graft_entry__.build() or mpres-blas_gb300/build.py")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, what=""):
    if rc != 0:
        msg = lib().mpres_last_error().decode()
        raise MpresError("%s failed (status %d): %s" % (what, rc, msg))


def init(nmod):
    check(lib().mpres_init(nmod), "mpres_init")


def int_constants(nmod):
    out = (ctypes.c_int * 5)()
    check(lib().mpres_get_int_constants(nmod, out), "mpres_get_int_constants")
    return dict(mp_precision=out[0], mp_h=out[1], mp_j=out[2], ref_factor=out[3], log2m=out[4])


def set_d(nmod, x):
    """Host conversion of doubles (the reference's mp_set_d)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(x.size, mp_dtype(nmod))
    check(lib().mpres_set_d(nmod, x.ctypes.data, x.size, out.ctypes.data), "mpres_set_d")
    return out


def set_d_device(nmod, x, out=None, stream=None):
    """Device conversion (bit-identical to set_d) of a float64 torch CUDA tensor
    into AoS records; returns the DeviceBytes it wrote."""
    n = x.numel()
    out = out if out is not None else DeviceBytes(n * mp_size(nmod))
    check(lib().mpres_set_d_device(nmod, x.data_ptr(), n, out.ptr, _stream_handle(stream)), "mpres_set_d_device")
    return out


def array_set_d(nmod, arr, offset, x, stream=None):
    """Device conversion of a float64 torch CUDA tensor into elements
    [offset, offset + x.numel()) of a DeviceArray."""
    if offset < 0 or offset + x.numel() > arr.size:
        raise MpresError("array_set_d: elements [%d, %d) outside an array of %d" % (offset, offset + x.numel(), arr.size))
    check(lib().mpres_array_set_d(nmod, arr.ref, offset, x.data_ptr(), x.numel(), _stream_handle(stream)),
          "mpres_array_set_d")


def mp_size(nmod):
    return 4 * nmod + 40


def v2_vec(nmod, op, n, x, y, r, alpha=None, threads=32, stream=None):
    """op "diff": r = x - y; "axpy": r = alpha x + y; "maxpy": r = -alpha x + y (DeviceBytes records)."""
    h = _stream_handle(stream)
    if op == "diff":
        check(lib().mpres_v2_diff(nmod, n, x.ptr, y.ptr, r.ptr, threads, h), "mpres_v2_diff")
    else:
        f = lib().mpres_v2_axpy if op == "axpy" else lib().mpres_v2_maxpy
        check(f(nmod, n, alpha.ptr, x.ptr, y.ptr, r.ptr, threads, h), "mpres_v2_" + op)


def v2_dot(nmod, n, x, y, r, blocks=256, threads=32, stream=None):
    check(lib().mpres_v2_dot(nmod, n, x.ptr, y.ptr, r.ptr, blocks, threads, _stream_handle(stream)), "mpres_v2_dot")


def v2_norm2(nmod, n, x, blocks=256, threads=32, stream=None):
    out = ctypes.c_double()
    check(lib().mpres_v2_norm2(nmod, n, x.ptr, ctypes.byref(out), blocks, threads, _stream_handle(stream)),
          "mpres_v2_norm2")
    return out.value


def cg_csr(nmod, n, csr, b, x, tol, maxit, M=None, threads=None, blocks=256, stream=None):
    """mp_cg_csr (M None) / mp_pcg_csr (M: DeviceBytes of n doubles, the inverse
    diagonal): x (DeviceBytes records) is the guess and the solution; returns
    (iterations, resvec)."""
    res = np.zeros(maxit + 2)
    k = ctypes.c_int()
    h = _stream_handle(stream)
    if M is None:
        check(lib().mpres_cg_csr(nmod, n, ctypes.byref(csr.c), b.ptr, tol, maxit, x.ptr, res.ctypes.data, len(res),
                                 ctypes.byref(k), threads or 32, blocks, h), "mpres_cg_csr")
    else:
        check(lib().mpres_pcg_csr(nmod, n, ctypes.byref(csr.c), b.ptr, tol, maxit, 1, M.ptr, x.ptr,
                                  res.ctypes.data, len(res), ctypes.byref(k), threads or 64, blocks, h),
              "mpres_pcg_csr")
    return k.value, res[: k.value + 1]


def div(nmod, x, y):
    """Host ::mp_div record by record (MPFR semantics at MP_PRECISION bits)."""
    out = np.zeros(len(x), mp_dtype(nmod))
    for i in range(len(x)):
        check(lib().mpres_div(nmod, x[i:i + 1].ctypes.data, y[i:i + 1].ctypes.data, out[i:i + 1].ctypes.data),
              "mpres_div")
    return out


def sqrt(nmod, x):
    out = np.zeros(len(x), mp_dtype(nmod))
    for i in range(len(x)):
        check(lib().mpres_sqrt(nmod, x[i:i + 1].ctypes.data, out[i:i + 1].ctypes.data), "mpres_sqrt")
    return out


def dsqrt(nmod, x):
    out = np.zeros(len(x))
    for i in range(len(x)):
        check(lib().mpres_dsqrt(nmod, x[i:i + 1].ctypes.data, out[i:i + 1].ctypes.data), "mpres_dsqrt")
    return out


def mtx_stats(path):
    """collect_mtx_stats of a Matrix Market file."""
    v = [ctypes.c_int() for _ in range(6)]
    dt = ctypes.create_string_buffer(16)
    check(lib().mpres_mtx_stats(str(path).encode(), *[ctypes.byref(x) for x in v], dt), "mpres_mtx_stats")
    m, n, lines, maxnzr, nzmd, sym = (x.value for x in v)
    nnz = 2 * (lines - nzmd) + nzmd if sym else lines
    return dict(m=m, n=n, lines=lines, maxnzr=maxnzr, nzmd=nzmd, symmetric=sym, nnz=nnz, datatype=dt.value.decode())


def mtx_csr(path, st=None):
    """build_csr: (irp, ja, as) host arrays in the reference's entry order."""
    st = st or mtx_stats(path)
    irp, ja, vals = np.zeros(st["m"] + 1, np.int32), np.zeros(st["nnz"], np.int32), np.zeros(st["nnz"])
    check(lib().mpres_mtx_build_csr(str(path).encode(), st["m"], st["nnz"], st["lines"], st["symmetric"],
                                    vals.ctypes.data, ja.ctypes.data, irp.ctypes.data), "mpres_mtx_build_csr")
    return irp, ja, vals


def mtx_ell(path, st=None):
    """build_ell: (ja, as) column-major m x maxnzr host arrays."""
    st = st or mtx_stats(path)
    size = st["m"] * st["maxnzr"]
    ja, vals = np.zeros(size, np.int32), np.zeros(size)
    check(lib().mpres_mtx_build_ell(str(path).encode(), st["m"], st["maxnzr"], st["lines"], st["symmetric"],
                                    vals.ctypes.data, ja.ctypes.data), "mpres_mtx_build_ell")
    return ja, vals


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", stream)


class DeviceArray:
    """An mp_array_t (SoA) in device memory, allocated by mpres_array_init."""

    def __init__(self, nmod, size):
        self.nmod, self.size = nmod, size
        self.a = MpArrayT()
        check(lib().mpres_array_init(nmod, ctypes.byref(self.a), size), "mpres_array_init")
        self._live = True

    @classmethod
    def from_host(cls, nmod, host):
        d = cls(nmod, len(host))
        d.upload(host)
        return d

    def upload(self, host):
        host = np.ascontiguousarray(host)
        assert host.dtype.itemsize == 4 * self.nmod + 40 and len(host) == self.size
        check(lib().mpres_array_host2device(self.nmod, ctypes.byref(self.a), host.ctypes.data, self.size),
              "mpres_array_host2device")

    def download(self, out=None):
        """The records as a host array; `out` (e.g. a pinned buffer of this
        size and record type) is filled and returned instead of a new array."""
        if out is None:
            out = np.zeros(self.size, mp_dtype(self.nmod))
        assert out.dtype.itemsize == 4 * self.nmod + 40 and len(out) == self.size and out.flags.c_contiguous
        check(lib().mpres_array_device2host(self.nmod, out.ctypes.data, ctypes.byref(self.a), self.size),
              "mpres_array_device2host")
        return out

    @property
    def ref(self):
        return ctypes.byref(self.a)

    def free(self):
        if self._live:
            check(lib().mpres_array_clear(ctypes.byref(self.a)), "mpres_array_clear")
            self._live = False

    def __del__(self):
        try:
            if self._live and _lib is not None:
                _lib.mpres_array_clear(ctypes.byref(self.a))
                self._live = False
        except Exception:
            pass


class TensorArray:
    """An mp_array_t whose SoA fields are torch CUDA tensors (digits int32
    [size*nmod], sign and exp int32 [size], eval int64 [2*size, 2] holding the
    er_float_t {frac, exp} pairs of the lower then the upper bounds).  view()
    gives mp_array_t views of contiguous element ranges: their fields point
    into this array and share its len, so a view's upper bounds are found where
    the kernels look for them (eval + len)."""

    def __init__(self, nmod, size, device="cuda"):
        import torch
        self.nmod, self.size = nmod, int(size)
        self.digits = torch.empty(self.size * nmod, dtype=torch.int32, device=device)
        self.sign = torch.empty(self.size, dtype=torch.int32, device=device)
        self.exp = torch.empty(self.size, dtype=torch.int32, device=device)
        self.eval = torch.empty((2 * self.size, 2), dtype=torch.int64, device=device)
        self.len = torch.tensor([self.size], dtype=torch.int32, device=device)
        self.a = self._struct(0)

    def _struct(self, off):
        return MpArrayT(self.digits.data_ptr() + 4 * self.nmod * off, self.sign.data_ptr() + 4 * off,
                        self.exp.data_ptr() + 4 * off, self.eval.data_ptr() + 16 * off, None, self.len.data_ptr())

    @property
    def ref(self):
        return ctypes.byref(self.a)

    def view(self, offset, length):
        if offset < 0 or offset + length > self.size:
            raise MpresError("TensorArray.view: [%d, %d) outside %d elements" % (offset, offset + length, self.size))
        return _ArrayView(self, self._struct(offset), length)

    def gather_from(self, src, index, offset=0):
        """Elements [offset, offset + len(index)) = src[index] (src a TensorArray)."""
        k = index.numel()
        n = self.nmod
        self.digits.view(-1, n)[offset:offset + k] = src.digits.view(-1, n).index_select(0, index)
        self.sign[offset:offset + k] = src.sign.index_select(0, index)
        self.exp[offset:offset + k] = src.exp.index_select(0, index)
        self.eval[offset:offset + k] = src.eval[: src.size].index_select(0, index)
        self.eval[self.size + offset:self.size + offset + k] = src.eval[src.size:].index_select(0, index)

    def set_d(self, x, offset=0, stream=None):
        """Device conversion of a float64 CUDA tensor into elements [offset, offset + x.numel())."""
        array_set_d(self.nmod, self, offset, x, stream)

    def upload(self, host):
        """Elements from a host mp_float_t array (the inverse of download)."""
        import torch
        host = np.ascontiguousarray(host)
        assert host.dtype.itemsize == 4 * self.nmod + 40 and len(host) == self.size
        dev = self.digits.device
        self.digits.copy_(torch.from_numpy(np.ascontiguousarray(host["digits"]).reshape(-1)).to(dev))
        self.sign.copy_(torch.from_numpy(np.ascontiguousarray(host["sign"])).to(dev))
        self.exp.copy_(torch.from_numpy(np.ascontiguousarray(host["exp"])).to(dev))
        ev = np.empty((2 * self.size, 2), np.int64)
        for h in (0, 1):
            ev[h * self.size:(h + 1) * self.size, 0] = np.ascontiguousarray(host["eval"][:, h]["frac"]).view(np.int64)
            ev[h * self.size:(h + 1) * self.size, 1] = host["eval"][:, h]["exp"]
        self.eval.copy_(torch.from_numpy(ev).to(dev))

    def copy_(self, src):
        """Every element from another TensorArray of the same size (device copies
        on the current stream)."""
        assert src.nmod == self.nmod and src.size == self.size
        for a, b in ((self.digits, src.digits), (self.sign, src.sign), (self.exp, src.exp), (self.eval, src.eval)):
            a.copy_(b)

    def download(self):
        out = np.zeros(self.size, mp_dtype(self.nmod))
        out["digits"] = self.digits.view(-1, self.nmod).cpu().numpy()
        out["sign"] = self.sign.cpu().numpy()
        out["exp"] = self.exp.cpu().numpy()
        ev = self.eval.cpu().numpy()
        for h in (0, 1):
            half = ev[h * self.size:(h + 1) * self.size]
            out["eval"][:, h]["frac"] = half[:, 0].view(np.float64)
            out["eval"][:, h]["exp"] = half[:, 1]
        return out


class _ArrayView:
    def __init__(self, owner, struct, size):
        self.owner, self.a, self.size, self.nmod = owner, struct, size, owner.nmod

    @property
    def ref(self):
        return ctypes.byref(self.a)


class DeviceBytes:
    """Raw device memory for AoS mp_float_t vectors (the SpMV operands), held as a
    torch uint8 tensor so that torch's allocator owns it."""

    def __init__(self, nbytes, device="cuda"):
        import torch
        self.t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)
        self.nbytes = int(nbytes)

    @property
    def ptr(self):
        return self.t.data_ptr()

    @classmethod
    def from_numpy(cls, arr):
        import torch
        arr = np.ascontiguousarray(arr)
        d = cls(arr.nbytes)
        if arr.nbytes:
            d.t[: arr.nbytes].copy_(torch.from_numpy(arr.view(np.uint8).reshape(-1)))
        return d

    def to_numpy(self, dtype, count):
        raw = self.t[: np.dtype(dtype).itemsize * count].cpu().numpy()
        return raw.view(dtype).copy()


class DeviceCsr:
    def __init__(self, m, irp, ja, vals):
        irp = np.ascontiguousarray(irp, dtype=np.int32)
        ja = np.ascontiguousarray(ja, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.m, self.nnz = m, len(ja)
        self.c = CsrT()
        check(lib().mpres_csr_init(ctypes.byref(self.c), m, self.nnz), "mpres_csr_init")
        host = CsrT(vals.ctypes.data, ja.ctypes.data, irp.ctypes.data)
        check(lib().mpres_csr_host2device(ctypes.byref(self.c), ctypes.byref(host), m, self.nnz),
              "mpres_csr_host2device")
        self._live = True

    def upload(self, irp, ja, vals):
        """Copies host arrays of the same shape into this matrix (csr_host2device);
        contiguous int32 / int32 / float64 arrays, e.g. in pinned memory, are used in place."""
        irp = np.ascontiguousarray(irp, dtype=np.int32)
        ja = np.ascontiguousarray(ja, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        assert len(irp) == self.m + 1 and len(ja) == self.nnz and len(vals) == self.nnz
        host = CsrT(vals.ctypes.data, ja.ctypes.data, irp.ctypes.data)
        check(lib().mpres_csr_host2device(ctypes.byref(self.c), ctypes.byref(host), self.m, self.nnz),
              "mpres_csr_host2device")

    def free(self):
        if self._live:
            check(lib().mpres_csr_clear(ctypes.byref(self.c)), "mpres_csr_clear")
            self._live = False


class DeviceEll:
    def __init__(self, m, maxnzr, ja, vals):
        ja = np.ascontiguousarray(ja, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.m, self.maxnzr = m, maxnzr
        self.e = EllT()
        check(lib().mpres_ell_init(ctypes.byref(self.e), m, maxnzr), "mpres_ell_init")
        host = EllT(vals.ctypes.data, ja.ctypes.data)
        check(lib().mpres_ell_host2device(ctypes.byref(self.e), ctypes.byref(host), m, maxnzr),
              "mpres_ell_host2device")
        self._live = True

    @classmethod
    def from_tensors(cls, m, maxnzr, ja, vals):
        """An ell_t over CUDA tensors (int32 ja, float64 vals, maxnzr * m slots
        each, column-major) that torch owns; free() only drops the references."""
        assert ja.numel() == vals.numel() == m * maxnzr
        self = cls.__new__(cls)
        self.m, self.maxnzr = m, maxnzr
        self._tensors = (ja, vals)
        self.e = EllT(vals.data_ptr(), ja.data_ptr())
        self._live = False
        return self

    def free(self):
        if self._live:
            check(lib().mpres_ell_clear(ctypes.byref(self.e)), "mpres_ell_clear")
            self._live = False
        self._tensors = None


def dot(nmod, n, x, y, r, incx=1, incy=1, order=(512, 128, 8192, 256, 64), buffer=None, stream=None):
    """cuda::mp_dot<g1,b1,g2,g3,b3>(n, x, incx, y, incy, r, buffer); order = the template arguments."""
    g1, b1, g2, g3, b3 = order
    check(lib().mpres_dot(nmod, n, x.ref, incx, y.ref, incy, r.ref, buffer.ref if buffer else None,
                          g1, b1, g2, g3, b3, _stream_handle(stream)), "mpres_dot")


def gemv(nmod, trans, m, n, alpha, A, lda, x, beta, y, incx=1, incy=1, order=(256, 128, 256, 32), stream=None):
    """cuda::mp_gemv<g1,b1,g2,b3>(trans, m, n, alpha, A, lda, x, incx, beta, y, incy, buf1, buf2)."""
    g1, b1, g2, b3 = order
    check(lib().mpres_gemv(nmod, trans, m, n, alpha.ref, A.ref, lda, x.ref, incx, beta.ref, y.ref, incy, None, None,
                           g1, b1, g2, b3, _stream_handle(stream)), "mpres_gemv")


def gemm(nmod, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, transa=NO_TRANS, transb=NO_TRANS,
         order=(32, 1, 128, 64, 16), stream=None):
    """cuda::mp_gemm<b1x,b1y,g2x,g2y,b3>(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, buffer)."""
    b1x, b1y, g2x, g2y, b3 = order
    check(lib().mpres_gemm(nmod, transa, transb, m, n, k, alpha.ref, A.ref, lda, B.ref, ldb, beta.ref, C.ref, ldc,
                           None, b1x, b1y, g2x, g2y, b3, _stream_handle(stream)), "mpres_gemm")


GEMM_PHASES = ("prescale_a", "prescale_b", "limbs", "scalar_chain", "residue_product", "epilogue", "redo")


def probe_gemm_phases(nmod, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream=None):
    """mp_gemm's split form (32 moduli) with each of its phases timed by events
    (mpres_probe_gemm_phases): {phase: milliseconds}, GEMM_PHASES order."""
    ms = (ctypes.c_float * len(GEMM_PHASES))()
    check(lib().mpres_probe_gemm_phases(nmod, m, n, k, alpha.ref, A.ref, lda, B.ref, ldb, beta.ref, C.ref, ldc, ms,
                                        _stream_handle(stream)), "mpres_probe_gemm_phases")
    return dict(zip(GEMM_PHASES, list(ms)))


def spmv_csr(nmod, m, csr, x, y, threads=32, stream=None):
    check(lib().mpres_spmv_csr(nmod, m, ctypes.byref(csr.c), x.ptr, y.ptr, threads, _stream_handle(stream)),
          "mpres_spmv_csr")


def spmv_csrv(nmod, m, csr, x, y, tpr, threads=32, stream=None):
    check(lib().mpres_spmv_csrv(nmod, m, ctypes.byref(csr.c), x.ptr, y.ptr, threads, tpr, _stream_handle(stream)),
          "mpres_spmv_csrv")


def spmv_ell(nmod, m, ell, x, y, threads=32, stream=None):
    check(lib().mpres_spmv_ell(nmod, m, ell.maxnzr, ctypes.byref(ell.e), x.ptr, y.ptr, threads,
                               _stream_handle(stream)), "mpres_spmv_ell")


BATCH_GRAPH, BATCH_AUTOTUNE = 1, 2


class Batch:
    """A batch of mp_gemv / mp_dot / mp_spmv_csr operations run as one persistent
    launch (include/mpres_gb300_batch.h).  Operands must outlive the batch."""

    def __init__(self, nmod):
        self.nmod = nmod
        self.h = ctypes.c_void_p()
        check(lib().mpres_batch_create(nmod, ctypes.byref(self.h)), "mpres_batch_create")
        self._keep = []

    def add_gemv(self, trans, m, n, alpha, A, lda, x, beta, y, incx=1, incy=1, b3=32):
        self._keep += [alpha, A, x, beta, y]
        check(lib().mpres_batch_add_gemv(self.h, trans, m, n, alpha.ref, A.ref, lda, x.ref, incx, beta.ref, y.ref,
                                         incy, b3), "mpres_batch_add_gemv")

    def add_dot(self, n, x, y, r, incx=1, incy=1, g3=256, b3=64):
        self._keep += [x, y, r]
        check(lib().mpres_batch_add_dot(self.h, n, x.ref, incx, y.ref, incy, r.ref, g3, b3), "mpres_batch_add_dot")

    def add_spmv_csr(self, m, csr, x, y):
        self._keep += [csr, x, y]
        check(lib().mpres_batch_add_spmv_csr(self.h, m, ctypes.byref(csr.c), x.ptr, y.ptr),
              "mpres_batch_add_spmv_csr")

    def add_gemm(self, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, transa=NO_TRANS, transb=NO_TRANS):
        self._keep += [alpha, A, B, beta, C]
        check(lib().mpres_batch_add_gemm(self.h, transa, transb, m, n, k, alpha.ref, A.ref, lda, B.ref, ldb, beta.ref,
                                         C.ref, ldc), "mpres_batch_add_gemm")

    def add_spmv_csrv(self, m, csr, x, y, tpr):
        self._keep += [csr, x, y]
        check(lib().mpres_batch_add_spmv_csrv(self.h, m, ctypes.byref(csr.c), x.ptr, y.ptr, tpr),
              "mpres_batch_add_spmv_csrv")

    def add_spmv_ell(self, m, ell, x, y):
        self._keep += [ell, x, y]
        check(lib().mpres_batch_add_spmv_ell(self.h, m, ell.maxnzr, ctypes.byref(ell.e), x.ptr, y.ptr),
              "mpres_batch_add_spmv_ell")

    def commit(self, flags=BATCH_GRAPH, stream=None):
        check(lib().mpres_batch_commit(self.h, flags, _stream_handle(stream)), "mpres_batch_commit")

    def run(self, stream=None):
        check(lib().mpres_batch_run(self.h, _stream_handle(stream)), "mpres_batch_run")

    def info(self):
        out = (ctypes.c_longlong * 8)()
        check(lib().mpres_batch_info(self.h, out), "mpres_batch_info")
        keys = ("ops", "tasks", "threads", "ctas", "graph", "autotuned", "scratch_bytes", "candidates")
        return dict(zip(keys, list(out)))

    def destroy(self):
        if self.h:
            check(lib().mpres_batch_destroy(self.h), "mpres_batch_destroy")
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """The serving loop (include/mpres_gb300_server.h): requests over
    device-resident operands, admitted under an HBM budget and run as
    continuous batches.  Operands must stay alive until their request is done."""

    def __init__(self, nmod, budget_bytes, slots=4, max_batch_ops=64):
        self.nmod = nmod
        self.h = ctypes.c_void_p()
        check(lib().mpres_server_create(nmod, int(budget_bytes), slots, max_batch_ops, ctypes.byref(self.h)),
              "mpres_server_create")
        self._keep = {}

    def submit_gemv(self, trans, m, n, alpha, A, lda, x, beta, y, incx=1, incy=1, b3=32):
        i = ctypes.c_longlong()
        check(lib().mpres_server_submit_gemv(self.h, trans, m, n, alpha.ref, A.ref, lda, x.ref, incx, beta.ref,
                                             y.ref, incy, b3, ctypes.byref(i)), "mpres_server_submit_gemv")
        self._keep[i.value] = (alpha, A, x, beta, y)
        return i.value

    def submit_dot(self, n, x, y, r, incx=1, incy=1, g3=256, b3=64):
        i = ctypes.c_longlong()
        check(lib().mpres_server_submit_dot(self.h, n, x.ref, incx, y.ref, incy, r.ref, g3, b3, ctypes.byref(i)),
              "mpres_server_submit_dot")
        self._keep[i.value] = (x, y, r)
        return i.value

    def submit_spmv_csr(self, m, ncols, csr, x, y):
        i = ctypes.c_longlong()
        check(lib().mpres_server_submit_spmv_csr(self.h, m, ncols, csr.nnz, ctypes.byref(csr.c), x.ptr, y.ptr,
                                                 ctypes.byref(i)), "mpres_server_submit_spmv_csr")
        self._keep[i.value] = (csr, x, y)
        return i.value

    def wait(self, rid, timeout=-1.0):
        check(lib().mpres_server_wait(self.h, rid, timeout), "mpres_server_wait")

    def drain(self):
        check(lib().mpres_server_drain(self.h), "mpres_server_drain")

    def cancel(self, rid):
        """True if the request was withdrawn before it ran, False if it had started."""
        rc = lib().mpres_server_cancel(self.h, rid)
        if rc == 4:
            return False
        check(rc, "mpres_server_cancel")
        return True

    def times(self, first, count):
        out = np.zeros(3 * count)
        check(lib().mpres_server_times(self.h, first, count, out.ctypes.data), "mpres_server_times")
        return out.reshape(count, 3)

    def stats(self):
        out = np.zeros(8)
        check(lib().mpres_server_stats(self.h, out.ctypes.data), "mpres_server_stats")
        keys = ("done", "batches", "mean_batch", "p50_s", "p99_s", "peak_bytes", "max_in_flight", "errors")
        return dict(zip(keys, out.tolist()))

    def destroy(self):
        if self.h:
            h, self.h = self.h, ctypes.c_void_p()
            check(lib().mpres_server_destroy(h), "mpres_server_destroy")
            self._keep.clear()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


OP_ADD, OP_MUL, OP_MUL_D = 0, 1, 2


def elementwise(nmod, op, x, y):
    """Element-wise device arithmetic on host numpy records (copies in and out)."""
    import torch
    dx = DeviceBytes.from_numpy(x)
    dy = DeviceBytes.from_numpy(y)
    dr = DeviceBytes(x.nbytes)
    check(lib().mpres_elementwise(nmod, op, dx.ptr, dy.ptr, dr.ptr, len(x), None), "mpres_elementwise")
    torch.cuda.synchronize()
    return dr.to_numpy(x.dtype, len(x))


def rns_scale2pow(nmod, digits, D):
    import torch
    digits = np.ascontiguousarray(digits, dtype=np.int32)
    D = np.ascontiguousarray(D, dtype=np.uint32)
    dd, dD, do = DeviceBytes.from_numpy(digits), DeviceBytes.from_numpy(D), DeviceBytes(digits.nbytes)
    check(lib().mpres_rns_scale2pow(nmod, dd.ptr, dD.ptr, do.ptr, D.size, None), "mpres_rns_scale2pow")
    torch.cuda.synchronize()
    return do.to_numpy(np.int32, digits.size).reshape(digits.shape)


def rns_eval(nmod, digits, fast):
    import torch
    digits = np.ascontiguousarray(digits, dtype=np.int32)
    cnt = digits.size // nmod
    dd, lo, up = DeviceBytes.from_numpy(digits), DeviceBytes(16 * cnt), DeviceBytes(16 * cnt)
    check(lib().mpres_rns_eval(nmod, int(fast), dd.ptr, lo.ptr, up.ptr, cnt, None), "mpres_rns_eval")
    torch.cuda.synchronize()
    return lo.to_numpy(ER, cnt), up.to_numpy(ER, cnt)


def probe_ceil_log2(x):
    """ceil(log2(x)) evaluated on the GPU with the CUDA math library."""
    import torch
    x = np.ascontiguousarray(x, dtype=np.float64)
    dx, do = DeviceBytes.from_numpy(x), DeviceBytes(x.nbytes)
    check(lib().mpres_probe_ceil_log2(dx.ptr, do.ptr, x.size, None), "mpres_probe_ceil_log2")
    torch.cuda.synchronize()
    return do.to_numpy(np.float64, x.size)


PROBE_MUL_ADD, PROBE_ADD, PROBE_MULD_ADD, PROBE_FIXED_POINT = 0, 1, 2, 16


def probe_chain(nmod, kind, x, y, length):
    """One warp's reduction chains (mpres_probe_chain): x, y host arrays of
    32*length records (y doubles for PROBE_MULD_ADD, unused for PROBE_ADD);
    kind + PROBE_FIXED_POINT evaluates intervals in fixed point.
    Returns (cycles per step, lanes whose product rounded, lanes whose sum
    rounded, the 32 chains' sums)."""
    import torch
    x = np.ascontiguousarray(x)
    assert len(x) == 32 * length
    dx = DeviceBytes.from_numpy(x)
    dy = DeviceBytes.from_numpy(np.ascontiguousarray(y)) if y is not None else None
    cyc, rnd, res = DeviceBytes(8 * length), DeviceBytes(4 * length), DeviceBytes(32 * x.dtype.itemsize)
    check(lib().mpres_probe_chain(nmod, kind, dx.ptr, dy.ptr if dy else None, length, cyc.ptr, rnd.ptr, res.ptr,
                                  None), "mpres_probe_chain")
    torch.cuda.synchronize()
    r = rnd.to_numpy(np.uint32, length)
    return (cyc.to_numpy(np.int64, length), (r & 0xff).astype(np.int64), ((r >> 8) & 0xff).astype(np.int64),
            res.to_numpy(x.dtype, 32))


def probe_rounding(nmod, digits, D, count):
    """Cycles of a rounding's parts (mpres_probe_rounding) for 32*count numbers:
    digits int32[32*count, nmod], D uint32[32*count]; returns int64[count, 5]."""
    import torch
    digits = np.ascontiguousarray(digits, dtype=np.int32)
    D = np.ascontiguousarray(D, dtype=np.uint32)
    dd, dD = DeviceBytes.from_numpy(digits), DeviceBytes.from_numpy(D)
    cyc, out = DeviceBytes(8 * 5 * count), DeviceBytes(4 * 32)
    check(lib().mpres_probe_rounding(nmod, dd.ptr, dD.ptr, count, cyc.ptr, out.ptr, None), "mpres_probe_rounding")
    torch.cuda.synchronize()
    return cyc.to_numpy(np.int64, 5 * count).reshape(count, 5)


def probe_eval_phases(nmod, digits, count):
    """Cycles of the interval evaluation's phases (mpres_probe_eval_phases) for
    32*count numbers digits int32[32*count, nmod]; returns int64[count, 40]."""
    import torch
    dd = DeviceBytes.from_numpy(np.ascontiguousarray(digits, dtype=np.int32))
    cyc, out = DeviceBytes(8 * 40 * count), DeviceBytes(4 * 32)
    check(lib().mpres_probe_eval_phases(nmod, dd.ptr, count, cyc.ptr, out.ptr, None), "mpres_probe_eval_phases")
    torch.cuda.synchronize()
    return cyc.to_numpy(np.int64, 40 * count).reshape(count, 40)


def probe_fraction_sum_cycles(nmod, digits, reps=64):
    """Cycles per upward fraction sum on one warp: {FP64, fixed point, integer leaves + FP64 tree}."""
    import torch
    dd = DeviceBytes.from_numpy(np.ascontiguousarray(digits, dtype=np.int32))
    cyc, out = DeviceBytes(8 * 3), DeviceBytes(4 * 32)
    check(lib().mpres_probe_fraction_sum(nmod, 0, dd.ptr, reps, cyc.ptr, out.ptr, None), "mpres_probe_fraction_sum")
    torch.cuda.synchronize()
    return cyc.to_numpy(np.int64, 3)


def probe_int_leaves(nmod, digits):
    """{integer RU, __dmul_ru, integer RD, __dmul_rd} leaf bits per residue (mpres_probe_fraction_sum)."""
    import torch
    digits = np.ascontiguousarray(digits, dtype=np.int32)
    count = digits.size // nmod
    dd, res = DeviceBytes.from_numpy(digits), DeviceBytes(8 * 4 * digits.size)
    check(lib().mpres_probe_fraction_sum(nmod, 1, dd.ptr, count, res.ptr, None, None), "mpres_probe_fraction_sum")
    torch.cuda.synchronize()
    return res.to_numpy(np.uint64, 4 * digits.size).reshape(-1, 4)


def probe_check(which, nmod, a, b=None):
    """Runs a replacement self-check (see mpres_gb300_probe.h) and returns its output pairs."""
    import torch
    a = np.ascontiguousarray(a)
    da = DeviceBytes.from_numpy(a)
    db = DeviceBytes.from_numpy(np.ascontiguousarray(b)) if b is not None else None
    width, dt = {0: (4, np.float64), 1: (2, np.float64), 2: (2, np.int32), 3: (2, np.int32)}[which]
    out = DeviceBytes(len(a) * width * np.dtype(dt).itemsize)
    check(lib().mpres_probe_check(which, nmod, da.ptr, db.ptr if db else None, out.ptr, len(a), None),
          "mpres_probe_check")
    torch.cuda.synchronize()
    return out.to_numpy(dt, len(a) * width).reshape(len(a), width)
