"""The reference library's own device code on the GPU: oracle/_ref/ref_kernels_<N>.cubin
(its headers compiled unmodified for sm_103a by oracle/ref/build_ref.sh) loaded with the
CUDA driver API through ctypes, its constant tables filled from oracle/_ref/ref_consts_<N>.bin
(what its rns_const_init / mp_const_init compute; oracle/ref/dump_consts.py).

TEST AND BENCHMARK INFRASTRUCTURE ONLY: the checker and the GPU baseline, never the
product.  Device memory comes from torch; the module is loaded into the context torch
made current.  The host launch sequences of the reference's drivers, which live in
templates of its headers, are restated here with the file:line they follow:

    dot()   cuda::mp_dot<g1, b1, g2, g3, b3>   src/blas/dot.cuh:85-108 (and mp_array_reduce_sum, :42-66)
    gemm()  cuda::mp_gemm<b1x, b1y, g2x, g2y, b3> src/blas/gemm.cuh:70-168 (no transposition)
    gemv()  cuda::mp_gemv<g1, b1, g2, b3>    src/blas/gemv.cuh:150-220 (no transposition, unit strides)
    spmv_csr()  cuda::mp_spmv_csr<32><<<m/32+1, 32>>>  tests/sparse/spmv/csr/test_mpres_spmv_csr.cuh
    spmv_csrv() cuda::mp_spmv_csrv<32, tpr><<<m/(32/tpr)+1, 32>>>  tests/sparse/spmv/csr/test_mpres_spmv_csrv.cuh:40-65
    spmv_ell()  cuda::mp_spmv_ell<32><<<m/32+1, 32>>>  tests/sparse/spmv/ell/test_mpres_spmv_ell.cuh:39-62

Numbers travel as AoS mp_float_t records (oracle.ffi.mp_dtype) or SoA mp_array_t
views of torch tensors (RefArray).
"""
import ctypes
import pathlib
import struct

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
P = ctypes.c_void_p
BLOCK_SIZE_FOR_RESIDUES = 64  # src/kernel_config.cuh:53 for 8, 16 and 32 moduli
CU_LIMIT_MALLOC_HEAP_SIZE = 0x02
CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8

K = {
    "mul_esi": "_ZN4cuda24mp_vector_mul_esi_kernelE10mp_array_tiS0_iS0_ii",
    "mul_digits": "_ZN4cuda27mp_vector_mul_digits_kernelE10mp_array_tiS0_iS0_ii",
    "vec_round": "_ZN4cuda22mp_vector_round_kernelE10mp_array_tii",
    "reduce1": "_ZN4cuda27mp_array_reduce_sum_kernel1Ej10mp_array_tP10mp_float_tj",
    "reduce2": "_ZN4cuda27mp_array_reduce_sum_kernel2EjP10mp_float_t10mp_array_tj",
    "gemm_nn": "_ZN4cuda30matrix_multiply_notrans_kernelEjjj10mp_array_tS0_iS0_iS0_i",
    "mat2scal_esi": "_ZN4cuda26mp_mat2scal_mul_esi_kernelE10mp_array_tiS0_iS0_ii",
    "mat2scal_digits": "_ZN4cuda29mp_mat2scal_mul_digits_kernelE10mp_array_tiS0_iS0_ii",
    "mat_round": "_ZN4cuda22mp_matrix_round_kernelE10mp_array_tiii",
    "vec2scal_esi": "_ZN4cuda26mp_vec2scal_mul_esi_kernelE10mp_array_tiS0_iS0_i",
    "vec2scal_digits": "_ZN4cuda29mp_vec2scal_mul_digits_kernelE10mp_array_tiS0_iS0_i",
    "mat2vec_esi": "_ZN4cuda32mp_mat2vec_right_scal_esi_kernelE10mp_array_tiS0_iS0_iii",
    "mat2vec_digits": "_ZN4cuda35mp_mat2vec_right_scal_digits_kernelE10mp_array_tiS0_iS0_iii",  # internal linkage
    "row_sum": "_ZN4cuda21matrix_row_sum_kernelEjj10mp_array_tS0_ij",  # internal linkage
    "mat_add_esi": "_ZN4cuda24mp_matrix_add_esi_kernelE10mp_array_tiS0_iS0_iii",
    "mat_add_digits": "_ZN4cuda27mp_matrix_add_digits_kernelE10mp_array_tiS0_iS0_iii",  # internal linkage
    "spmv_csr": "_ZN4cuda11mp_spmv_csrILi32EEEvi5csr_tP10mp_float_tS3_",
    "spmv_ell": "_ZN4cuda11mp_spmv_ellILi32EEEvii5ell_tP10mp_float_tS3_",
    **{"spmv_csrv%d" % t: "_ZN4cuda12mp_spmv_csrvILi32ELi%dEEEvi5csr_tP10mp_float_tS3_" % t for t in (1, 2, 4, 8, 16, 32)},
    "ew_add": "ref_ew_add",
    "ew_mul": "ref_ew_mul",
    "ew_mul_d": "ref_ew_mul_d",
}


class MpArrayT(ctypes.Structure):
    _fields_ = [(f, P) for f in ("digits", "sign", "exp", "eval", "buf", "len")]


class CsrT(ctypes.Structure):
    _fields_ = [("as_", P), ("ja", P), ("irp", P)]


class EllT(ctypes.Structure):
    _fields_ = [("as_", P), ("ja", P)]


def available(n):
    return (REF_DIR / ("ref_kernels_%d.cubin" % n)).exists() and (REF_DIR / ("ref_consts_%d.bin" % n)).exists()


def next_pow2(v):
    return 1 << max(0, (int(v) - 1).bit_length())


class RefArray:
    """An mp_array_t (SoA, src/types.cuh:85-92) over torch CUDA tensors."""

    def __init__(self, n, size):
        import torch
        self.n, self.size = n, size
        s = max(size, 1)
        self.digits = torch.zeros(s * n, dtype=torch.int32, device="cuda")
        self.sign = torch.zeros(s, dtype=torch.int32, device="cuda")
        self.exp = torch.zeros(s, dtype=torch.int32, device="cuda")
        self.eval = torch.zeros((2 * s, 2), dtype=torch.int64, device="cuda")
        self.buf = torch.zeros(s * 4, dtype=torch.int32, device="cuda")
        self.len = torch.tensor([size], dtype=torch.int32, device="cuda")
        self.a = MpArrayT(self.digits.data_ptr(), self.sign.data_ptr(), self.exp.data_ptr(), self.eval.data_ptr(),
                          self.buf.data_ptr(), self.len.data_ptr())

    def upload(self, rec):
        import torch
        n = self.n
        self.digits.copy_(torch.from_numpy(np.ascontiguousarray(rec["digits"]).reshape(-1)))
        self.sign.copy_(torch.from_numpy(np.ascontiguousarray(rec["sign"])))
        self.exp.copy_(torch.from_numpy(np.ascontiguousarray(rec["exp"])))
        ev = np.empty((2 * self.size, 2), np.int64)
        for h in (0, 1):
            ev[h * self.size:(h + 1) * self.size, 0] = np.ascontiguousarray(rec["eval"][:, h]["frac"]).view(np.int64)
            ev[h * self.size:(h + 1) * self.size, 1] = rec["eval"][:, h]["exp"]
        self.eval.copy_(torch.from_numpy(ev))
        del n
        return self

    @classmethod
    def copy_of(cls, ta, offset, length):
        """A RefArray holding elements [offset, offset + length) of an array with the same
        SoA tensors (digits [size*n], sign, exp [size], eval [2*size, 2]): its own
        storage, so that its `len` is its length.  The reference's kernels need that:
        scalar operands are read as eval[0], eval[1] (src/mpvector.cuh:147-148)."""
        r = cls(ta.nmod, length)
        n, o = ta.nmod, offset
        r.digits.copy_(ta.digits[o * n:(o + length) * n])
        r.sign.copy_(ta.sign[o:o + length])
        r.exp.copy_(ta.exp[o:o + length])
        r.eval[:length].copy_(ta.eval[o:o + length])
        r.eval[length:2 * length].copy_(ta.eval[ta.size + o:ta.size + o + length])
        return r

    def copy_into(self, ta, offset):
        """The inverse of copy_of: this array's elements into [offset, offset + size) of ta."""
        n, o, k = self.n, offset, self.size
        ta.digits[o * n:(o + k) * n].copy_(self.digits[:k * n])
        ta.sign[o:o + k].copy_(self.sign[:k])
        ta.exp[o:o + k].copy_(self.exp[:k])
        ta.eval[o:o + k].copy_(self.eval[:k])
        ta.eval[ta.size + o:ta.size + o + k].copy_(self.eval[k:2 * k])

    def download(self, dtype):
        out = np.zeros(self.size, dtype)
        out["digits"] = self.digits.view(-1, self.n).cpu().numpy()
        out["sign"] = self.sign.cpu().numpy()
        out["exp"] = self.exp.cpu().numpy()
        ev = self.eval.cpu().numpy()
        for h in (0, 1):
            half = ev[h * self.size:(h + 1) * self.size]
            out["eval"][:, h]["frac"] = half[:, 0].view(np.float64)
            out["eval"][:, h]["exp"] = half[:, 1]
        return out


_heap_set = False
_loaded = {}


def ref_gpu(n):
    """The reference's cubin for n moduli, loaded once per process."""
    if n not in _loaded:
        _loaded[n] = RefGPU(n)
    return _loaded[n]


class RefGPU:
    """The reference's cubin for one moduli set, loaded into the current context."""

    def __init__(self, n, heap_bytes=1 << 30):
        global _heap_set
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the primary context, current on this thread
        self.n = n
        cu = ctypes.CDLL("libcuda.so.1")
        self.cu = cu
        self._check(cu.cuInit(0), "cuInit")
        if not _heap_set:
            # cuda::mrd allocates with device `new` (src/rns.cuh:589): room for every
            # resident thread's digits at once (2048 threads x 152 SMs x 128 B is 40 MB)
            self._check(cu.cuCtxSetLimit(CU_LIMIT_MALLOC_HEAP_SIZE, ctypes.c_size_t(heap_bytes)), "cuCtxSetLimit")
            _heap_set = True
        self.mod = P()
        path = str(REF_DIR / ("ref_kernels_%d.cubin" % n)).encode()
        self._check(cu.cuModuleLoad(ctypes.byref(self.mod), path), "cuModuleLoad")
        self._upload_constants()
        self.funcs = {}

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def _upload_constants(self):
        blob = (REF_DIR / ("ref_consts_%d.bin" % self.n)).read_bytes()
        assert blob[:4] == b"MPRC"
        (count,), off = struct.unpack_from("<I", blob, 4), 8
        for _ in range(count):
            (ln,) = struct.unpack_from("<H", blob, off)
            name = blob[off + 2:off + 2 + ln]
            off += 2 + ln
            (size,) = struct.unpack_from("<I", blob, off)
            off += 4
            data = blob[off:off + size]
            off += size
            dptr, dsize = ctypes.c_uint64(), ctypes.c_size_t()
            self._check(self.cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(dsize), self.mod, name),
                        "cuModuleGetGlobal(%s)" % name.decode())
            if dsize.value != size:
                raise RuntimeError("%s: %d bytes in the cubin, %d dumped" % (name.decode(), dsize.value, size))
            self._check(self.cu.cuMemcpyHtoD_v2(dptr, data, ctypes.c_size_t(size)), "cuMemcpyHtoD")

    def func(self, key):
        if key not in self.funcs:
            f = P()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, K[key].encode()),
                        "cuModuleGetFunction(%s)" % key)
            self.funcs[key] = f
        return self.funcs[key]

    def launch(self, key, grid, block, args, smem=0, stream=0):
        f = self.func(key)
        if smem > 48 * 1024:
            self._check(self.cu.cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem),
                        "cuFuncSetAttribute")
        grid = tuple(grid) + (1,) * (3 - len(grid))
        block = tuple(block) + (1,) * (3 - len(block))
        params = (P * len(args))(*[ctypes.cast(ctypes.pointer(a), P) for a in args])
        self._check(self.cu.cuLaunchKernel(f, *[ctypes.c_uint(v) for v in grid], *[ctypes.c_uint(v) for v in block],
                                           ctypes.c_uint(smem), P(stream), params, None), "cuLaunchKernel(%s)" % key)

    def sync(self):
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    # ------------------------------------------------------------------ element-wise

    def elementwise(self, op, x, y):
        """r[i] = x[i] + y[i] / x[i] * y[i] / x[i] * d[i] by cuda::mp_add / mp_mul / mp_mul_d."""
        import torch
        dx = torch.from_numpy(np.ascontiguousarray(x).view(np.uint8)).cuda()
        dy = torch.from_numpy(np.ascontiguousarray(y).view(np.uint8)).cuda()
        dr = torch.empty_like(dx)
        count = len(x)
        self.launch({"add": "ew_add", "mul": "ew_mul", "mul_d": "ew_mul_d"}[op], ((count + 127) // 128,), (128,),
                    [P(dx.data_ptr()), P(dy.data_ptr()), P(dr.data_ptr()), ctypes.c_int(count)])
        self.sync()
        return dr.cpu().numpy().view(x.dtype).copy()

    # ------------------------------------------------------------------ BLAS

    def dot(self, count, x, y, r, buffer, order=(512, 128, 8192, 256, 64), stream=0):
        """cuda::mp_dot (src/blas/dot.cuh:85-108) on RefArrays, incx = incy = 1; `buffer`
        holds count elements and `parts` the gridDim3 block sums (mp_array_reduce_sum's
        buffer, allocated there per call, :42-66, here by the caller once)."""
        g1, b1, g2, g3, b3 = order
        xa, ya, ra, ba = x.a, y.a, r.a, buffer.a
        one, cnt = ctypes.c_int(1), ctypes.c_int(count)
        self.launch("mul_esi", (g1,), (b1,), [ba, one, xa, one, ya, one, cnt], stream=stream)
        self.launch("mul_digits", (g2,), (BLOCK_SIZE_FOR_RESIDUES,), [ba, one, xa, one, ya, one, cnt], stream=stream)
        self.launch("vec_round", (g1,), (b1,), [ba, one, cnt], stream=stream)
        smem = b3 * (4 * self.n + 40)
        pw = ctypes.c_uint(next_pow2(b3))
        self.launch("reduce1", (g3,), (b3,), [ctypes.c_uint(count), ba, P(self._parts(g3)), pw], smem=smem,
                    stream=stream)
        self.launch("reduce2", (1,), (b3,), [ctypes.c_uint(g3), P(self._parts(g3)), ra, pw], smem=smem, stream=stream)

    def _parts(self, g3):
        import torch
        need = g3 * (4 * self.n + 40)
        if getattr(self, "_parts_t", None) is None or self._parts_t.numel() < need:
            self._parts_t = torch.empty(need, dtype=torch.uint8, device="cuda")
        return self._parts_t.data_ptr()

    def gemm(self, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, buffer, order=(32, 1, 128, 64, 16), stream=0):
        """cuda::mp_gemm, no transposition (src/blas/gemm.cuh:70-168), on RefArrays;
        `buffer` holds m * n elements."""
        b1x, b1y, g2x, g2y, b3 = order
        u = ctypes.c_uint
        i = ctypes.c_int
        self.launch("gemm_nn", ((n + b3 - 1) // b3, (m + b3 - 1) // b3), (b3, b3),
                    [u(m), u(n), u(k), alpha.a, A.a, i(lda), B.a, i(ldb), buffer.a, i(m)], stream=stream)
        g1 = ((m + b1x - 1) // b1x, (n + b1y - 1) // b1y)
        g3 = ((m + 15) // 16, (n + 15) // 16)
        self.launch("mat2scal_esi", g1, (b1x, b1y), [buffer.a, i(m), buffer.a, i(m), alpha.a, i(m), i(n)], stream=stream)
        self.launch("mat2scal_digits", (g2x, g2y), (BLOCK_SIZE_FOR_RESIDUES,),
                    [buffer.a, i(m), buffer.a, i(m), alpha.a, i(m), i(n)], stream=stream)
        self.launch("mat_round", g3, (16, 16), [buffer.a, i(m), i(m), i(n)], stream=stream)
        self.launch("mat2scal_esi", g1, (b1x, b1y), [C.a, i(ldc), C.a, i(ldc), beta.a, i(m), i(n)], stream=stream)
        self.launch("mat2scal_digits", (g2x, g2y), (BLOCK_SIZE_FOR_RESIDUES,),
                    [C.a, i(ldc), C.a, i(ldc), beta.a, i(m), i(n)], stream=stream)
        self.launch("mat_round", g3, (16, 16), [C.a, i(ldc), i(m), i(n)], stream=stream)
        self.launch("mat_add_esi", g1, (b1x, b1y), [C.a, i(ldc), C.a, i(ldc), buffer.a, i(m), i(m), i(n)],
                    stream=stream)
        self.launch("mat_add_digits", (g2x, g2y), (BLOCK_SIZE_FOR_RESIDUES,),
                    [C.a, i(ldc), C.a, i(ldc), buffer.a, i(m), i(m), i(n)], stream=stream)
        self.launch("mat_round", g3, (16, 16), [C.a, i(ldc), i(m), i(n)], stream=stream)

    def gemv(self, m, n, alpha, A, lda, x, beta, y, buffer1, buffer2, order=(256, 128, 256, 32), stream=0):
        """cuda::mp_gemv<g1, b1, g2, b3>(mblas_no_trans, m, n, alpha, A, lda, x, 1, beta, y, 1, buffer1,
        buffer2) (src/blas/gemv.cuh:150-220): buffer1 = alpha*x and y = beta*y (each rounded),
        buffer2 = A*diag(buffer1) (rounded), then per row the b3-thread sum plus y."""
        g1, b1, g2, b3 = order
        i, u = ctypes.c_int, ctypes.c_uint
        one = i(1)
        self.launch("vec2scal_esi", (g1,), (b1,), [buffer1.a, one, x.a, one, alpha.a, i(n)], stream=stream)
        self.launch("vec2scal_digits", (g2,), (BLOCK_SIZE_FOR_RESIDUES,), [buffer1.a, one, x.a, one, alpha.a, i(n)],
                    stream=stream)
        self.launch("vec_round", (g1,), (b1,), [buffer1.a, one, i(n)], stream=stream)
        self.launch("vec2scal_esi", (g1,), (b1,), [y.a, one, y.a, one, beta.a, i(m)], stream=stream)
        self.launch("vec2scal_digits", (g2,), (BLOCK_SIZE_FOR_RESIDUES,), [y.a, one, y.a, one, beta.a, i(m)],
                    stream=stream)
        self.launch("vec_round", (g1,), (b1,), [y.a, one, i(m)], stream=stream)
        self.launch("mat2vec_esi", (g1, g1), (b1,), [buffer2.a, i(m), A.a, i(lda), buffer1.a, one, i(m), i(n)],
                    stream=stream)
        self.launch("mat2vec_digits", (g2, g2), (BLOCK_SIZE_FOR_RESIDUES,),
                    [buffer2.a, i(m), A.a, i(lda), buffer1.a, one, i(m), i(n)], stream=stream)
        self.launch("vec_round", (g1,), (b1,), [buffer2.a, one, i(m * n)], stream=stream)
        self.launch("row_sum", (m,), (b3,), [u(m), u(n), buffer2.a, y.a, one, u(next_pow2(b3))],
                    smem=b3 * (4 * self.n + 40), stream=stream)

    def spmv_csr(self, m, irp_ptr, ja_ptr, as_ptr, x_ptr, y_ptr, stream=0):
        """cuda::mp_spmv_csr<32><<<m / 32 + 1, 32>>>(m, csr, x, y) as the reference's driver
        launches it (tests/sparse/spmv/csr/test_mpres_spmv_csr.cuh), device pointers."""
        csr = CsrT(as_ptr, ja_ptr, irp_ptr)
        self.launch("spmv_csr", (m // 32 + 1,), (32,), [ctypes.c_int(m), csr, P(x_ptr), P(y_ptr)], stream=stream)

    def spmv_csrv(self, m, tpr, irp_ptr, ja_ptr, as_ptr, x_ptr, y_ptr, stream=0):
        """cuda::mp_spmv_csrv<32, tpr><<<m / (32 / tpr) + 1, 32>>>(m, csr, x, y) as the reference's
        driver launches it (tests/sparse/spmv/csr/test_mpres_spmv_csrv.cuh:40-65)."""
        csr = CsrT(as_ptr, ja_ptr, irp_ptr)
        self.launch("spmv_csrv%d" % tpr, (m // (32 // tpr) + 1,), (32,), [ctypes.c_int(m), csr, P(x_ptr), P(y_ptr)],
                    stream=stream)

    def spmv_ell(self, m, maxnzr, ja_ptr, as_ptr, x_ptr, y_ptr, stream=0):
        """cuda::mp_spmv_ell<32><<<m / 32 + 1, 32>>>(m, maxnzr, ell, x, y) as the reference's driver
        launches it (tests/sparse/spmv/ell/test_mpres_spmv_ell.cuh:39-62)."""
        ell = EllT(as_ptr, ja_ptr)
        self.launch("spmv_ell", (m // 32 + 1,), (32,), [ctypes.c_int(m), ctypes.c_int(maxnzr), ell, P(x_ptr),
                                                         P(y_ptr)], stream=stream)
