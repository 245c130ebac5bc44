/*
 * mpres_gb300: GB300-native RNS multiple-precision BLAS hot path.
 *
 * C ABI of libmpres_gb300.so.  Every entry point takes plain pointers and sizes
 * and replaces one interface of MPRES-BLAS (cited per function as
 * reference-file:line).  The data types keep the reference's memory layouts
 * (src/types.cuh:46-131), so arrays built by reference code can be passed as-is.
 *
 * Moduli sets.  The reference fixes one set per build through src/params.h.
 * This library holds the predefined 32-bit sets of 8, 16 and 32 moduli at once;
 * every call names its set by `nmod` (the reference's RNS_MODULI_SIZE), and an
 * mp_float_t of that set is 4*nmod + 40 bytes.  include/mpres_gb300.hpp wraps
 * these functions in the reference's own C++ names and template signatures.
 *
 * Errors.  The reference returns nothing and prints CUDA errors
 * (src/common.cuh:38-53).  Every function here returns MPRES_SUCCESS or an
 * error code; mpres_last_error() describes the last failure of this thread.
 * Invalid sizes or strides that the reference silently ignores are ignored
 * here too (MPRES_SUCCESS, nothing computed), with the same tests.
 *
 * Streams.  `stream` is a cudaStream_t (NULL = the legacy default stream).
 * Computations are asynchronous with respect to the host, like the reference's
 * kernel launches; the copy helpers are synchronous like the reference's.
 *
 * Inputs must hold canonical residues (0 <= digit < modulus), as every array
 * produced by the reference's and this library's conversions does.
 */
#ifndef MPRES_GB300_H
#define MPRES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- types, identical in layout to src/types.cuh:46-131 ---------------- */
#ifndef MPRES_REFERENCE_TYPES_DEFINED
#define MPRES_REFERENCE_TYPES_DEFINED
typedef struct {
    double frac; /* significand */
    long exp;    /* exponent, base 2 */
} er_float_t;

typedef struct { int x, y, z, w; } mpres_int4;

/* SoA multiple-precision array: digits element-major ([x0 residues][x1 residues]...),
 * sign[len], exp[len], eval[2*len] = [lower bounds][upper bounds], buf[len], and
 * len = DEVICE pointer to the element count. */
typedef struct {
    int *digits;
    int *sign;
    int *exp;
    er_float_t *eval;
    mpres_int4 *buf;
    int *len;
} mp_array_t;

typedef struct {
    double *as; /* nonzeros, row-major */
    int *ja;    /* column indices */
    int *irp;   /* row start pointers, m + 1 entries */
} csr_t;

typedef struct {
    double *as; /* m * maxnzr slots, column-major, zero padded */
    int *ja;
} ell_t;
#endif

enum mpres_status {
    MPRES_SUCCESS = 0,
    MPRES_ERR_INVALID_VALUE = 1, /* unsupported moduli set or argument */
    MPRES_ERR_NOT_INITIALIZED = 2,
    MPRES_ERR_CUDA = 3,          /* a CUDA runtime call or a kernel launch failed */
    MPRES_ERR_NOT_SUPPORTED = 4, /* e.g. a transposed mp_gemm (the reference prints and returns) */
    MPRES_ERR_CANCELLED = 5      /* a serving request withdrawn before it ran (mpres_gb300_server.h) */
};

/* mblas_trans_type values of src/blas/mblas_enum.cuh:25-29 */
#define MPRES_NO_TRANS 111
#define MPRES_TRANS 112
#define MPRES_CONJ_TRANS 113

/* Last error of the calling host thread, or "" after a success. */
const char *mpres_last_error(void);

/* Bytes of one mp_float_t of the given set (4*nmod + 40), 0 if unsupported. */
size_t mpres_mp_float_size(int nmod);

/* Replaces rns_const_init() (src/rns.cuh:324-442) and mp_const_init()
 * (src/arith/arith_utils.cuh:44-90): computes the set's constants and places
 * them on the current device.  Idempotent; must precede any other call of the
 * set on that device. */
int mpres_init(int nmod);

/* Integer constants of the set: out[0] = MP_PRECISION, out[1] = MP_H,
 * out[2] = MP_J, out[3] = RNS_EVAL_REF_FACTOR, out[4] = RNS_MODULI_PRODUCT_LOG2. */
int mpres_get_int_constants(int nmod, int *out);

/* ---- containers (src/mparray.cuh:35-160, src/sparse/utils/*.cuh) -------- */

/* cuda::mp_array_init (src/mparray.cuh:35-56): allocates the six device arrays. */
int mpres_array_init(int nmod, mp_array_t *a, size_t size);
/* cuda::mp_array_clear (src/mparray.cuh:59-68). */
int mpres_array_clear(mp_array_t *a);
/* cuda::mp_array_host2device (src/mparray.cuh:76-118): host mp_float_t[size] ->
 * device SoA, packed on the host and sent with four bulk copies. */
int mpres_array_host2device(int nmod, mp_array_t *dst, const void *host_src, size_t size);
/* cuda::mp_array_device2host (src/mparray.cuh:125-160). */
int mpres_array_device2host(int nmod, void *host_dst, const mp_array_t *src, size_t size);

/* cuda::csr_init / csr_host2device / csr_clear (src/sparse/utils/csr_utils.cuh:58-78). */
int mpres_csr_init(csr_t *csr, int m, int nnz);
int mpres_csr_host2device(csr_t *dev, const csr_t *host, int m, int nnz);
int mpres_csr_clear(csr_t *csr);
/* cuda::ell_init / ell_host2device / ell_clear (src/sparse/utils/ell_utils.cuh:55-71). */
int mpres_ell_init(ell_t *ell, int m, int maxnzr);
int mpres_ell_host2device(ell_t *dev, const ell_t *host, int m, int maxnzr);
int mpres_ell_clear(ell_t *ell);

/* ---- Matrix Market files (host) ----------------------------------------- */

/* collect_mtx_stats (src/sparse/utils/mtx_reader.cuh:52-101): sizes of a
 * coordinate file, the longest row (mirrored entries of a symmetric matrix
 * counted), the diagonal entries, symmetry, and the data type ("real" or
 * "integer"; datatype may be NULL, else 16 bytes).  Pattern and complex files
 * are rejected with MPRES_ERR_NOT_SUPPORTED. */
int mpres_mtx_stats(const char *path, int *m, int *n, int *lines, int *maxnzr, int *nzmd, int *symmetric,
                    char *datatype);
/* build_csr (mtx_reader.cuh:200-253): as[nnz], ja[nnz], irp[m + 1], host arrays
 * the caller allocates; nnz = lines, or 2*(lines - nzmd) + nzmd if symmetric.
 * The entry order within rows is the reference's, so SpMV results match. */
int mpres_mtx_build_csr(const char *path, int m, int nnz, int lines, int symmetric, double *as, int *ja, int *irp);
/* build_ell (mtx_reader.cuh:374-406): as[m*maxnzr], ja[m*maxnzr], column-major,
 * padding 0.0 / -1. */
int mpres_mtx_build_ell(const char *path, int m, int maxnzr, int lines, int symmetric, double *as, int *ja);

/* ---- conversion --------------------------------------------------------- */

/* mp_set_d (src/arith/assign.cuh:54-81), host: x[count] -> mp_float_t[count]. */
int mpres_set_d(int nmod, const double *x, size_t count, void *out);

/* The same conversion on the device, bit-identical to mpres_set_d (the
 * reference's host mp_set_d with its host interval evaluation,
 * src/rns.cuh:645-716); no counterpart in the reference, which converts on the
 * host and copies with mp_array_host2device (src/mparray.cuh:76-118).
 * x is a device array of count doubles.  mpres_set_d_device writes count AoS
 * mp_float_t records to the device buffer out; mpres_array_set_d writes
 * elements [offset, offset + count) of dst.  Both wait for the stream (they
 * read back a flag: MPRES_ERR_NOT_SUPPORTED if an input would leave the replayed
 * host behaviour, which no finite double is known to do). */
int mpres_set_d_device(int nmod, const double *x, size_t count, void *out, void *stream);
int mpres_array_set_d(int nmod, mp_array_t *dst, size_t offset, const double *x, size_t count, void *stream);

/* ---- v2 vector kernels over AoS mp_float_t vectors (device memory) -------- */

/* cuda::mp_diff (src/blas/v2/diff_v2.cuh): r = x - y;
 * cuda::mp_axpy (axpy_v2.cuh): r = alpha*x + y;  cuda::mp_maxpy (maxpy_v2.cuh):
 * r = -alpha*x + y (alpha a device record).  The reference's kernels are launched
 * by their callers with <<<n/threads + 1, threads>>>; element-wise results do
 * not depend on the launch. */
int mpres_v2_diff(int nmod, int n, const void *x, const void *y, void *r, int threads, void *stream);
int mpres_v2_axpy(int nmod, int n, const void *alpha, const void *x, const void *y, void *r, int threads,
                  void *stream);
int mpres_v2_maxpy(int nmod, int n, const void *alpha, const void *x, const void *y, void *r, int threads,
                   void *stream);
/* cuda::mp_dot<blocks, threads> (dot_v2.cuh): r[0] = x.y, blocks*threads strided
 * chains, a tree per block, one block over the block sums (the order is the
 * reference's for the same blocks and threads, threads <= 256). */
int mpres_v2_dot(int nmod, int n, const void *x, const void *y, void *r, int blocks, int threads, void *stream);
/* cuda::mp_norm2<blocks, threads> (norm2_v2.cuh): the sum of squares with
 * mp_add_abs in the same two-pass order, then mp_dsqrt on the host; waits for
 * the stream. */
int mpres_v2_norm2(int nmod, int n, const void *x, double *out, int blocks, int threads, void *stream);

/* ---- conjugate gradients over CSR ---------------------------------------- */

/* mp_cg_csr<threads, blocks_reduce> (src/sparse/solver/cg_csr.cuh) and
 * mp_pcg_csr (pcg_csr.cuh, Jacobi preconditioner: ptype 1, M = the inverse
 * diagonal as doubles in device memory): solves A x = b for a double CSR matrix
 * A (device) with AoS mp_float_t vectors b and x (device; x holds the initial
 * guess and receives the solution).  resvec (host, resvec_cap doubles)
 * receives ||r_k|| / ||r_0|| for k = 0..iters, as the reference's resvec;
 * *iters the iterations run.  Bit-identical to the reference for the same
 * threads and blocks_reduce (32 and 256 in cg_csr.cuh, 64 and 256 in
 * pcg_csr.cuh).  Synchronous: the divisions run on the host each iteration. */
int mpres_cg_csr(int nmod, int n, const csr_t *A, const void *b, double tol, int maxit, void *x, double *resvec,
                 int resvec_cap, int *iters, int threads, int blocks_reduce, void *stream);
int mpres_pcg_csr(int nmod, int n, const csr_t *A, const void *b, double tol, int maxit, int ptype, const double *M,
                  void *x, double *resvec, int resvec_cap, int *iters, int threads, int blocks_reduce, void *stream);

/* ---- host MPFR operations ------------------------------------------------ */

/* ::mp_div (src/arith/div.cuh:33-45), ::mp_sqrt and ::mp_dsqrt (src/arith/sqrt.cuh):
 * the operands rounded to MP_PRECISION bits, the correctly rounded (nearest-even)
 * quotient or root at MP_PRECISION bits, converted back as mp_set_mpfr does
 * (mp_dsqrt: rounded again to a double).  Host mp_float_t records; exact
 * integer arithmetic gives MPFR's bits without MPFR.  Division by zero and
 * roots of negative numbers return MPRES_ERR_INVALID_VALUE. */
int mpres_div(int nmod, const void *x, const void *y, void *r);
int mpres_sqrt(int nmod, const void *x, void *r);
int mpres_dsqrt(int nmod, const void *x, double *out);
/* cuda::mp_div and cuda::mp_dsqrt (src/arith/div.cuh:56-65, sqrt.cuh): the same
 * with the records in device memory (synchronous copies, host computation). */
int mpres_div_device(int nmod, const void *x, const void *y, void *r);
int mpres_dsqrt_device(int nmod, const void *x, double *out);

/* ---- BLAS ---------------------------------------------------------------- */

/* cuda::mp_dot<gridDim1, blockDim1, gridDim2, gridDim3, blockDim3>
 * (src/blas/dot.cuh:84-108): r[0] = sum x_i * y_i.  The launch parameters are the
 * reference's template arguments; gridDim3 and blockDim3 fix the summation order
 * (gridDim3*blockDim3 strided partial sums, a tree over each block of
 * blockDim3, then one block over the gridDim3 block sums), so results are
 * bit-identical to the reference called with the same arguments.  `buffer`
 * (len >= n in the reference) is accepted and not touched. */
int mpres_dot(int nmod, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy, mp_array_t *r,
              mp_array_t *buffer, int gridDim1, int blockDim1, int gridDim2, int gridDim3, int blockDim3,
              void *stream);

/* mp_dot that allocates nothing: no counterpart in the reference.  For callers
 * that cannot allocate device memory once they are running -- a serving process
 * that has reserved the whole device under a fixed memory budget, or a host
 * application whose own allocator owns the GPU -- and for loops that cannot
 * afford the device-wide synchronisation of cudaFree.  mpres_dot allocates a
 * workspace on the first call on each stream; this variant keeps the gridDim3
 * block sums in a static device array of MPRES_DOT_NOALLOC_MAX_BLOCKS entries
 * (688 KB, held by every GPU that loads the library until the process exits)
 * and rejects a larger gridDim3 with MPRES_ERR_INVALID_VALUE.  The first call
 * on a device looks the array's address up (cudaGetSymbolAddress); make that
 * first call before any stream capture.  All calls share the one array: calls
 * whose executions overlap on the GPU (other streams, other host threads) race
 * and must be serialised by the caller.  The array needs no clearing: each call
 * writes every block sum before it reads it.  Results are bit-identical to
 * mpres_dot with the same gridDim3 and blockDim3. */
#define MPRES_DOT_NOALLOC_MAX_BLOCKS 4096
int mpres_dot_noalloc(int nmod, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy, mp_array_t *r,
                      int gridDim3, int blockDim3, void *stream);

/* cuda::mp_gemv<gridDim1, blockDim1, gridDim2, blockDim3> (src/blas/gemv.cuh:150-269):
 * y = alpha*op(A)*x + beta*y, A column-major.  blockDim3 fixes the summation order
 * (blockDim3 strided partial sums per row, then a tree).  buffer1/buffer2 are
 * accepted and not touched. */
int mpres_gemv(int nmod, int trans, int m, int n, const mp_array_t *alpha, const mp_array_t *A, int lda,
               const mp_array_t *x, int incx, const mp_array_t *beta, mp_array_t *y, int incy,
               mp_array_t *buffer1, mp_array_t *buffer2, int gridDim1, int blockDim1, int gridDim2,
               int blockDim3, void *stream);

/* cuda::mp_gemm<blockDim1x, blockDim1y, gridDim2x, gridDim2y, blockDim3>
 * (src/blas/gemm.cuh:69-168): C = alpha*A*B + beta*C, column-major, no-transpose
 * only (the reference prints and returns for the other cases; this returns
 * MPRES_ERR_NOT_SUPPORTED).  Launch parameters do not affect results.  The
 * signed, power-of-two-scaled residues of A and B, (m*k + k*n)*4*nmod bytes, go
 * to the per-(device, stream) workspace; without room for them the same result
 * comes from the slower step-by-step chain, which needs no scratch. */
int mpres_gemm(int nmod, int transa, int transb, int m, int n, int k, const mp_array_t *alpha,
               const mp_array_t *A, int lda, const mp_array_t *B, int ldb, const mp_array_t *beta, mp_array_t *C,
               int ldc, mp_array_t *buffer, int blockDim1x, int blockDim1y, int gridDim2x, int gridDim2y,
               int blockDim3, void *stream);

/* cuda::mp_spmv_csr<threads> (src/sparse/spmv/spmv_csr.cuh:48-63): y = A*x with a
 * double CSR matrix and AoS mp_float_t vectors x (>= max(ja)+1) and y (>= m) in
 * device memory.  The reference is a kernel its caller launches; `threads` is
 * its template argument (any value gives the same result). */
int mpres_spmv_csr(int nmod, int m, const csr_t *csr, const void *x, void *y, int threads, void *stream);

/* cuda::mp_spmv_csrv<threads, threadsPerRow> (src/sparse/spmv/spmv_csrv.cuh:48-86);
 * threadsPerRow in {1, 2, 4, 8, 16, 32} fixes the summation order. */
int mpres_spmv_csrv(int nmod, int m, const csr_t *csr, const void *x, void *y, int threads, int threadsPerRow,
                    void *stream);

/* cuda::mp_spmv_ell<threads> (src/sparse/spmv/spmv_ell.cuh:49-67): ELLPACK,
 * column-major slots, explicit zeros skipped. */
int mpres_spmv_ell(int nmod, int m, int maxnzr, const ell_t *ell, const void *x, void *y, int threads,
                   void *stream);

#ifdef __cplusplus
}
#endif

#endif
