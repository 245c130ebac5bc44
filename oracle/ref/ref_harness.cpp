/*
 * CPU build of the reference library's hot path (MPRES-BLAS, src/), used only to
 * pin the oracle and to generate golden vectors.
 *
 * The reference headers are compiled UNMODIFIED from where they lie; cuda_emu.h
 * supplies host stand-ins for the CUDA features they use.  Device functions
 * (namespace cuda: mp_add, mp_mul, mp_mul_d, mp_round, rns_eval_compute_fast,
 * rns_scale2pow, ...) and barrier-free kernels run exactly as written.  The host
 * drivers that contain `<<<...>>>` launches (blas/dot.cuh, blas/gemv.cuh,
 * blas/gemm.cuh) cannot be parsed by g++, so their launch sequences -- and the
 * three kernels that live in those files -- are transcribed below, each citing
 * the file:line it follows; the arithmetic inside them is still the reference's.
 *
 * Built once per moduli set by oracle/ref/build_ref.sh into
 * oracle/_ref/libmpres_ref_<N>.so.  Test infrastructure only.
 */
#include "cuda_emu.h"

#include "arith/assign.cuh"
#include "arith/add.cuh"
#include "arith/mul.cuh"
#include "arith/muld.cuh"
#include "arith/div.cuh"
#include "arith/sqrt.cuh"
#include "arith/addabs.cuh"
#include "arith/sub.cuh"
#include "mpvector.cuh"
#include "mpmatrix.cuh"
#include "mpreduct.cuh"
#include "blas/mblas_enum.cuh"
#include "kernel_config.cuh"
#include "sparse/spmv/spmv_csr.cuh"
#include "sparse/spmv/spmv_csrv.cuh"
#include "sparse/spmv/spmv_ell.cuh"
#include "sparse/utils/mtx_reader.cuh"

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
namespace emu {
    Block *g_block = nullptr;
    std::vector<char> g_stacks;
}
/* Storage behind `extern __shared__ mp_float_t sdata[]` (one block at a time). */
namespace cuda {
    mp_float_t sdata[8192];
}

namespace {

/* An mp_array_t in host memory, in the reference's SoA layout (src/types.cuh:85-92). */
struct HostArray {
    std::vector<int> digits, sign, exp;
    std::vector<er_float_t> eval;
    std::vector<int4> buf;
    int len = 0;
    mp_array_t a;
    explicit HostArray(int n) : digits((size_t)RNS_MODULI_SIZE * (n > 0 ? n : 1)),
                                sign(n > 0 ? n : 1), exp(n > 0 ? n : 1), eval(2 * (n > 0 ? n : 1)),
                                buf(n > 0 ? n : 1), len(n) {
        a.digits = digits.data(); a.sign = sign.data(); a.exp = exp.data();
        a.eval = eval.data(); a.buf = buf.data(); a.len = &len;
    }
    void load(const mp_float_t *src) {
        for (int i = 0; i < len; i++) {
            for (int j = 0; j < RNS_MODULI_SIZE; j++) digits[(size_t)i * RNS_MODULI_SIZE + j] = src[i].digits[j];
            sign[i] = src[i].sign; exp[i] = src[i].exp;
            eval[i] = src[i].eval[0]; eval[len + i] = src[i].eval[1];
        }
    }
    void store(mp_float_t *dst) const {
        for (int i = 0; i < len; i++) {
            for (int j = 0; j < RNS_MODULI_SIZE; j++) dst[i].digits[j] = digits[(size_t)i * RNS_MODULI_SIZE + j];
            dst[i].sign = sign[i]; dst[i].exp = exp[i];
            dst[i].eval[0] = eval[i]; dst[i].eval[1] = eval[len + i];
        }
    }
};

int stride_len(int n, int inc) { return n <= 0 ? 0 : 1 + (n - 1) * (inc < 0 ? -inc : inc); }

/* src/blas/dot.cuh:42-66 (mp_array_reduce_sum) */
void reduce_sum(int g, int b, int n, mp_array_t &x, mp_array_t &result) {
    std::vector<mp_float_t> d_buf(g);
    mp_float_t *pbuf = d_buf.data();
    const unsigned int POW = nextPow2(b);
    emu::launch(dim3(g), dim3(b), [&] { cuda::mp_array_reduce_sum_kernel1(n, x, pbuf, POW); }, true);
    emu::launch(dim3(1), dim3(b), [&] { cuda::mp_array_reduce_sum_kernel2(g, pbuf, result, POW); }, true);
}

/* src/blas/gemv.cuh:44-85 (matrix_row_sum_kernel), transcribed */
void matrix_row_sum(unsigned m, unsigned n, mp_array_t A, mp_array_t y, int incy, unsigned nextPow2v) {
    using cuda::sdata;
    const unsigned tid = threadIdx.x, bid = blockIdx.x, bsize = blockDim.x;
    unsigned i = threadIdx.x;
    sdata[tid] = cuda::MP_ZERO;
    while (i < n) {
        cuda::mp_add(&sdata[tid], sdata[tid], A, i * m + bid);
        i += bsize;
    }
    __syncthreads();
    i = nextPow2v >> 1;
    while (i >= 1) {
        if ((tid < i) && (tid + i < bsize)) cuda::mp_add(&sdata[tid], sdata[tid], sdata[tid + i]);
        i = i >> 1;
        __syncthreads();
    }
    if (tid == 0) {
        int iy = incy > 0 ? bid * incy : (-(int)m + (int)bid + 1) * incy;
        cuda::mp_add(y, iy, y, iy, sdata[tid]);
    }
}

/* src/blas/gemv.cuh:88-128 (matrix_col_sum_kernel), transcribed */
void matrix_col_sum(unsigned m, unsigned n, mp_array_t A, mp_array_t y, int incy, unsigned nextPow2v) {
    using cuda::sdata;
    const unsigned tid = threadIdx.x, bid = blockIdx.x, bsize = blockDim.x;
    unsigned i = tid;
    sdata[tid] = cuda::MP_ZERO;
    while (i < m) {
        cuda::mp_add(&sdata[tid], sdata[tid], A, bid * m + i);
        i += bsize;
    }
    __syncthreads();
    i = nextPow2v >> 1;
    while (i >= 1) {
        if ((tid < i) && (tid + i < bsize)) cuda::mp_add(&sdata[tid], sdata[tid], sdata[tid + i]);
        i = i >> 1;
        __syncthreads();
    }
    if (tid == 0) {
        int iy = incy > 0 ? bid * incy : (-(int)n + (int)bid + 1) * incy;
        cuda::mp_add(y, iy, y, iy, sdata[tid]);
    }
}

/* src/blas/gemm.cuh:39-60 (matrix_multiply_notrans_kernel), transcribed */
void matrix_multiply_notrans(unsigned m, unsigned n, unsigned k, mp_array_t A, int lda, mp_array_t B, int ldb,
                             mp_array_t C, int ldc) {
    int col = blockIdx.x * blockDim.x + threadIdx.x;
    int row = blockIdx.y * blockDim.y + threadIdx.y;
    int indexC = row + col * ldc;
    if (col < (int)n && row < (int)m) {
        mp_float_t mul = cuda::MP_ZERO;
        mp_float_t sum = cuda::MP_ZERO;
        for (int i = 0; i < (int)k; i++) {
            cuda::mp_mul(&mul, A, (lda * i + row), B, (col * ldb + i));
            cuda::mp_add(&sum, sum, mul);
        }
        C.exp[indexC] = sum.exp;
        C.sign[indexC] = sum.sign;
        C.eval[indexC] = sum.eval[0];
        C.eval[indexC + C.len[0]] = sum.eval[1];
        for (int i = 0; i < RNS_MODULI_SIZE; i++) C.digits[indexC * RNS_MODULI_SIZE + i] = sum.digits[i];
    }
}

} // namespace

extern "C" {

int ref_moduli_size() { return RNS_MODULI_SIZE; }
int ref_mp_float_size() { return (int)sizeof(mp_float_t); }

void ref_init() {
    rns_const_init();
    mp_const_init();
}

/* Every table rns_const_init()/mp_const_init() computes (src/rns.cuh:324-442,
 * src/arith/arith_utils.cuh:44-90), copied out of the device-side symbols. */
void ref_tables(int *part_inv, int *pow2, int *m_pow2_res, int *part_pow2_res, int *pow2_inv, double *recip_rd,
                double *recip_ru, int *mrc_inv, double *eval_acc, int *ref_factor, er_float_t *units,
                int *mp_consts) {
    const int N = RNS_MODULI_SIZE, T = RNS_P2_SCALING_THRESHOLD;
    memcpy(part_inv, cuda::RNS_PART_MODULI_PRODUCT_INVERSE, sizeof(int) * N);
    memcpy(pow2, cuda::RNS_POW2, sizeof(int) * N * (RNS_MODULI_PRODUCT_LOG2 + 1));
    memcpy(m_pow2_res, cuda::RNS_MODULI_PRODUCT_POW2_RESIDUES, sizeof(int) * T);
    memcpy(part_pow2_res, cuda::RNS_PART_MODULI_PRODUCT_POW2_RESIDUES, sizeof(int) * T * N);
    memcpy(pow2_inv, cuda::RNS_POW2_INVERSE, sizeof(int) * T * N);
    memcpy(recip_rd, cuda::RNS_MODULI_RECIP_RD, sizeof(double) * N);
    memcpy(recip_ru, cuda::RNS_MODULI_RECIP_RU, sizeof(double) * N);
    memcpy(mrc_inv, cuda::MRC_MULT_INV, sizeof(int) * N * N);
    *eval_acc = cuda::RNS_EVAL_ACCURACY;
    *ref_factor = cuda::RNS_EVAL_REF_FACTOR;
    units[0] = cuda::RNS_EVAL_UNIT.low;
    units[1] = cuda::RNS_EVAL_UNIT.upp;
    units[2] = cuda::RNS_EVAL_INV_UNIT.low;
    units[3] = cuda::RNS_EVAL_INV_UNIT.upp;
    mp_consts[0] = MP_PRECISION;
    mp_consts[1] = cuda::MP_H;
    mp_consts[2] = cuda::MP_J;
}

/* Host conversion double -> mp_float_t (src/arith/assign.cuh:54-81). */
void ref_set_d(const double *x, long n, mp_float_t *out) {
    for (long i = 0; i < n; i++) mp_set_d(&out[i], x[i]);
}

/* Element-wise device arithmetic (src/arith/{add,mul,muld}.cuh, namespace cuda). */
void ref_dev_add(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long n) {
    for (long i = 0; i < n; i++) cuda::mp_add(&r[i], x[i], y[i]);
}
void ref_dev_mul(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long n) {
    for (long i = 0; i < n; i++) cuda::mp_mul(&r[i], x[i], y[i]);
}
void ref_dev_mul_d(const mp_float_t *x, const double *y, mp_float_t *r, long n) {
    for (long i = 0; i < n; i++) cuda::mp_mul_d(&r[i], x[i], y[i]);
}
/* Host (CPU) arithmetic of the reference, for the timed CPU baseline. */
void ref_host_add(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long n) {
    for (long i = 0; i < n; i++) mp_add(&r[i], x[i], y[i]);
}
void ref_host_mul(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long n) {
    for (long i = 0; i < n; i++) mp_mul(&r[i], x[i], y[i]);
}
/* src/rns.cuh:878-933 */
void ref_dev_eval_fast(const int *digits, er_float_t *low, er_float_t *upp, long n) {
    for (long i = 0; i < n; i++) {
        int d[RNS_MODULI_SIZE];
        memcpy(d, digits + i * RNS_MODULI_SIZE, sizeof(d));
        cuda::rns_eval_compute_fast(&low[i], &upp[i], d);
    }
}
/* src/rns.cuh:797-868 */
void ref_dev_eval(const int *digits, er_float_t *low, er_float_t *upp, long n) {
    for (long i = 0; i < n; i++) {
        int d[RNS_MODULI_SIZE];
        memcpy(d, digits + i * RNS_MODULI_SIZE, sizeof(d));
        cuda::rns_eval_compute(&low[i], &upp[i], d);
    }
}
/* src/rns.cuh:1132-1160 */
void ref_dev_scale2pow(const int *digits, const unsigned *D, int *out, long n) {
    for (long i = 0; i < n; i++) {
        int d[RNS_MODULI_SIZE], r[RNS_MODULI_SIZE];
        memcpy(d, digits + i * RNS_MODULI_SIZE, sizeof(d));
        cuda::rns_scale2pow(r, d, D[i]);
        memcpy(out + i * RNS_MODULI_SIZE, r, sizeof(r));
    }
}

/* cuda::mp_dot<g1,b1,g2,g3,b3> (src/blas/dot.cuh:85-108), launch sequence transcribed. */
void ref_dot(int n, const mp_float_t *x, int incx, const mp_float_t *y, int incy, mp_float_t *r,
             int g1, int b1, int g2, int g3, int b3) {
    if (n <= 0) return;
    HostArray hx(stride_len(n, incx)), hy(stride_len(n, incy)), hr(1), hbuf(n);
    hx.load(x); hy.load(y); hr.load(r);
    int numThreadsXY = (incx == 1 && incy == 1) ? BLOCK_SIZE_FOR_RESIDUES : RNS_MODULI_SIZE;
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_mul_esi_kernel(hbuf.a, 1, hx.a, incx, hy.a, incy, n); }, false);
    emu::launch(dim3(g2), dim3(numThreadsXY), [&] { cuda::mp_vector_mul_digits_kernel(hbuf.a, 1, hx.a, incx, hy.a, incy, n); }, false);
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_round_kernel(hbuf.a, 1, n); }, false);
    reduce_sum(g3, b3, n, hbuf.a, hr.a);
    hr.store(r);
}

/* cuda::mp_gemv<g1,b1,g2,b3> (src/blas/gemv.cuh:151-269), launch sequence transcribed. */
void ref_gemv(int trans, int m, int n, const mp_float_t *alpha, const mp_float_t *A, int lda, const mp_float_t *x,
              int incx, const mp_float_t *beta, mp_float_t *y, int incy, int g1, int b1, int g2, int b3) {
    if ((m <= 0) || (n <= 0)) return;
    if ((incx == 0) || (incy == 0) || (lda < MAX(1, m))) return;
    const bool nt = (trans == mblas_no_trans);
    const int lx = nt ? n : m, ly = nt ? m : n;
    HostArray ha(lda * n), hx(stride_len(lx, incx)), hy(stride_len(ly, incy)), hal(1), hbe(1), hb1(lx), hb2(m * n);
    ha.load(A); hx.load(x); hy.load(y); hal.load(alpha); hbe.load(beta);
    dim3 grid1(g1, g1), grid2(g2, g2);
    int numThreadsX = (incx == 1) ? BLOCK_SIZE_FOR_RESIDUES : RNS_MODULI_SIZE;
    int numThreadsY = (incy == 1) ? BLOCK_SIZE_FOR_RESIDUES : RNS_MODULI_SIZE;
    const unsigned POW = nextPow2(b3);
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vec2scal_mul_esi_kernel(hb1.a, 1, hx.a, incx, hal.a, lx); }, false);
    emu::launch(dim3(g2), dim3(numThreadsX), [&] { cuda::mp_vec2scal_mul_digits_kernel(hb1.a, 1, hx.a, incx, hal.a, lx); }, false);
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_round_kernel(hb1.a, 1, lx); }, false);
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vec2scal_mul_esi_kernel(hy.a, incy, hy.a, incy, hbe.a, ly); }, false);
    emu::launch(dim3(g2), dim3(numThreadsY), [&] { cuda::mp_vec2scal_mul_digits_kernel(hy.a, incy, hy.a, incy, hbe.a, ly); }, false);
    emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_round_kernel(hy.a, incy, ly); }, false);
    if (nt) {
        emu::launch(grid1, dim3(b1), [&] { cuda::mp_mat2vec_right_scal_esi_kernel(hb2.a, m, ha.a, lda, hb1.a, 1, m, n); }, false);
        emu::launch(grid2, dim3(BLOCK_SIZE_FOR_RESIDUES), [&] { cuda::mp_mat2vec_right_scal_digits_kernel(hb2.a, m, ha.a, lda, hb1.a, 1, m, n); }, false);
        emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_round_kernel(hb2.a, 1, m * n); }, false);
        emu::launch(dim3(m), dim3(b3), [&] { matrix_row_sum(m, n, hb2.a, hy.a, incy, POW); }, true);
    } else {
        emu::launch(grid1, dim3(b1), [&] { cuda::mp_mat2vec_left_scal_esi_kernel(hb2.a, m, ha.a, lda, hb1.a, 1, m, n); }, false);
        emu::launch(grid2, dim3(BLOCK_SIZE_FOR_RESIDUES), [&] { cuda::mp_mat2vec_left_scal_digits_kernel(hb2.a, m, ha.a, lda, hb1.a, 1, m, n); }, false);
        emu::launch(dim3(g1), dim3(b1), [&] { cuda::mp_vector_round_kernel(hb2.a, 1, m * n); }, false);
        emu::launch(dim3(n), dim3(b3), [&] { matrix_col_sum(m, n, hb2.a, hy.a, incy, POW); }, true);
    }
    hy.store(y);
}

/* cuda::mp_gemm<b1x,b1y,g2x,g2y,b3> NN case (src/blas/gemm.cuh:70-168), launch sequence transcribed. */
void ref_gemm(int m, int n, int k, const mp_float_t *alpha, const mp_float_t *A, int lda, const mp_float_t *B,
              int ldb, const mp_float_t *beta, mp_float_t *C, int ldc, int b1x, int b1y, int g2x, int g2y, int b3) {
    if ((m <= 0) || (n <= 0) || (k <= 0)) return;
    if (lda < MAX(1, m) || ldb < MAX(1, k) || ldc < MAX(1, m)) return;
    HostArray ha(lda * k), hb(ldb * n), hc(ldc * n), hal(1), hbe(1), hbuf(m * n);
    ha.load(A); hb.load(B); hc.load(C); hal.load(alpha); hbe.load(beta);
    {
        dim3 block(b3, b3), grid((n + b3 - 1) / b3, (m + b3 - 1) / b3);
        emu::launch(grid, block, [&] { matrix_multiply_notrans(m, n, k, ha.a, lda, hb.a, ldb, hbuf.a, m); }, false);
    }
    dim3 block1(b1x, b1y), grid1((m + b1x - 1) / b1x, (n + b1y - 1) / b1y), grid2(g2x, g2y);
    dim3 block3(16, 16), grid3((m + 15) / 16, (n + 15) / 16);
    emu::launch(grid1, block1, [&] { cuda::mp_mat2scal_mul_esi_kernel(hbuf.a, m, hbuf.a, m, hal.a, m, n); }, false);
    emu::launch(grid2, dim3(BLOCK_SIZE_FOR_RESIDUES), [&] { cuda::mp_mat2scal_mul_digits_kernel(hbuf.a, m, hbuf.a, m, hal.a, m, n); }, false);
    emu::launch(grid3, block3, [&] { cuda::mp_matrix_round_kernel(hbuf.a, m, m, n); }, false);
    emu::launch(grid1, block1, [&] { cuda::mp_mat2scal_mul_esi_kernel(hc.a, ldc, hc.a, ldc, hbe.a, m, n); }, false);
    emu::launch(grid2, dim3(BLOCK_SIZE_FOR_RESIDUES), [&] { cuda::mp_mat2scal_mul_digits_kernel(hc.a, ldc, hc.a, ldc, hbe.a, m, n); }, false);
    emu::launch(grid3, block3, [&] { cuda::mp_matrix_round_kernel(hc.a, ldc, m, n); }, false);
    emu::launch(grid1, block1, [&] { cuda::mp_matrix_add_esi_kernel(hc.a, ldc, hc.a, ldc, hbuf.a, m, m, n); }, false);
    emu::launch(grid2, dim3(BLOCK_SIZE_FOR_RESIDUES), [&] { cuda::mp_matrix_add_digits_kernel(hc.a, ldc, hc.a, ldc, hbuf.a, m, m, n); }, false);
    emu::launch(grid3, block3, [&] { cuda::mp_matrix_round_kernel(hc.a, ldc, m, n); }, false);
    hc.store(C);
}

/* cuda::mp_spmv_csr<32> (src/sparse/spmv/spmv_csr.cuh:49-63), run as written;
 * launch shape of tests/sparse/spmv/csr/test_mpres_spmv_csr.cuh:39-40. */
void ref_spmv_csr(int m, const int *irp, const int *ja, const double *as, const mp_float_t *x, mp_float_t *y) {
    csr_t csr;
    csr.irp = (int *)irp; csr.ja = (int *)ja; csr.as = (double *)as;
    mp_float_ptr px = (mp_float_ptr)x;
    emu::launch(dim3(m / 32 + 1), dim3(32), [&] { cuda::mp_spmv_csr<32>(m, csr, px, y); }, false);
}

/* cuda::mp_spmv_csrv<32,tpr> (src/sparse/spmv/spmv_csrv.cuh:49-86), transcribed: the kernel's lane tree has no
 * barrier and relies on lock-step lanes, which a coroutine emulation does not give. */
void ref_spmv_csrv(int m, int tpr, const int *irp, const int *ja, const double *as, const mp_float_t *x,
                   mp_float_t *y) {
    std::vector<mp_float_t> sums(tpr), prods(tpr);
    for (int row = 0; row < m; row++) {
        int row_start = irp[row], row_end = irp[row + 1];
        for (int lane = 0; lane < tpr; lane++) {
            sums[lane] = cuda::MP_ZERO;
            for (int i = row_start + lane; i < row_end; i += tpr) {
                cuda::mp_mul_d(&prods[lane], x[ja[i]], as[i]);
                cuda::mp_add(&sums[lane], sums[lane], prods[lane]);
            }
        }
        for (int s = 16; s >= 1; s >>= 1)
            if (tpr >= 2 * s)
                for (int lane = 0; lane < s; lane++) cuda::mp_add(&sums[lane], sums[lane], sums[lane + s]);
        cuda::mp_set(&y[row], sums[0]);
    }
}

/* cuda::mp_spmv_ell<32> (src/sparse/spmv/spmv_ell.cuh:50-67), run as written;
 * launch shape of tests/sparse/spmv/ell/test_mpres_spmv_ell.cuh:39-40. */
void ref_spmv_ell(int m, int maxnzr, const int *ja, const double *as, const mp_float_t *x, mp_float_t *y) {
    ell_t ell;
    ell.ja = (int *)ja; ell.as = (double *)as;
    mp_float_ptr px = (mp_float_ptr)x;
    emu::launch(dim3(m / 32 + 1), dim3(32), [&] { cuda::mp_spmv_ell<32>(m, maxnzr, ell, px, y); }, false);
}

/* ::mp_div, ::mp_sqrt, ::mp_dsqrt (src/arith/div.cuh:33-45, src/arith/sqrt.cuh),
 * host functions on MPFR, called as written, element by element. */
void ref_div(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long count) {
    for (long i = 0; i < count; i++) {
        mp_float_t a = x[i], b = y[i];
        ::mp_div(&r[i], &a, &b);
    }
}
void ref_sqrt(const mp_float_t *x, mp_float_t *r, long count) {
    for (long i = 0; i < count; i++) {
        mp_float_t a = x[i];
        ::mp_sqrt(&r[i], &a);
    }
}
void ref_dsqrt(const mp_float_t *x, double *r, long count) {
    for (long i = 0; i < count; i++) {
        mp_float_t a = x[i];
        r[i] = ::mp_dsqrt(&a);
    }
}

/* cuda::mp_add_abs (src/arith/addabs.cuh:118-127), element by element */
void ref_add_abs(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, long count) {
    for (long i = 0; i < count; i++) cuda::mp_add_abs(&r[i], x[i], y[i]);
}

/* mp_sumsq_kernel1/2 of cuda::mp_norm2<blocks, threads> (src/blas/v2/norm2_v2.cuh:39-112)
 * and mp_dot_kernel1/2 of cuda::mp_dot<blocks, threads> (src/blas/v2/dot_v2.cuh),
 * transcribed with one block's shared array at a time: the kernels keep their
 * partial sums in static __shared__ arrays, which the coroutine launcher cannot
 * share.  The arithmetic is the reference's device functions. */
static void v2_reduce(bool sumsq, int n, const mp_float_t *x, const mp_float_t *y, mp_float_t *r, int blocks,
                      int threads) {
    const unsigned POW = nextPow2(threads);
    std::vector<mp_float_t> parts(blocks), sdata(threads);
    mp_float_t prod;
    auto add = [&](mp_float_t *d, const mp_float_t &a, const mp_float_t &b) {
        if (sumsq) cuda::mp_add_abs(d, a, b);
        else cuda::mp_add(d, a, b);
    };
    auto tree = [&](int bsize) {
        for (unsigned i = POW >> 1; i >= 1; i >>= 1)
            for (unsigned tid = 0; tid < i; tid++)
                if (tid + i < (unsigned)bsize) add(&sdata[tid], sdata[tid], sdata[tid + i]);
    };
    const unsigned k = (unsigned)blocks * threads;
    for (int bid = 0; bid < blocks; bid++) {
        for (int tid = 0; tid < threads; tid++) {
            sdata[tid] = cuda::MP_ZERO;
            for (unsigned i = bid * threads + tid; i < (unsigned)n; i += k) {
                cuda::mp_mul(&prod, x[i], sumsq ? x[i] : y[i]);
                add(&sdata[tid], sdata[tid], prod);
            }
        }
        tree(threads);
        parts[bid] = sdata[0];
    }
    for (int tid = 0; tid < threads; tid++) {
        sdata[tid] = cuda::MP_ZERO;
        for (unsigned i = tid; i < (unsigned)blocks; i += threads) add(&sdata[tid], sdata[tid], parts[i]);
    }
    tree(threads);
    r[0] = sdata[0];
}

void ref_reduce_v2(int sumsq, int n, const mp_float_t *x, const mp_float_t *y, mp_float_t *r, int blocks, int threads) {
    v2_reduce(sumsq != 0, n, x, y, r, blocks, threads);
}

/* mp_cg_csr / mp_pcg_csr (src/sparse/solver/cg_csr.cuh, pcg_csr.cuh) with the
 * launch sequence transcribed: mp_spmv_csr runs as written; the v2 vector
 * kernels (diff, axpy, maxpy, prod_d: one device function per element) and the
 * reductions are transcribed as above; mp_div and mp_dsqrt are the reference's
 * host MPFR functions.  M == nullptr: plain CG. */
int ref_cg_csr(int n, const int *irp, const int *ja, const double *as, const mp_float_t *b, double tol, int maxit,
               const double *M, mp_float_t *x, double *resvec, int cap, int threads, int blocks_reduce) {
    std::vector<mp_float_t> r(n), p(n), q(n), z(n);
    mp_float_t rho = cuda::MP_ZERO, rhop, alpha, beta, pq, nrm;
    csr_t A;
    A.irp = (int *)irp; A.ja = (int *)ja; A.as = (double *)as;
    auto spmv = [&](mp_float_t *in, mp_float_t *out) {
        emu::launch(dim3(n / threads + 1), dim3(threads), [&] {
            if (threads == 32) cuda::mp_spmv_csr<32>(n, A, in, out);
            else cuda::mp_spmv_csr<64>(n, A, in, out);
        }, false);
    };
    auto norm2 = [&](const mp_float_t *v) {
        v2_reduce(true, n, v, v, &nrm, blocks_reduce, threads);
        return ::mp_dsqrt(&nrm);
    };
    spmv(x, r.data());
    for (int i = 0; i < n; i++) cuda::mp_sub(&r[i], b[i], r[i]);
    const double norm0 = norm2(r.data());
    const double eps = norm0 * tol;
    double normk = norm0;
    int nres = 0, k = 0;
    if (nres < cap) resvec[nres] = normk / norm0;
    nres++;
    mp_float_t *zz = M ? z.data() : r.data();
    while (normk > eps && k < maxit) {
        if (M)
            for (int i = 0; i < n; i++) cuda::mp_mul_d(&z[i], r[i], M[i]);
        rhop = rho;
        v2_reduce(false, n, r.data(), zz, &rho, blocks_reduce, threads);
        if (k == 0) {
            for (int i = 0; i < n; i++) p[i] = zz[i];
        } else {
            ::mp_div(&beta, &rho, &rhop);
            for (int i = 0; i < n; i++) {
                mp_float_t ax;
                cuda::mp_mul(&ax, beta, p[i]);
                cuda::mp_add(&p[i], ax, zz[i]);
            }
        }
        spmv(p.data(), q.data());
        v2_reduce(false, n, p.data(), q.data(), &pq, blocks_reduce, threads);
        ::mp_div(&alpha, &rho, &pq);
        for (int i = 0; i < n; i++) {
            mp_float_t ax;
            cuda::mp_mul(&ax, alpha, p[i]);
            cuda::mp_add(&x[i], ax, x[i]);
        }
        mp_float_t malpha = alpha;
        malpha.sign = malpha.sign ^ 1;
        for (int i = 0; i < n; i++) {
            mp_float_t ax;
            cuda::mp_mul(&ax, malpha, q[i]);
            cuda::mp_add(&r[i], ax, r[i]);
        }
        normk = norm2(r.data());
        if (nres < cap) resvec[nres] = normk / norm0;
        nres++;
        k++;
    }
    return k;
}

/* The Matrix Market reader, src/sparse/utils/mtx_reader.cuh:52-101, :249-253,
 * :374-406, called as written.  out = {m, n, lines, maxnzr, nzmd, symmetric}. */
void ref_mtx_stats(const char *path, int *out) {
    int m, n, lines, maxnzr, nzmd;
    bool sym;
    std::string dtype;
    collect_mtx_stats(path, m, n, lines, maxnzr, nzmd, sym, dtype);
    out[0] = m; out[1] = n; out[2] = lines; out[3] = maxnzr; out[4] = nzmd; out[5] = sym;
}
void ref_mtx_csr(const char *path, int m, int nnz, int lines, int symmetric, double *as, int *ja, int *irp) {
    csr_t csr;
    csr.as = as; csr.ja = ja; csr.irp = irp;
    build_csr(path, m, nnz, lines, symmetric != 0, csr);
}
void ref_mtx_ell(const char *path, int m, int maxnzr, int lines, int symmetric, double *as, int *ja) {
    ell_t ell;
    ell.as = as; ell.ja = ja;
    build_ell(path, m, maxnzr, lines, symmetric != 0, ell);
}

} // extern "C"
