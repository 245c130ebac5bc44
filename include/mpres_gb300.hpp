/*
 * Drop-in C++ interface for code written against MPRES-BLAS's hot path.
 *
 * Reference code includes src/params.h (a moduli set), src/mparray.cuh,
 * src/blas/{dot,gemv,gemm}.cuh and src/sparse/spmv/*.cuh and calls the names
 * below.  Including this header instead (after defining RNS_MODULI_SIZE, or
 * including the reference's params.h) gives the same names, template
 * parameters and argument lists, implemented by libmpres_gb300.so:
 *
 *   rns_const_init(), mp_const_init()                 src/rns.cuh:324, src/arith/arith_utils.cuh:44
 *   cuda::mp_array_init/clear/host2device/device2host src/mparray.cuh:35-160
 *   cuda::mp_dot<g1,b1,g2,g3,b3>(...)                 src/blas/dot.cuh:84-85
 *   cuda::mp_gemv<g1,b1,g2,b3>(...)                   src/blas/gemv.cuh:150-152
 *   cuda::mp_gemm<b1x,b1y,g2x,g2y,b3>(...)            src/blas/gemm.cuh:69-70
 *   cuda::csr_init/csr_host2device/csr_clear          src/sparse/utils/csr_utils.cuh:58-78
 *   cuda::ell_init/ell_host2device/ell_clear          src/sparse/utils/ell_utils.cuh:55-71
 *   cuda::mp_spmv_csr<threads>, mp_spmv_csrv<threads,tpr>, mp_spmv_ell<threads>
 *                                                     src/sparse/spmv/spmv_{csr,csrv,ell}.cuh
 *   cuda::mp_diff/mp_axpy/mp_maxpy, cuda::mp_dot<blocks,threads>, cuda::mp_norm2<blocks,threads>
 *                                                     src/blas/v2/{diff,axpy,maxpy,dot,norm2}_v2.cuh
 *   mp_cg_csr<threads,blocks>, mp_pcg_csr<threads,blocks>  src/sparse/solver/{cg,pcg}_csr.cuh
 *   ::mp_div, ::mp_sqrt, ::mp_dsqrt, cuda::mp_div, cuda::mp_dsqrt  src/arith/{div,sqrt}.cuh
 *   collect_mtx_stats, build_csr, build_ell           src/sparse/utils/mtx_reader.cuh
 *
 * The reference's SpMV routines are kernels the caller launches with
 * <<<blocks, threads>>>; here they are host functions taking the same
 * arguments, so `cuda::mp_spmv_csr<32><<<b, t>>>(m, csr, x, y)` becomes
 * `cuda::mp_spmv_csr<32>(m, csr, x, y)`.  Like the reference, the void
 * functions report failures on stderr and return; the mpres_* C functions of
 * mpres_gb300.h return a status instead.  Work is queued on the default stream.
 */
#ifndef MPRES_GB300_HPP
#define MPRES_GB300_HPP

#include <cstdio>
#include <string>
#include <vector>

#include "mpres_gb300.h"

#ifndef RNS_MODULI_SIZE
#error "define RNS_MODULI_SIZE (8, 16 or 32) or include the reference's params.h first"
#endif

#ifndef MPRES_TYPES_CUH
#define MPRES_TYPES_CUH
/* mp_float_t of src/types.cuh:69-74 */
typedef struct {
    int digits[RNS_MODULI_SIZE];
    int sign;
    int exp;
    er_float_t eval[2];
} mp_float_t;
typedef mp_float_t *mp_float_ptr;
typedef er_float_t *er_float_ptr;
#endif

#ifndef MPRES_MBLAS_ENUM_CUH
#define MPRES_MBLAS_ENUM_CUH
enum mblas_trans_type { mblas_no_trans = 111, mblas_trans = 112, mblas_conj_trans = 113 };
#endif

namespace mpres_detail {
inline void report(int status, const char *what) {
    if (status != MPRES_SUCCESS) std::fprintf(stderr, "%s: %s\n", what, mpres_last_error());
}
} // namespace mpres_detail

inline void rns_const_init() { mpres_detail::report(mpres_init(RNS_MODULI_SIZE), "rns_const_init"); }
inline void mp_const_init() { mpres_detail::report(mpres_init(RNS_MODULI_SIZE), "mp_const_init"); }

namespace cuda {

inline void mp_array_init(mp_array_t &dev_dest, size_t size) {
    mpres_detail::report(mpres_array_init(RNS_MODULI_SIZE, &dev_dest, size), "mp_array_init");
}
inline void mp_array_clear(mp_array_t &dev_dest) {
    mpres_detail::report(mpres_array_clear(&dev_dest), "mp_array_clear");
}
inline void mp_array_host2device(mp_array_t &dev_dest, mp_float_ptr host_src, size_t size) {
    mpres_detail::report(mpres_array_host2device(RNS_MODULI_SIZE, &dev_dest, host_src, size), "mp_array_host2device");
}
inline void mp_array_device2host(mp_float_ptr host_dest, mp_array_t &dev_src, size_t size) {
    mpres_detail::report(mpres_array_device2host(RNS_MODULI_SIZE, host_dest, &dev_src, size), "mp_array_device2host");
}

template <int gridDim1, int blockDim1, int gridDim2, int gridDim3, int blockDim3>
void mp_dot(const int n, mp_array_t &x, const int incx, mp_array_t &y, const int incy, mp_array_t &r,
            mp_array_t &buffer) {
    mpres_detail::report(mpres_dot(RNS_MODULI_SIZE, n, &x, incx, &y, incy, &r, &buffer, gridDim1, blockDim1,
                                   gridDim2, gridDim3, blockDim3, nullptr),
                         "mp_dot");
}

template <int gridDim1, int blockDim1, int gridDim2, int blockDim3>
void mp_gemv(enum mblas_trans_type trans, const int m, const int n, mp_array_t &alpha, mp_array_t &A, const int lda,
             mp_array_t &x, const int incx, mp_array_t &beta, mp_array_t &y, const int incy, mp_array_t &buffer1,
             mp_array_t &buffer2) {
    mpres_detail::report(mpres_gemv(RNS_MODULI_SIZE, (int)trans, m, n, &alpha, &A, lda, &x, incx, &beta, &y, incy,
                                    &buffer1, &buffer2, gridDim1, blockDim1, gridDim2, blockDim3, nullptr),
                         "mp_gemv");
}

template <int blockDim1x, int blockDim1y, int gridDim2x, int gridDim2y, int blockDim3>
void mp_gemm(enum mblas_trans_type transa, enum mblas_trans_type transb, const int m, const int n, const int k,
             mp_array_t &alpha, mp_array_t &A, const int lda, mp_array_t &B, const int ldb, mp_array_t &beta,
             mp_array_t &C, const int ldc, mp_array_t &buffer) {
    int st = mpres_gemm(RNS_MODULI_SIZE, (int)transa, (int)transb, m, n, k, &alpha, &A, lda, &B, ldb, &beta, &C, ldc,
                        &buffer, blockDim1x, blockDim1y, gridDim2x, gridDim2y, blockDim3, nullptr);
    if (st == MPRES_ERR_NOT_SUPPORTED) std::printf("\nOnly non-transposed matrices are currently supported.");
    else mpres_detail::report(st, "mp_gemm");
}

inline void csr_init(csr_t &csr, const int m, const int nnz) {
    mpres_detail::report(mpres_csr_init(&csr, m, nnz), "csr_init");
}
inline void csr_clear(csr_t &csr) { mpres_detail::report(mpres_csr_clear(&csr), "csr_clear"); }
inline void csr_host2device(csr_t &csr_dev, const csr_t &csr_host, const int m, const int nnz) {
    mpres_detail::report(mpres_csr_host2device(&csr_dev, &csr_host, m, nnz), "csr_host2device");
}
inline void ell_init(ell_t &ell, const int m, const int maxnzr) {
    mpres_detail::report(mpres_ell_init(&ell, m, maxnzr), "ell_init");
}
inline void ell_clear(ell_t &ell) { mpres_detail::report(mpres_ell_clear(&ell), "ell_clear"); }
inline void ell_host2device(ell_t &ell_dev, const ell_t &ell_host, const int m, const int maxnzr) {
    mpres_detail::report(mpres_ell_host2device(&ell_dev, &ell_host, m, maxnzr), "ell_host2device");
}

template <int threads> void mp_spmv_csr(const int m, const csr_t csr, mp_float_ptr x, mp_float_ptr y) {
    mpres_detail::report(mpres_spmv_csr(RNS_MODULI_SIZE, m, &csr, x, y, threads, nullptr), "mp_spmv_csr");
}
template <int threads, int threadsPerRow>
void mp_spmv_csrv(const int m, const csr_t csr, mp_float_ptr x, mp_float_ptr y) {
    mpres_detail::report(mpres_spmv_csrv(RNS_MODULI_SIZE, m, &csr, x, y, threads, threadsPerRow, nullptr),
                         "mp_spmv_csrv");
}
template <int threads> void mp_spmv_ell(const int m, const int maxnzr, const ell_t ell, mp_float_ptr x, mp_float_ptr y) {
    mpres_detail::report(mpres_spmv_ell(RNS_MODULI_SIZE, m, maxnzr, &ell, x, y, threads, nullptr), "mp_spmv_ell");
}

/* v2 vector kernels (src/blas/v2/*_v2.cuh): host functions with the kernels' arguments */
inline void mp_diff(const int n, mp_float_ptr x, mp_float_ptr y, mp_float_ptr r) {
    mpres_detail::report(mpres_v2_diff(RNS_MODULI_SIZE, n, x, y, r, 32, nullptr), "mp_diff");
}
inline void mp_axpy(const int n, mp_float_ptr alpha, mp_float_ptr x, mp_float_ptr y, mp_float_ptr r) {
    mpres_detail::report(mpres_v2_axpy(RNS_MODULI_SIZE, n, alpha, x, y, r, 32, nullptr), "mp_axpy");
}
inline void mp_maxpy(const int n, mp_float_ptr alpha, mp_float_ptr x, mp_float_ptr y, mp_float_ptr r) {
    mpres_detail::report(mpres_v2_maxpy(RNS_MODULI_SIZE, n, alpha, x, y, r, 32, nullptr), "mp_maxpy");
}
template <int blocks, int threads> void mp_dot(const int n, mp_float_ptr x, mp_float_ptr y, mp_float_ptr r) {
    mpres_detail::report(mpres_v2_dot(RNS_MODULI_SIZE, n, x, y, r, blocks, threads, nullptr), "mp_dot");
}
template <int blocks, int threads> double mp_norm2(const int n, mp_float_ptr x) {
    double v = 0;
    mpres_detail::report(mpres_v2_norm2(RNS_MODULI_SIZE, n, x, &v, blocks, threads, nullptr), "mp_norm2");
    return v;
}
/* src/arith/div.cuh:56-65, src/arith/sqrt.cuh: device records, host computation */
inline void mp_div(mp_float_ptr result, mp_float_ptr x, mp_float_ptr y) {
    mpres_detail::report(mpres_div_device(RNS_MODULI_SIZE, x, y, result), "mp_div");
}
inline double mp_dsqrt(mp_float_ptr x) {
    double v = 0;
    mpres_detail::report(mpres_dsqrt_device(RNS_MODULI_SIZE, x, &v), "mp_dsqrt");
    return v;
}

} // namespace cuda

/* host MPFR operations (src/arith/div.cuh:33-45, src/arith/sqrt.cuh) */
inline void mp_div(mp_float_ptr result, mp_float_ptr x, mp_float_ptr y) {
    mpres_detail::report(mpres_div(RNS_MODULI_SIZE, x, y, result), "mp_div");
}
inline void mp_sqrt(mp_float_ptr result, mp_float_ptr x) {
    mpres_detail::report(mpres_sqrt(RNS_MODULI_SIZE, x, result), "mp_sqrt");
}
inline double mp_dsqrt(mp_float_ptr x) {
    double v = 0;
    mpres_detail::report(mpres_dsqrt(RNS_MODULI_SIZE, x, &v), "mp_dsqrt");
    return v;
}

/* conjugate gradients (src/sparse/solver/cg_csr.cuh, pcg_csr.cuh); resvec is
 * appended to, as in the reference */
#ifndef MPRES_MSPARSE_ENUM_CUH
#define MPRES_MSPARSE_ENUM_CUH
enum preconditioner_type { diag = 1 };
#endif
template <int threads = 32, int blocks_reduce = 256>
int mp_cg_csr(const int n, const csr_t &A, mp_float_ptr b, const double tol, const int maxit, mp_float_ptr x,
              std::vector<double> &resvec) {
    std::vector<double> res((size_t)maxit + 1);
    int k = 0;
    mpres_detail::report(mpres_cg_csr(RNS_MODULI_SIZE, n, &A, b, tol, maxit, x, res.data(), (int)res.size(), &k,
                                      threads, blocks_reduce, nullptr), "mp_cg_csr");
    resvec.insert(resvec.end(), res.begin(), res.begin() + k + 1);
    return k;
}
template <int threads = 64, int blocks_reduce = 256>
int mp_pcg_csr(const int n, const csr_t &A, mp_float_ptr b, const double tol, const int maxit,
               enum preconditioner_type ptype, double *M, mp_float_ptr x, std::vector<double> &resvec) {
    std::vector<double> res((size_t)maxit + 1);
    int k = 0;
    mpres_detail::report(mpres_pcg_csr(RNS_MODULI_SIZE, n, &A, b, tol, maxit, (int)ptype, M, x, res.data(),
                                       (int)res.size(), &k, threads, blocks_reduce, nullptr), "mp_pcg_csr");
    resvec.insert(resvec.end(), res.begin(), res.begin() + k + 1);
    return k;
}

/* src/sparse/utils/mtx_reader.cuh:52, :249, :374 (global functions in the reference) */
inline void collect_mtx_stats(const char *filename, int &m, int &n, int &lines, int &maxnzr, int &nzmd,
                              bool &symmetric, std::string &datatype) {
    int sym = 0;
    char dt[16] = {0};
    mpres_detail::report(mpres_mtx_stats(filename, &m, &n, &lines, &maxnzr, &nzmd, &sym, dt), "collect_mtx_stats");
    symmetric = sym != 0;
    datatype = dt;
}
inline void build_csr(const char filename[], const int m, const int nnz, const int lines, const bool symmetric,
                      csr_t &csr) {
    mpres_detail::report(mpres_mtx_build_csr(filename, m, nnz, lines, symmetric, csr.as, csr.ja, csr.irp),
                         "build_csr");
}
inline void build_ell(const char filename[], const int m, const int maxnzr, const int lines, const bool symmetric,
                      ell_t &ell) {
    mpres_detail::report(mpres_mtx_build_ell(filename, m, maxnzr, lines, symmetric, ell.as, ell.ja), "build_ell");
}

#endif
