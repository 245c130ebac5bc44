/*
 * The reference's CPU path for the benchmark workloads: its MPFR loops with
 * OpenMP, restated in C.  TEST AND BENCHMARK INFRASTRUCTURE ONLY (the CPU
 * baseline timed beside the GPU, and an MPFR cross-check); never part of the
 * product.
 *
 *   mpb_dot        tests/blas/performance/test_dot_performance.cu:152-174
 *                  (mpfr_dot: per-thread partial sums over an omp-for split,
 *                  then a critical section adds them to the result)
 *   mpb_gemm       tests/blas/v2/gemm/test_mpfr_gemm.cuh:29-60 (mpfr_gemm, NN:
 *                  rows split by omp for, one sequential k sum per output, then
 *                  C = alpha*dot + beta*C)
 *   mpb_spmv_csr   tests/sparse/spmv/csr/test_mpfr_spmv_csr.cuh:33-51
 *                  (mpfr_mpspmv_csr: rows split by omp for, mpfr_mul_d + add)
 *
 * Every operation rounds to nearest at `prec` bits; the reference runs these at
 * MP_PRECISION (src/arith/arith_utils.cuh:50: floor(log2 M)/2 - 1, i.e. 120,
 * 240 and 480 bits for 8, 16 and 32 moduli).  Inputs are the benchmark's
 * doubles, converted with mpfr_set_d outside the timed loop as the reference's
 * drivers convert them before their timers start.  Each entry point returns the
 * wall time of its loop in seconds (omp_get_wtime) and the results rounded to
 * double (for checks).  MPFR comes from the runtime library libmpfr.so.6; the
 * declarations are those of ref/shim/mpfr.h (written from the MPFR manual).
 */
#include <stdlib.h>

#include <omp.h>

#include "ref/shim/mpfr.h"

static mpfr_t *mp_vec(const double *v, long n, long prec) {
    mpfr_t *a = (mpfr_t *)malloc(sizeof(mpfr_t) * (size_t)(n > 0 ? n : 1));
    if (!a) return NULL;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        mpfr_init2(a[i], prec);
        mpfr_set_d(a[i], v ? v[i] : 0.0, MPFR_RNDN);
    }
    return a;
}

static void mp_free(mpfr_t *a, long n) {
    if (!a) return;
    for (long i = 0; i < n; i++) mpfr_clear(a[i]);
    free(a);
}

int mpb_max_threads(void) { return omp_get_max_threads(); }

/* result = sum x_i * y_i (mpfr_dot); *out the result rounded to double */
double mpb_dot(int n, const double *x, const double *y, long prec, int threads, double *out) {
    mpfr_t *mx = mp_vec(x, n, prec), *my = mp_vec(y, n, prec);
    mpfr_t result;
    mpfr_init2(result, prec);
    mpfr_set_d(result, 0, MPFR_RNDN);
    const double t0 = omp_get_wtime();
#pragma omp parallel num_threads(threads) shared(result)
    {
        mpfr_t tmp_sum, tmp;
        mpfr_init2(tmp_sum, prec);
        mpfr_init2(tmp, prec);
        mpfr_set_d(tmp_sum, 0, MPFR_RNDN);
        mpfr_set_d(tmp, 0, MPFR_RNDN);
#pragma omp for
        for (int i = 0; i < n; i++) {
            mpfr_mul(tmp, mx[i], my[i], MPFR_RNDN);
            mpfr_add(tmp_sum, tmp_sum, tmp, MPFR_RNDN);
        }
#pragma omp critical
        mpfr_add(result, result, tmp_sum, MPFR_RNDN);
        mpfr_clear(tmp);
        mpfr_clear(tmp_sum);
    }
    const double t = omp_get_wtime() - t0;
    if (out) *out = mpfr_get_d(result, MPFR_RNDN);
    mpfr_clear(result);
    mp_free(mx, n);
    mp_free(my, n);
    return t;
}

/* C(0:rows, 0:cols) = alpha * A(0:rows, :) * B(:, 0:cols) + beta * C(0:rows, 0:cols)
 * for column-major A (lda), B (ldb), C (ldc), k the inner dimension (mpfr_gemm,
 * NN); out (rows x cols, column-major with leading dimension rows) receives C
 * rounded to double when non-null */
double mpb_gemm(int rows, int cols, int k, double alpha, const double *A, int lda, const double *B, int ldb,
                double beta, const double *C, int ldc, long prec, int threads, double *out) {
    /* only the operand block the sample touches is converted */
    double *a = (double *)malloc(sizeof(double) * (size_t)rows * k);
    double *b = (double *)malloc(sizeof(double) * (size_t)k * cols);
    double *c = (double *)malloc(sizeof(double) * (size_t)rows * cols);
    if (!a || !b || !c) {
        free(a); free(b); free(c);
        return -1.0;
    }
    for (int i = 0; i < k; i++)
        for (int r = 0; r < rows; r++) a[(size_t)i * rows + r] = A[(size_t)i * lda + r];
    for (int j = 0; j < cols; j++)
        for (int i = 0; i < k; i++) b[(size_t)j * k + i] = B[(size_t)j * ldb + i];
    for (int j = 0; j < cols; j++)
        for (int r = 0; r < rows; r++) c[(size_t)j * rows + r] = C[(size_t)j * ldc + r];
    mpfr_t *mA = mp_vec(a, (long)rows * k, prec), *mB = mp_vec(b, (long)k * cols, prec);
    mpfr_t *mC = mp_vec(c, (long)rows * cols, prec);
    mpfr_t mal, mbe;
    mpfr_init2(mal, prec);
    mpfr_init2(mbe, prec);
    mpfr_set_d(mal, alpha, MPFR_RNDN);
    mpfr_set_d(mbe, beta, MPFR_RNDN);
    const double t0 = omp_get_wtime();
#pragma omp parallel num_threads(threads)
    {
        mpfr_t dot, prod;
        mpfr_init2(dot, prec);
        mpfr_init2(prod, prec);
#pragma omp for
        for (int row = 0; row < rows; row++) {
            for (int col = 0; col < cols; col++) {
                mpfr_set_d(dot, 0.0, MPFR_RNDN);
                for (int i = 0; i < k; i++) {
                    mpfr_mul(prod, mA[(size_t)i * rows + row], mB[(size_t)col * k + i], MPFR_RNDN);
                    mpfr_add(dot, dot, prod, MPFR_RNDN);
                }
                mpfr_mul(dot, dot, mal, MPFR_RNDN);
                mpfr_mul(prod, mbe, mC[(size_t)col * rows + row], MPFR_RNDN);
                mpfr_add(mC[(size_t)col * rows + row], dot, prod, MPFR_RNDN);
            }
        }
        mpfr_clear(dot);
        mpfr_clear(prod);
    }
    const double t = omp_get_wtime() - t0;
    if (out)
        for (long i = 0; i < (long)rows * cols; i++) out[i] = mpfr_get_d(mC[i], MPFR_RNDN);
    mpfr_clear(mal);
    mpfr_clear(mbe);
    mp_free(mA, (long)rows * k);
    mp_free(mB, (long)k * cols);
    mp_free(mC, (long)rows * cols);
    free(a); free(b); free(c);
    return t;
}

/* y = A * x over rows [0, m) of a CSR matrix (mpfr_mpspmv_csr); x has n entries;
 * out (m entries) receives y rounded to double when non-null */
double mpb_spmv_csr(int m, int n, const int *irp, const int *ja, const double *as, const double *x, long prec,
                    int threads, double *out) {
    mpfr_t *mx = mp_vec(x, n, prec), *my = mp_vec(NULL, m, prec);
    const double t0 = omp_get_wtime();
#pragma omp parallel num_threads(threads)
    {
        mpfr_t prod;
        mpfr_init2(prod, prec);
#pragma omp for
        for (int row = 0; row < m; row++) {
            mpfr_set_d(my[row], 0.0, MPFR_RNDN);
            for (int i = irp[row]; i < irp[row + 1]; i++) {
                mpfr_mul_d(prod, mx[ja[i]], as[i], MPFR_RNDN);
                mpfr_add(my[row], my[row], prod, MPFR_RNDN);
            }
        }
        mpfr_clear(prod);
    }
    const double t = omp_get_wtime() - t0;
    if (out)
        for (int i = 0; i < m; i++) out[i] = mpfr_get_d(my[i], MPFR_RNDN);
    mp_free(mx, n);
    mp_free(my, m);
    return t;
}
