/*
 * CPU oracle for the RNS multiple-precision hot path of MPRES-BLAS.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * arithmetic and of the summation order of its kernels, used as the checker for
 * the CUDA library (tests, __graft_entry__.smoke and the CPU baseline of
 * bench.py).  The product never links or calls it.
 *
 * Multiple-precision numbers are exchanged in the reference's AoS layout of
 * mp_float_t for a set of N moduli (src/types.cuh:69-74):
 *     int digits[N]; int sign; int exp; struct {double frac; long exp;} eval[2];
 * which is 4N + 40 bytes per number.
 */
#ifndef MPRES_ORACLE_H
#define MPRES_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAXN 32
#define ORA_T 30

typedef struct {
    double frac;
    int64_t exp;
} ora_er_t;

/* Every constant of rns_const_init()/mp_const_init() for one moduli set. */
typedef struct {
    int n, log2m;
    int moduli[ORA_MAXN];
    int part_inv[ORA_MAXN];
    int *pow2; /* [(log2m + 1) * n] */
    int m_pow2_res[ORA_T];
    int part_pow2_res[ORA_T][ORA_MAXN];
    int pow2_inv[ORA_T][ORA_MAXN];
    double recip_rd[ORA_MAXN], recip_ru[ORA_MAXN];
    int mrc_inv[ORA_MAXN][ORA_MAXN];
    double eval_acc;
    int ref_factor;
    ora_er_t unit_low, unit_upp, inv_unit_low, inv_unit_upp;
    int mp_precision, mp_h, mp_j;
} ora_ctx_t;

/* Set-up for a moduli set of n in {8, 16, 32}; returns NULL for other sizes. */
const ora_ctx_t *ora_init(int n);
int ora_mp_size(int n);
int ora_threads(void);

/* Constant tables in the reference's array shapes (for pinning against it). */
void ora_tables(int n, int *part_inv, int *pow2, int *m_pow2_res, int *part_pow2_res, int *pow2_inv,
                double *recip_rd, double *recip_ru, int *mrc_inv, double *eval_acc, int *ref_factor,
                ora_er_t *units, int *mp_consts);

/* Host conversion double -> mp_float_t. */
void ora_set_d(int n, const double *x, long count, void *out);

/* Element-wise device arithmetic. */
void ora_add(int n, const void *x, const void *y, void *r, long count);
void ora_mul(int n, const void *x, const void *y, void *r, long count);
void ora_mul_d(int n, const void *x, const double *y, void *r, long count);
void ora_eval_fast(int n, const int *digits, ora_er_t *low, ora_er_t *upp, long count);
void ora_eval(int n, const int *digits, ora_er_t *low, ora_er_t *upp, long count);
void ora_scale2pow(int n, const int *digits, const unsigned *D, int *out, long count);

/* BLAS in the reference kernels' summation order. */
void ora_add_abs(int n, const void *x, const void *y, void *r, long count);
void ora_reduce_v2(int n, int sumsq, int len, const void *x, const void *y, void *r, int blocks, int threads);
void ora_dot(int n, int len, const void *x, int incx, const void *y, int incy, void *r, int g3, int b3);
void ora_gemv(int n, int trans, int m, int cols, const void *alpha, const void *A, int lda, const void *x,
              int incx, const void *beta, void *y, int incy, int b3);
void ora_gemm(int n, int m, int cols, int k, const void *alpha, const void *A, int lda, const void *B, int ldb,
              const void *beta, void *C, int ldc);
void ora_spmv_csr(int n, int m, const int *irp, const int *ja, const double *as, const void *x, void *y);
void ora_spmv_csrv(int n, int m, int tpr, const int *irp, const int *ja, const double *as, const void *x, void *y);
void ora_spmv_ell(int n, int m, int maxnzr, const int *ja, const double *as, const void *x, void *y);

#ifdef __cplusplus
}
#endif

#endif
