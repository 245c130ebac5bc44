/*
 * mpres_gb300 batches: many mp_gemv / mp_gemm / mp_dot / mp_spmv (CSR,
 * CSR-vector, ELL) operations of uneven sizes run as ONE persistent kernel
 * launch, replayed from a captured CUDA graph.  No counterpart in the reference, which launches every operation on
 * its own (cuda::mp_gemv, src/blas/gemv.cuh:151-269: ten kernels per call;
 * cuda::mp_dot, src/blas/dot.cuh:85-108; cuda::mp_spmv_csr,
 * src/sparse/spmv/spmv_csr.cuh:49-63).
 *
 * Results.  Every operation of a batch gives, bit for bit, what the plain entry
 * point (mpres_gemv, mpres_gemm, mpres_dot, mpres_spmv_*) gives for the same arguments:
 * the summation order of each output is fixed by the operation's own
 * blockDim3 / gridDim3, never by the batch, the launch shape or the autotuner.
 *
 * Use.  mpres_batch_create, then any number of mpres_batch_add_*, then
 * mpres_batch_commit (uploads the operation table and the task list, sizes the
 * scratch, optionally autotunes the launch shape and captures the graph), then
 * mpres_batch_run as often as wanted (the operands are read at run time, so
 * new values in the same arrays are picked up).  The operand arrays must stay
 * allocated until the batch is destroyed.  Operations of one batch must not
 * write overlapping outputs, and one batch runs on one stream at a time.
 *
 * Scheduling.  The kernel's CTAs take tasks from one atomic counter over a task
 * list sorted by estimated length, longest first: tiles of R outputs of a
 * GEMV (R = threads / blockDim3), groups of first-pass blocks of a DOT (the CTA
 * that finishes a DOT's last group also runs its second pass), chunks of
 * length-sorted rows of an SpMV (threads / threadsPerRow rows for CSR-vector),
 * and 32 x (threads / 32) tiles of a GEMM's C.  GEMV's alpha*x and GEMM's
 * scaled residues run as one element-wise launch before it (two kernel nodes
 * and two memset nodes per graph).
 */
#ifndef MPRES_GB300_BATCH_H
#define MPRES_GB300_BATCH_H

#include "mpres_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpres_batch mpres_batch_t;

/* mpres_batch_commit flags */
#define MPRES_BATCH_GRAPH 1u    /* capture the launches once; mpres_batch_run replays the graph */
#define MPRES_BATCH_AUTOTUNE 2u /* time the candidate launch shapes on this batch and keep the fastest */

int mpres_batch_create(int nmod, mpres_batch_t **batch);
int mpres_batch_destroy(mpres_batch_t *batch);

/* Same arguments, quick returns and results as mpres_gemv (an operation that
 * the plain call would skip is accepted and skipped). */
int mpres_batch_add_gemv(mpres_batch_t *batch, int trans, int m, int n, const mp_array_t *alpha, const mp_array_t *A,
                         int lda, const mp_array_t *x, int incx, const mp_array_t *beta, const mp_array_t *y, int incy,
                         int blockDim3);
/* Same as mpres_dot (n <= 0 is skipped). */
int mpres_batch_add_dot(mpres_batch_t *batch, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy,
                        const mp_array_t *r, int gridDim3, int blockDim3);
/* Same as mpres_spmv_csr: y[0..m) = A*x with AoS mp_float_t vectors. */
int mpres_batch_add_spmv_csr(mpres_batch_t *batch, int m, const csr_t *csr, const void *x, void *y);
/* Same as mpres_spmv_csrv (cuda::mp_spmv_csrv<threads, threadsPerRow>,
 * src/sparse/spmv/spmv_csrv.cuh:49-86): threadsPerRow lane-strided chains per
 * row and the fixed tree; threadsPerRow a power of two <= 32. */
int mpres_batch_add_spmv_csrv(mpres_batch_t *batch, int m, const csr_t *csr, const void *x, void *y,
                              int threadsPerRow);
/* Same as mpres_spmv_ell (cuda::mp_spmv_ell<threads>, src/sparse/spmv/spmv_ell.cuh:50-67):
 * maxnzr column-major slots per row, stored zeros skipped.  The commit reads
 * the slots once to order the rows by length. */
int mpres_batch_add_spmv_ell(mpres_batch_t *batch, int m, int maxnzr, const ell_t *ell, const void *x, void *y);

/* Same arguments, quick returns and results as mpres_gemm (cuda::mp_gemm,
 * src/blas/gemm.cuh:69-168): C = alpha*A*B + beta*C, no transposition, one
 * sequential k chain per output.  The commit sizes a scratch for the operands'
 * residues scaled by their powers of two ((m*k + k*n) * 4*nmod bytes).  A
 * batch holding GEMMs runs CTAs of 128 or 256 threads, so its blockDim3 and
 * threadsPerRow values must not exceed 256. */
int mpres_batch_add_gemm(mpres_batch_t *batch, int transa, int transb, int m, int n, int k, const mp_array_t *alpha,
                         const mp_array_t *A, int lda, const mp_array_t *B, int ldb, const mp_array_t *beta,
                         mp_array_t *C, int ldc);

int mpres_batch_commit(mpres_batch_t *batch, unsigned flags, void *stream);
int mpres_batch_run(mpres_batch_t *batch, void *stream);

/* out[0..7]: operations, tasks, threads per CTA, CTAs, graph (0/1), autotuned
 * (0/1), scratch bytes, candidate shapes timed */
int mpres_batch_info(const mpres_batch_t *batch, long long *out);

#ifdef __cplusplus
}
#endif

#endif
