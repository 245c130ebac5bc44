/*
 * Internal interface of the persistent batch kernel (batch.cu), shared by the
 * batch entry points (mpres_batch_*) and the serving loop (server.cpp).
 *
 * A batch is a list of operations (GEMV, DOT, SpMV in its CSR, CSR-vector and
 * ELL forms, GEMM) with device pointers to their operands, a task list over
 * them, and scratch: GEMM's W(A) and W(B) (`w`), GEMV's alpha*x
 * (`buf1`, one record per inner index) and DOT's block sums (`parts`, gridDim3
 * records per DOT).  The host builds everything in BatchHost; the device copy
 * of the tables lives wherever the caller put it (BatchDev).
 */
#ifndef MPRES_BATCH_H
#define MPRES_BATCH_H

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "tables.h"

namespace mpres {

struct GemvOp {
    const int *Ad, *As, *Ae;
    const er_t *Av;
    const int *Alen;
    const int *xd, *xs, *xe;
    const er_t *xv;
    const int *xlen;
    const int *ad, *as, *ae;
    const er_t *av;
    const int *alen;
    const int *bd, *bs, *be;
    const er_t *bv;
    const int *blen;
    int *yd, *ys, *ye;
    er_t *yv;
    const int *ylen;
    int m, n, lda, incx, incy, trans, b3, R;
    long long buf1_off;
};

struct DotOp {
    const int *xd, *xs, *xe;
    const er_t *xv;
    const int *xlen;
    const int *yd, *ys, *ye;
    const er_t *yv;
    const int *ylen;
    int *rd, *rs, *re;
    er_t *rv;
    const int *rlen;
    int n, incx, incy, g3, b3, groups;
    long long part_off;
};

/* SpMV forms: CSR (one chain per row), CSR-vector (tpr lane-strided chains
 * per row and the fixed tree), ELL (one chain per row over column-major slots,
 * stored zeros skipped; irp unused) */
enum SpmvForm { kCsr = 0, kCsrv = 1, kEll = 2 };

struct SpmvOp {
    const int *irp, *ja;
    const double *as;
    const void *x;
    void *y;
    const int *perm; /* rows by length, longest first */
    int m, form, tpr, maxnzr;
};

/* C = alpha*A*B + beta*C (no transposition), the lazy-residue chain of
 * gemm_chain.cuh; W(A) and W(B) live in the batch's W scratch at the int4
 * offsets wa, wb */
struct GemmOp {
    const int *ad, *as, *ae;
    const er_t *av;
    const int *alen;
    const int *Ad, *As, *Ae;
    const er_t *Av;
    const int *Alen;
    const int *Bd, *Bs, *Be;
    const er_t *Bv;
    const int *Blen;
    const int *bd, *bs, *be;
    const er_t *bv;
    const int *blen;
    int *Cd, *Cs, *Ce;
    er_t *Cv;
    const int *Clen;
    int m, n, k, lda, ldb, ldc;
    long long wa, wb;
};

enum TaskKind { kGemvTile = 0, kDotGroup = 1, kSpmvChunk = 2, kGemmTile = 3 };

struct Task {
    int kind, op, a, b; /* GEMV: first output; DOT: first block, blocks; SpMV: first sorted row, rows;
                           GEMM: first row, first column of a 32 x (threads / 32) tile */
};

enum ChunkKind { kChunkAlphaX = 0, kChunkWA = 1, kChunkWB = 2 };

struct ScaleChunk {
    /* GEMV alpha*x: entries [start, start + count) of GEMV op; GEMM W(A) / W(B):
     * elements [start, start + count) of GEMM op's A / B */
    int op, start, count, kind;
};

struct BatchHost {
    std::vector<GemvOp> gemv;
    std::vector<DotOp> dot;
    std::vector<SpmvOp> spmv;
    std::vector<GemmOp> gemm;
    long long w_elems = 0; /* int4 entries of the GEMM W scratch */
    std::vector<std::vector<int>> spmv_len; /* row lengths in perm order, per SpMV */
    std::vector<Task> tasks;
    std::vector<ScaleChunk> chunks;
    long long buf1_elems = 0, part_elems = 0;
};

struct BatchDev {
    GemvOp *gemv = nullptr;
    DotOp *dot = nullptr;
    SpmvOp *spmv = nullptr;
    GemmOp *gemm = nullptr;
    void *w = nullptr; /* GEMM W(A), W(B): w_elems int4 */
    Task *tasks = nullptr;
    ScaleChunk *chunks = nullptr;
    int *counters = nullptr; /* 1 + number of DOTs */
    void *buf1 = nullptr;    /* buf1_elems records */
    void *parts = nullptr;   /* part_elems records */
};

/* the operation records of the public arguments (quick returns: false, nothing added) */
bool batch_add_gemv(BatchHost &b, int trans, int m, int n, const mp_array_t &alpha, const mp_array_t &A, int lda,
                    const mp_array_t &x, int incx, const mp_array_t &beta, const mp_array_t &y, int incy, int b3);
bool batch_add_dot(BatchHost &b, int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy,
                   const mp_array_t &r, int g3, int b3);
void batch_add_spmv(BatchHost &b, int m, const csr_t &csr, const void *x, void *y, const int *perm,
                    std::vector<int> lens, int form = kCsr, int tpr = 1);
void batch_add_spmv_ell(BatchHost &b, int m, int maxnzr, const ell_t &ell, const void *x, void *y);
/* quick returns of src/blas/gemm.cuh:77-96: false, nothing added */
bool batch_add_gemm(BatchHost &b, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                    const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc, int nmod);

/* rows of a CSR matrix by length, longest first, equal lengths in row order,
 * from host row pointers; lens[i] = length of row order[i] */
void spmv_row_order(const int *irp, int m, std::vector<int> &order, std::vector<int> &lens);

/* element-wise chunks (GEMV alpha*x, GEMM W(A), W(B)) and the task list for
 * `threads` per CTA, longest task first; false if an operation's blockDim3
 * exceeds `threads`, or a GEMM meets more than 256 threads */
bool batch_plan(BatchHost &b, int threads);

/* bytes of the device tables (operations, tasks, chunks, counters) and their
 * packing into one buffer: the offsets of each part */
struct TableLayout {
    size_t gemv, dot, spmv, gemm, tasks, chunks, counters, total;
};
TableLayout batch_layout(const BatchHost &b);
void batch_pack(const BatchHost &b, const TableLayout &l, void *host_buf);
BatchDev batch_dev_at(const BatchHost &b, const TableLayout &l, void *dev_buf, void *buf1, void *parts, void *w);

/* counters reset, the alpha*x launch and the persistent launch, on stream s */
cudaError_t batch_launch(int nmod, const BatchHost &b, const BatchDev &d, int threads, int ctas, cudaStream_t s);
/* largest CTAs per SM for `threads` (sets the kernel's shared-memory attribute);
 * gemm: the variant with GEMM tiles (128 or 256 threads) */
int batch_ctas_per_sm(int nmod, int threads, bool gemm = false);
/* the autotuned shape of this set on the current device, if any: {threads, CTAs per SM} */
bool batch_cached_shape(int nmod, int &threads, int &per_sm);

} // namespace mpres

#endif
