/*
 * Host-side launchers of the kernels (one translation unit per operation) and
 * the per-unit table upload hooks.  Internal to libmpres_gb300.so.
 */
#ifndef MPRES_KERNELS_H
#define MPRES_KERNELS_H

#include <cuda_runtime.h>

#include "../../include/mpres_gb300.h"
#include "per_device.h"
#include "tables.h"

namespace mpres {

/* the current device ordinal, -1 if it cannot be read */
inline int current_device() {
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess ? dev : -1;
}
inline bool cuda_ok(const cudaError_t &e) { return e == cudaSuccess; }
inline bool positive(const int &v) { return v > 0; }

cudaError_t upload_tables_dot(int n, const void *tab);
cudaError_t upload_tables_gemv(int n, const void *tab);
cudaError_t upload_tables_gemm(int n, const void *tab);
cudaError_t upload_tables_spmv(int n, const void *tab);
cudaError_t upload_tables_elementwise(int n, const void *tab);
cudaError_t upload_tables_convert(int n, const void *tab);
cudaError_t upload_tables_batch(int n, const void *tab);
cudaError_t upload_tables_solver(int n, const void *tab);
cudaError_t upload_tables_probe_fx(int n, const void *tab);

/* Scratch for one call, carved from a per-device workspace. */
struct Workspace {
    void *ptr = nullptr;
    size_t bytes = 0;
};

/* mp_dot: g3 block sums go to ws (g3 * (4n+40) bytes). */
cudaError_t launch_dot(int nmod, int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy,
                       const mp_array_t &r, int g3, int b3, Workspace ws, cudaStream_t s);

/* address and size of the file-scope scratch of mpres_dot_noalloc on the current
 * device (looked up once per device) */
cudaError_t dot_noalloc_scratch(Workspace &ws);

cudaError_t launch_gemv(int nmod, bool trans, int m, int n, const mp_array_t &alpha, const mp_array_t &A, int lda,
                        const mp_array_t &x, int incx, const mp_array_t &beta, const mp_array_t &y, int incy,
                        int b3, Workspace ws, cudaStream_t s);

/* mp_gemm: W(A) and W(B), the signed residues scaled by 2^exp, go to ws
 * (gemm_workspace_bytes); with a smaller ws the chain runs step by step */
size_t gemm_workspace_bytes(int nmod, int m, int n, int k);
/* the split form's scratch (32 moduli; 0 for the other sets and for shapes
 * beyond its grids, which do not take that form): W(A), W(B), their bf16 limb
 * planes, the modular product and the scalar chain's results, about
 * (mk + kn + mn) * 4n + 8n k'(m' + n') + 48 mn bytes (m', n', k' padded to 64, 64,
 * 32).  A ws of at least this size selects it. */
size_t gemm_split_workspace_bytes(int nmod, int m, int n, int k);
/* the split form alone, with marks[0..kGemmSplitPhases] recorded on s before
 * its first launch and after each phase (W(A); W(B); the limb planes; the
 * scalar chain; the modular product; the epilogue; the per-output chain);
 * cudaErrorNotSupported for another set or a ws too small for that form */
constexpr int kGemmSplitPhases = 7;
cudaError_t launch_gemm_split_marked(int nmod, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A,
                                     int lda, const mp_array_t &B, int ldb, const mp_array_t &beta,
                                     const mp_array_t &C, int ldc, Workspace ws, cudaStream_t s, cudaEvent_t *marks);
cudaError_t launch_gemm(int nmod, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                        const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc,
                        Workspace ws, cudaStream_t s);

/* SpMV: the row schedule (length-sorted order) goes to ws */
size_t spmv_workspace_bytes(int m);
cudaError_t launch_spmv_csr(int nmod, int m, const csr_t &csr, const void *x, void *y, Workspace ws, cudaStream_t s);
cudaError_t launch_spmv_csrv(int nmod, int m, int tpr, const csr_t &csr, const void *x, void *y, Workspace ws,
                             cudaStream_t s);
cudaError_t launch_spmv_ell(int nmod, int m, int maxnzr, const ell_t &ell, const void *x, void *y, Workspace ws,
                            cudaStream_t s);

/* double -> mp_float_t on the device (host mp_set_d semantics): into AoS
 * out_aos when non-null, else into elements [offset, offset + count) of out_soa;
 * *flag |= 1 if an input took a path outside the replayed host behaviour */
cudaError_t launch_set_d(int nmod, const double *x, long long count, void *out_aos, const mp_array_t *out_soa,
                         long long offset, int *flag, cudaStream_t s);

/* AoS records in device memory <-> elements [offset, offset + count) of an
 * mp_array_t whose upper bounds start at eval + layout_len */
cudaError_t launch_pack(int nmod, bool to_soa, void *aos, const mp_array_t &a, long long layout_len, long long offset,
                        long long count, cudaStream_t s);

cudaError_t launch_elementwise(int nmod, int op, const void *x, const void *y, void *r, long long count,
                               cudaStream_t s);
/* the chain latency probe with the FP64 (elementwise.cu) or fixed-point (probe_fx.cu) evaluation */
cudaError_t launch_chain_probe_fp64(int nmod, int kind, const void *x, const void *y, int len, long long *cycles,
                                    unsigned *rounds, void *res, cudaStream_t s);
cudaError_t launch_round_probe(int nmod, const int *digits, const unsigned *D, int count, long long *cycles, int *out,
                               cudaStream_t s);
cudaError_t launch_psum_probe(int nmod, int which, const int *digits, long long count, void *cycles_or_out, int *out,
                              cudaStream_t s);
cudaError_t launch_eval_phase_probe(int nmod, const int *digits, int count, long long *cycles, int *out,
                                    cudaStream_t s);
cudaError_t launch_chain_probe_fx(int nmod, int kind, const void *x, const void *y, int len, long long *cycles,
                                  unsigned *rounds, void *res, cudaStream_t s);
cudaError_t launch_scale2pow(int nmod, const int *digits, const unsigned *D, int *out, long long count,
                             cudaStream_t s);
cudaError_t launch_check(int which, int nmod, const void *a, const void *b, void *out, long long count,
                         cudaStream_t s);
cudaError_t launch_eval(int nmod, int fast, const int *digits, er_t *low, er_t *upp, long long count,
                        cudaStream_t s);

/* conjugate gradients and the v2 vector kernels (solver.cu); M == nullptr: plain CG */
int solve_cg(int nmod, const HostTables &t, int n, const csr_t &A, const void *b, double tol, int maxit,
             const double *M, void *x, double *resvec, int resvec_cap, int *iters, int threads, int blocks_reduce,
             cudaStream_t s);
/* op 0: r = x - y, 1: r = alpha x + y, 2: r = -alpha x + y (AoS records) */
cudaError_t launch_vec_v2(int nmod, int op, int n, int threads, const void *alpha, const void *x, const void *y,
                          void *r, cudaStream_t s);
/* r[0] = x.y (sumsq: sum of |x_i^2| with mp_add_abs); parts holds `blocks` records */
cudaError_t launch_reduce_v2(int nmod, bool sumsq, int n, int blocks, int threads, const void *x, const void *y,
                             void *parts, void *r, cudaStream_t s);

/* status reporting shared by the C entry points (capi.cu): set the thread's
 * last-error text and return the status */
int status_fail(int code, const char *fmt, ...);
int status_ok();
int status_cuda(cudaError_t e, const char *what);
int status_require(int nmod); /* MPRES_SUCCESS if mpres_init(nmod) ran on the current device */

} // namespace mpres

#endif
