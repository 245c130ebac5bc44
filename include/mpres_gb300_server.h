/*
 * mpres_gb300 serving loop: a request loop over device-resident operands that
 * admits mixed mp_gemv / mp_dot / mp_spmv_csr requests under an HBM budget and
 * runs whatever is admitted together as one persistent batch launch
 * (include/mpres_gb300_batch.h), several batches in flight on their own
 * streams.  No counterpart in the reference, which has no serving layer.
 *
 * Continuous batching: a loop thread owned by the server takes, whenever a
 * batch slot is free, every pending request (in arrival order) whose bytes fit
 * in what the budget has left, launches them as one batch, and returns their
 * bytes when that batch's completion event fires; requests that arrive while
 * batches run join the next one, and its launch overlaps the tail of the
 * running ones on the device.
 *
 * Results: each request gives exactly what the plain call with the same
 * arguments gives (its summation order is its own), alone or in any mix.
 * Operands are the caller's device arrays; they must stay allocated, and a
 * request's outputs unread and its inputs unchanged, until the request is done.
 * Requests in flight together must not write overlapping outputs.
 *
 * Latency of a request = completion seen by the loop - submit call; the loop
 * polls completion events every few microseconds while batches run.
 */
#ifndef MPRES_GB300_SERVER_H
#define MPRES_GB300_SERVER_H

#include "mpres_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpres_server mpres_server_t;

/* hbm_budget: bytes of operands and scratch that admitted, unfinished requests
 * may touch together; slots: batches in flight at once (1..16); max_batch_ops:
 * most requests per batch.  The loop thread uses the current device. */
int mpres_server_create(int nmod, size_t hbm_budget, int slots, int max_batch_ops, mpres_server_t **server);
/* stops admitting, waits for every submitted request, joins the loop thread */
int mpres_server_destroy(mpres_server_t *server);

/* Requests; *id receives the request number (0, 1, 2, ... in submit order).
 * Arguments, quick returns and results as mpres_gemv / mpres_dot /
 * mpres_spmv_csr (a quick return completes at once).  For the SpMV, ncols (the
 * length of x) and nnz only size the request's bytes for admission. */
int mpres_server_submit_gemv(mpres_server_t *server, int trans, int m, int n, const mp_array_t *alpha,
                             const mp_array_t *A, int lda, const mp_array_t *x, int incx, const mp_array_t *beta,
                             const mp_array_t *y, int incy, int blockDim3, long long *id);
int mpres_server_submit_dot(mpres_server_t *server, int n, const mp_array_t *x, int incx, const mp_array_t *y,
                            int incy, const mp_array_t *r, int gridDim3, int blockDim3, long long *id);
int mpres_server_submit_spmv_csr(mpres_server_t *server, int m, int ncols, long long nnz, const csr_t *csr,
                                 const void *x, void *y, long long *id);

/* blocks until request id is done (timeout_s < 0: no limit); MPRES_ERR_CUDA if
 * the loop met a CUDA error or the request could never fit the budget,
 * MPRES_ERR_CANCELLED if it was cancelled, MPRES_ERR_NOT_SUPPORTED on timeout */
int mpres_server_wait(mpres_server_t *server, long long id, double timeout_s);
/* blocks until every request submitted so far is done */
int mpres_server_drain(mpres_server_t *server);
/* withdraws request id if it is still waiting for admission: it completes at
 * once, its outputs untouched, and waiting for it returns MPRES_ERR_CANCELLED.
 * MPRES_ERR_NOT_SUPPORTED if it was already launched or done. */
int mpres_server_cancel(mpres_server_t *server, long long id);

/* Per-request times in seconds since the server was created, for requests
 * [first, first + count): out[3*i] = submitted, out[3*i+1] = launched,
 * out[3*i+2] = done (-1 while not done). */
int mpres_server_times(mpres_server_t *server, long long first, long long count, double *out);
/* out[0..7]: requests done, batches launched, mean requests per batch, p50 and
 * p99 latency of the done requests (seconds), peak bytes admitted at once,
 * largest batches in flight at once, loop errors */
int mpres_server_stats(mpres_server_t *server, double *out);

#ifdef __cplusplus
}
#endif

#endif
