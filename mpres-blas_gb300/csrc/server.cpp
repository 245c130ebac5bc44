/*
 * The serving loop of include/mpres_gb300_server.h: admission under an HBM
 * budget, continuous batching into the persistent batch kernel (batch.h), and
 * per-request latency.  No counterpart in the reference.
 *
 * One loop thread owns every CUDA call after creation.  Each batch slot has a
 * non-blocking stream, a completion event, a device buffer for the batch's
 * operation tables and a pinned staging copy of them; the scratch of a batch
 * (GEMV alpha*x, DOT block sums) comes from one device arena allocated at
 * creation.  So the loop allocates device memory only when a slot meets a
 * batch with larger tables than any before it (they grow by doubling) and when
 * an SpMV matrix appears for the first time (its row order is computed once
 * and kept until the server is destroyed): cudaFree waits for the whole
 * device, which would stall the batches in flight.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/mpres_gb300_server.h"
#include "batch.h"
#include "kernels.h"

using namespace mpres;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqKind { kGemv = 0, kDot = 1, kSpmv = 2 };

struct Req {
    long long id = 0;
    int kind = 0;
    int trans = 0, m = 0, n = 0, lda = 0, incx = 0, incy = 0, b3 = 0, g3 = 0;
    mp_array_t alpha{}, A{}, x{}, beta{}, y{}, r{};
    csr_t csr{};
    const void *xv = nullptr;
    void *yv = nullptr;
    size_t bytes = 0; /* operands and scratch, for admission */
};

struct Times {
    double submit = -1, launch = -1, done = -1;
};

/* first-fit allocator over one device allocation (offsets, 256-byte aligned) */
class Arena {
  public:
    cudaError_t init(size_t bytes) {
        size_ = (bytes + 255) & ~(size_t)255;
        free_.clear();
        cudaError_t e = cudaMalloc(&base_, size_ ? size_ : 256);
        if (e == cudaSuccess && size_) free_[0] = size_;
        return e;
    }
    void destroy() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
    }
    /* offset, or -1 */
    long long alloc(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        if (bytes == 0) return 0;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > bytes) free_[off + bytes] = len - bytes;
            return (long long)off;
        }
        return -1;
    }
    void release(long long off, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        if (off < 0 || bytes == 0) return;
        auto it = free_.emplace((size_t)off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    char *at(long long off) const { return base_ + off; }
    size_t size() const { return size_; }

  private:
    char *base_ = nullptr;
    size_t size_ = 0;
    std::map<size_t, size_t> free_;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<long long> ids;
    size_t bytes = 0;
    void *tables = nullptr;
    size_t tables_cap = 0;
    void *staging = nullptr;
    size_t staging_cap = 0;
    long long scratch_off = -1;
    size_t scratch_bytes = 0;
};

struct RowOrder {
    int *perm = nullptr;
    std::vector<int> lens;
};

} // namespace

struct mpres_server {
    int nmod = 0, device = 0, max_ops = 0, sms = 0, threads = 256, per_sm = 1;
    size_t budget = 0, rec = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> pending;
    std::vector<Times> times;
    std::vector<char> failed; /* per request: 1 if the loop could not run it, 2 if cancelled */
    long long cancelled = 0;
    size_t inflight = 0, peak = 0;
    int busy = 0, max_busy = 0, errors = 0;
    long long done_count = 0, batches = 0, batched = 0;
    bool stop = false;
    std::vector<Slot> slots;
    Arena arena;
    std::map<std::pair<const int *, int>, RowOrder> orders;
    cudaStream_t aux = nullptr;
    Clock::time_point t0;
    std::thread loop;
};

namespace {

double now(const mpres_server *s) { return std::chrono::duration<double>(Clock::now() - s->t0).count(); }

/* completions of the busy slots (mu held) */
void reap(mpres_server *s) {
    for (Slot &sl : s->slots) {
        if (!sl.busy) continue;
        const cudaError_t q = cudaEventQuery(sl.done);
        if (q == cudaErrorNotReady) continue;
        const double t = now(s);
        if (q != cudaSuccess) {
            s->errors++;
            status_cuda(q, "mpres_server (batch)");
        }
        for (long long id : sl.ids) {
            s->times[id].done = t;
            if (q != cudaSuccess) s->failed[id] = 1;
        }
        s->done_count += (long long)sl.ids.size();
        s->inflight -= sl.bytes;
        s->arena.release(sl.scratch_off, sl.scratch_bytes);
        sl.busy = false;
        sl.ids.clear();
        s->busy--;
        s->cv_done.notify_all();
    }
}

/* the row order of a CSR matrix, cached per (row pointers, rows) */
const RowOrder *row_order(mpres_server *s, const csr_t &csr, int m) {
    auto key = std::make_pair((const int *)csr.irp, m);
    auto it = s->orders.find(key);
    if (it != s->orders.end()) return &it->second;
    std::vector<int> irp((size_t)m + 1), order;
    RowOrder ro;
    if (cudaMemcpyAsync(irp.data(), csr.irp, sizeof(int) * irp.size(), cudaMemcpyDeviceToHost, s->aux) != cudaSuccess ||
        cudaStreamSynchronize(s->aux) != cudaSuccess)
        return nullptr;
    spmv_row_order(irp.data(), m, order, ro.lens);
    if (cudaMalloc(&ro.perm, sizeof(int) * (size_t)m) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(ro.perm, order.data(), sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, s->aux) != cudaSuccess ||
        cudaStreamSynchronize(s->aux) != cudaSuccess) {
        cudaFree(ro.perm);
        return nullptr;
    }
    return &(s->orders[key] = std::move(ro));
}

template <class T> cudaError_t grow(T *&p, size_t &cap, size_t want, bool pinned) {
    if (want <= cap) return cudaSuccess;
    size_t c = cap ? cap : (1u << 20);
    while (c < want) c *= 2;
    if (p) {
        if (pinned) cudaFreeHost(p);
        else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
    void *q = nullptr;
    cudaError_t e = pinned ? cudaHostAlloc(&q, c, cudaHostAllocDefault) : cudaMalloc(&q, c);
    if (e != cudaSuccess) return e;
    p = static_cast<T *>(q);
    cap = c;
    return cudaSuccess;
}

/* Builds and launches one batch of `reqs` on slot sl (mu not held).  false if
 * the scratch did not fit the arena right now (nothing launched). */
bool launch(mpres_server *s, Slot &sl, std::vector<Req> &reqs, cudaError_t &err) {
    err = cudaSuccess;
    BatchHost h;
    for (const Req &r : reqs) {
        if (r.kind == kGemv)
            batch_add_gemv(h, r.trans, r.m, r.n, r.alpha, r.A, r.lda, r.x, r.incx, r.beta, r.y, r.incy, r.b3);
        else if (r.kind == kDot)
            batch_add_dot(h, r.n, r.x, r.incx, r.y, r.incy, r.r, r.g3, r.b3);
        else {
            const RowOrder *ro = row_order(s, r.csr, r.m);
            if (!ro) {
                err = cudaErrorMemoryAllocation;
                return true;
            }
            batch_add_spmv(h, r.m, r.csr, r.xv, r.yv, ro->perm, ro->lens);
        }
    }
    int threads = s->threads;
    for (const GemvOp &g : h.gemv) threads = std::max(threads, g.b3);
    for (const DotOp &d : h.dot) threads = std::max(threads, d.b3);
    int t2 = 32;
    while (t2 < threads) t2 *= 2;
    threads = t2;
    const int per_sm = threads == s->threads ? s->per_sm : std::max(1, batch_ctas_per_sm(s->nmod, threads));
    batch_plan(h, threads);
    const size_t buf1 = s->rec * (size_t)h.buf1_elems, parts = s->rec * (size_t)h.part_elems;
    const size_t scratch = ((buf1 + 255) & ~(size_t)255) + parts;
    long long off;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        off = s->arena.alloc(scratch);
    }
    if (off < 0) return false;
    const TableLayout l = batch_layout(h);
    if ((err = grow(sl.staging, sl.staging_cap, l.total, true)) != cudaSuccess ||
        (err = grow(sl.tables, sl.tables_cap, l.total, false)) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->arena.release(off, scratch);
        return true;
    }
    batch_pack(h, l, sl.staging);
    char *sbase = s->arena.at(off);
    const BatchDev d = batch_dev_at(h, l, sl.tables, buf1 ? sbase : nullptr,
                                    parts ? sbase + ((buf1 + 255) & ~(size_t)255) : nullptr, nullptr);
    err = cudaMemcpyAsync(sl.tables, sl.staging, l.total, cudaMemcpyHostToDevice, sl.stream);
    if (err == cudaSuccess) err = batch_launch(s->nmod, h, d, threads, per_sm * s->sms, sl.stream);
    if (err == cudaSuccess) err = cudaEventRecord(sl.done, sl.stream);
    std::lock_guard<std::mutex> lk(s->mu);
    if (err != cudaSuccess) {
        s->arena.release(off, scratch);
        return true;
    }
    const double t = now(s);
    sl.busy = true;
    sl.scratch_off = off;
    sl.scratch_bytes = scratch;
    sl.bytes = 0;
    sl.ids.clear();
    for (const Req &r : reqs) {
        sl.ids.push_back(r.id);
        sl.bytes += r.bytes;
        s->times[r.id].launch = t;
    }
    s->busy++;
    s->max_busy = std::max(s->max_busy, s->busy);
    s->batches++;
    s->batched += (long long)reqs.size();
    return true;
}

void loop_main(mpres_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        reap(s);
        if (s->stop && s->pending.empty() && s->busy == 0) break;
        Slot *free_slot = nullptr;
        for (Slot &sl : s->slots)
            if (!sl.busy) {
                free_slot = &sl;
                break;
            }
        if (free_slot && !s->pending.empty()) {
            /* admit in arrival order while the budget lasts */
            std::vector<Req> take;
            size_t bytes = 0;
            while (!s->pending.empty() && (int)take.size() < s->max_ops) {
                const Req &r = s->pending.front();
                if (r.bytes > s->budget) { /* can never fit: fail it */
                    s->times[r.id].done = now(s);
                    s->failed[r.id] = 1;
                    s->done_count++;
                    s->errors++;
                    s->pending.pop_front();
                    s->cv_done.notify_all();
                    continue;
                }
                if (s->inflight + bytes + r.bytes > s->budget) break;
                bytes += r.bytes;
                take.push_back(r);
                s->pending.pop_front();
            }
            if (!take.empty()) {
                s->inflight += bytes;
                s->peak = std::max(s->peak, s->inflight);
                lk.unlock();
                cudaError_t err;
                const bool launched = launch(s, *free_slot, take, err);
                lk.lock();
                if (err != cudaSuccess) {
                    s->errors++;
                    status_cuda(err, "mpres_server (launch)");
                    s->inflight -= bytes;
                    for (const Req &r : take) {
                        s->times[r.id].done = now(s);
                        s->failed[r.id] = 1;
                        s->done_count++;
                    }
                    s->cv_done.notify_all();
                } else if (!launched) { /* no scratch now: back to the queue front, wait for a completion */
                    s->inflight -= bytes;
                    for (auto it = take.rbegin(); it != take.rend(); ++it) s->pending.push_front(*it);
                    if (s->busy == 0) { /* nothing will free scratch: the batch is too large for the arena */
                        const Req r = s->pending.front();
                        s->pending.pop_front();
                        s->times[r.id].done = now(s);
                        s->failed[r.id] = 1;
                        s->done_count++;
                        s->errors++;
                        s->cv_done.notify_all();
                    }
                }
                continue;
            }
        }
        if (s->busy > 0) {
            /* batches run: poll their events */
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(5));
            lk.lock();
        } else {
            s->cv_work.wait(lk, [s] { return s->stop || !s->pending.empty(); });
        }
    }
}

size_t mp_bytes(const mpres_server *s, long long elems) { return s->rec * (size_t)(elems > 0 ? elems : 0); }

int submit(mpres_server *s, Req &r, bool quick, long long *id) {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server: stopped");
    r.id = (long long)s->times.size();
    Times t;
    t.submit = now(s);
    if (quick) {
        t.launch = t.done = t.submit;
        s->done_count++;
    }
    s->times.push_back(t);
    s->failed.push_back(0);
    if (id) *id = r.id;
    if (!quick) {
        s->pending.push_back(r);
        s->cv_work.notify_one();
    } else {
        s->cv_done.notify_all();
    }
    return status_ok();
}

} // namespace

extern "C" {

int mpres_server_create(int nmod, size_t hbm_budget, int slots, int max_batch_ops, mpres_server_t **server) {
    if (!server) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_create: null handle");
    if (int st = status_require(nmod)) return st;
    if (slots < 1 || slots > 16 || max_batch_ops < 1 || hbm_budget == 0)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_create: slots %d / max_batch_ops %d / budget", slots,
                           max_batch_ops);
    mpres_server *s = new (std::nothrow) mpres_server;
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_create: out of host memory");
    s->nmod = nmod;
    s->budget = hbm_budget;
    s->max_ops = max_batch_ops;
    s->rec = 4 * (size_t)nmod + 40;
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    if (!batch_cached_shape(nmod, s->threads, s->per_sm)) {
        s->threads = 256;
        s->per_sm = std::max(1, batch_ctas_per_sm(nmod, 256));
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking);
    s->slots.resize((size_t)slots);
    for (Slot &sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    }
    /* scratch: a sixteenth of the budget, at least 64 MB, at most 4 GB */
    size_t arena = std::min<size_t>(std::max<size_t>(hbm_budget / 16, (size_t)64 << 20), (size_t)4 << 30);
    if (e == cudaSuccess) e = s->arena.init(arena);
    if (e != cudaSuccess) {
        const int st = status_cuda(e, "mpres_server_create");
        for (Slot &sl : s->slots) {
            if (sl.stream) cudaStreamDestroy(sl.stream);
            if (sl.done) cudaEventDestroy(sl.done);
        }
        if (s->aux) cudaStreamDestroy(s->aux);
        s->arena.destroy();
        delete s;
        return st;
    }
    s->t0 = Clock::now();
    s->loop = std::thread(loop_main, s);
    *server = s;
    return status_ok();
}

int mpres_server_destroy(mpres_server_t *s) {
    if (!s) return status_ok();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->loop.joinable()) s->loop.join();
    for (Slot &sl : s->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.tables) cudaFree(sl.tables);
        if (sl.staging) cudaFreeHost(sl.staging);
    }
    for (auto &kv : s->orders)
        if (kv.second.perm) cudaFree(kv.second.perm);
    if (s->aux) cudaStreamDestroy(s->aux);
    s->arena.destroy();
    const int errors = s->errors;
    delete s;
    return errors ? status_fail(MPRES_ERR_CUDA, "mpres_server_destroy: %d request(s) failed", errors) : status_ok();
}

int mpres_server_submit_gemv(mpres_server_t *s, int trans, int m, int n, const mp_array_t *alpha, const mp_array_t *A,
                             int lda, const mp_array_t *x, int incx, const mp_array_t *beta, const mp_array_t *y,
                             int incy, int blockDim3, long long *id) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_gemv: null server");
    Req r;
    const bool quick = m <= 0 || n <= 0 || incx == 0 || incy == 0 || lda < (m > 1 ? m : 1);
    if (!quick) {
        if (!alpha || !A || !x || !beta || !y)
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_gemv: null array");
        if (blockDim3 <= 0 || blockDim3 > 1024)
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_gemv: blockDim3 %d out of range", blockDim3);
        r.kind = kGemv;
        r.trans = trans; r.m = m; r.n = n; r.lda = lda; r.incx = incx; r.incy = incy; r.b3 = blockDim3;
        r.alpha = *alpha; r.A = *A; r.x = *x; r.beta = *beta; r.y = *y;
        const long long inner = trans != MPRES_NO_TRANS ? m : n, outs = trans != MPRES_NO_TRANS ? n : m;
        r.bytes = mp_bytes(s, (long long)m * n + 2 * inner + outs + 2);
    }
    return submit(s, r, quick, id);
}

int mpres_server_submit_dot(mpres_server_t *s, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy,
                            const mp_array_t *r_, int gridDim3, int blockDim3, long long *id) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_dot: null server");
    Req r;
    const bool quick = n <= 0;
    if (!quick) {
        if (!x || !y || !r_) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_dot: null array");
        if (gridDim3 <= 0 || blockDim3 <= 0 || blockDim3 > 1024)
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_dot: gridDim3 %d / blockDim3 %d",
                               gridDim3, blockDim3);
        r.kind = kDot;
        r.n = n; r.incx = incx; r.incy = incy; r.g3 = gridDim3; r.b3 = blockDim3;
        r.x = *x; r.y = *y; r.r = *r_;
        r.bytes = mp_bytes(s, 2LL * n + gridDim3 + 1);
    }
    return submit(s, r, quick, id);
}

int mpres_server_submit_spmv_csr(mpres_server_t *s, int m, int ncols, long long nnz, const csr_t *csr, const void *x,
                                 void *y, long long *id) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_spmv_csr: null server");
    Req r;
    const bool quick = m <= 0;
    if (!quick) {
        if (!csr || !x || !y) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_submit_spmv_csr: null argument");
        r.kind = kSpmv;
        r.m = m; r.csr = *csr; r.xv = x; r.yv = y;
        r.bytes = (size_t)(nnz > 0 ? nnz : 0) * 12 + (size_t)m * 8 + 4 + mp_bytes(s, (long long)ncols + m);
    }
    return submit(s, r, quick, id);
}

int mpres_server_wait(mpres_server_t *s, long long id, double timeout_s) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    if (id < 0 || id >= (long long)s->times.size())
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_wait: no request %lld", id);
    auto ready = [&] { return s->times[id].done >= 0; };
    if (timeout_s < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
        return status_fail(MPRES_ERR_NOT_SUPPORTED, "mpres_server_wait: request %lld not done in %.3f s", id, timeout_s);
    if (s->failed[id] == 2) return status_fail(MPRES_ERR_CANCELLED, "mpres_server_wait: request %lld was cancelled", id);
    if (s->failed[id]) return status_fail(MPRES_ERR_CUDA, "mpres_server_wait: request %lld failed", id);
    return status_ok();
}

int mpres_server_cancel(mpres_server_t *s, long long id) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_cancel: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (id < 0 || id >= (long long)s->times.size())
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_cancel: no request %lld", id);
    for (auto it = s->pending.begin(); it != s->pending.end(); ++it) {
        if (it->id != id) continue;
        s->pending.erase(it);
        s->times[id].done = now(s);
        s->failed[id] = 2;
        s->done_count++;
        s->cancelled++;
        s->cv_done.notify_all();
        return status_ok();
    }
    return status_fail(MPRES_ERR_NOT_SUPPORTED, "mpres_server_cancel: request %lld already launched or done", id);
}

int mpres_server_drain(mpres_server_t *s) {
    if (!s) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_drain: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    const long long target = (long long)s->times.size();
    s->cv_done.wait(lk, [&] { return s->done_count >= target; });
    for (long long i = 0; i < target; i++)
        if (s->failed[i] == 1) return status_fail(MPRES_ERR_CUDA, "mpres_server_drain: request %lld failed", i);
    return status_ok();
}

int mpres_server_times(mpres_server_t *s, long long first, long long count, double *out) {
    if (!s || (!out && count > 0)) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_times: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (first < 0 || count < 0 || first + count > (long long)s->times.size())
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_times: range outside the requests");
    for (long long i = 0; i < count; i++) {
        const Times &t = s->times[first + i];
        out[3 * i] = t.submit;
        out[3 * i + 1] = t.launch;
        out[3 * i + 2] = t.done;
    }
    return status_ok();
}

int mpres_server_stats(mpres_server_t *s, double *out) {
    if (!s || !out) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_server_stats: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> lat;
    for (const Times &t : s->times)
        if (t.done >= 0) lat.push_back(t.done - t.submit);
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
        if (lat.empty()) return 0.0;
        size_t k = (size_t)std::ceil(p * (double)lat.size());
        return lat[k == 0 ? 0 : std::min(k - 1, lat.size() - 1)];
    };
    out[0] = (double)lat.size();
    out[1] = (double)s->batches;
    out[2] = s->batches ? (double)s->batched / (double)s->batches : 0.0;
    out[3] = pct(0.50);
    out[4] = pct(0.99);
    out[5] = (double)s->peak;
    out[6] = (double)s->max_busy;
    out[7] = (double)s->errors;
    return status_ok();
}

} // extern "C"
