/*
 * SpMV y = A*x with a double-precision sparse A and multiple-precision AoS
 * vectors x, y (mp_float_t[], src/types.cuh:69-74).
 *
 * References (kernels their callers launch directly):
 *   cuda::mp_spmv_csr<threads>        src/sparse/spmv/spmv_csr.cuh:49-63
 *   cuda::mp_spmv_csrv<threads, tpr>  src/sparse/spmv/spmv_csrv.cuh:49-86
 *   cuda::mp_spmv_ell<threads>        src/sparse/spmv/spmv_ell.cuh:50-67
 * Each output is a sequential chain y_row = (((0 + a_0*x) + a_1*x) + ...) of
 * mp_mul_d / mp_add; csrv runs tpr lane-strided chains and adds them with the
 * fixed tree 16, 8, 4, 2, 1.  Those orders are kept exactly: a row's result does
 * not depend on which thread computes it or when.
 *
 * Scheduling (this library's, not the reference's).  With one thread per row in
 * natural order, a warp runs as long as its longest row: on power-law rows only a
 * few lanes stay busy.  Each call therefore first sorts the rows by length into
 * buckets (exact lengths below 16, four buckets per octave above) with two short
 * passes over the row pointers, then warps take consecutive chunks of the
 * sorted order, longest bucket first, through one atomic counter: lanes of a warp
 * hold rows of similar length, and the longest chains start at once.  The
 * reference stages each thread's running sum and product in shared memory; here
 * they stay in registers and the csrv tree moves partial sums with shuffles.
 */
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(spmv)

namespace mpres {
namespace {
using namespace dev;

constexpr int kBuckets = 128;

/* bucket of a row length; larger lengths give larger buckets */
__device__ __forceinline__ int bucket_of(int len) {
    if (len < 16) return len;
    const int oct = 31 - __clz(len);            /* 4 .. 30 */
    const int sub = (len >> (oct - 2)) & 3;    /* next two bits */
    const int b = 16 + (oct - 4) * 4 + sub;
    return b < kBuckets ? b : kBuckets - 1;
}

/* Workspace layout (ints): [0, 128) counts, [128, 256) cursors, [256] chunk
 * counter, [257] unused, [258, 260) the total of the row lengths (64-bit),
 * [260, 512) blocks seen per SM, [512, 512 + m) the sorted row order,
 * [512 + m, 512 + 2m) ELL row ends. */
constexpr int kSlots = 252;
struct Sched {
    int *counts, *cursors, *next, *perm;
    unsigned long long *total;
    int *slots, *ends;
};

/* length of row r: CSR from the row pointers, ELL from its last nonzero slot */
struct CsrLen {
    const int *irp;
    __device__ int operator()(int r) const { return __ldg(irp + r + 1) - __ldg(irp + r); }
};
/* ELL: one past the last stored nonzero of the row (ell_row_ends) */
struct EllEnd {
    const int *ends;
    __device__ int operator()(int r) const { return __ldg(ends + r); }
};

template <class Len> __global__ void bucket_count(int m, Len lenf, Sched s) {
    __shared__ int hist[kBuckets];
    __shared__ unsigned long long tot;
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) hist[b] = 0;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    unsigned long long mine = 0;
    const int lane = threadIdx.x & 31;
    /* warp-uniform trip count; the lanes of one bucket add their count once */
    for (int r0 = blockIdx.x * blockDim.x; r0 < m; r0 += gridDim.x * blockDim.x) {
        const int r = r0 + (int)threadIdx.x;
        const bool ok = r < m;
        const unsigned act = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const int len = lenf(r);
            const int b = bucket_of(len);
            const unsigned peers = __match_any_sync(act, b);
            if (lane == __ffs(peers) - 1) atomicAdd(&hist[b], __popc(peers));
            mine += (unsigned)len;
        }
    }
    atomicAdd(&tot, mine);
    __syncthreads();
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
        if (hist[b]) atomicAdd(&s.counts[b], hist[b]);
    if (threadIdx.x == 0) atomicAdd(s.total, tot);
}

/* ELL row ends: one past the last nonzero slot of each row (the loop bound of
 * the row's chain; the reference's kernel visits all maxnzr slots and skips
 * zeros, src/sparse/spmv/spmv_ell.cuh:50-67, so stopping after the last
 * nonzero changes nothing).  Consecutive threads take consecutive rows and scan
 * their slots downwards from maxnzr - 1: each column is one coalesced read of
 * the warp's 32 rows, and the warp stops at its rows' largest end. */
__global__ void ell_row_ends(int m, int maxnzr, const double *__restrict__ as, int *ends) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        int c = maxnzr;
        while (c > 0 && !dnz(__ldg(as + (size_t)(c - 1) * m + r))) c--;
        ends[r] = c;
    }
}
/* the same two rows to a thread with 16-byte loads (m even, as 16-byte aligned):
 * a warp reads 512 contiguous bytes of a column at a time */
__global__ void ell_row_ends2(int m, int maxnzr, const double *__restrict__ as, int *ends) {
    const int pairs = m / 2;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < pairs; t += gridDim.x * blockDim.x) {
        const int r = 2 * t;
        int c0 = maxnzr, c1 = maxnzr;
        bool f0 = false, f1 = false;
        for (int c = maxnzr; c > 0 && !(f0 && f1); c--) {
            const double2 v = __ldg(reinterpret_cast<const double2 *>(as + (size_t)(c - 1) * m + r));
            if (!f0) {
                if (dnz(v.x)) f0 = true;
                else c0 = c - 1;
            }
            if (!f1) {
                if (dnz(v.y)) f1 = true;
                else c1 = c - 1;
            }
        }
        ends[r] = c0;
        ends[r + 1] = c1;
    }
}

/* cursors: exclusive offsets with the longest bucket first (one block) */
__global__ void bucket_offsets(Sched s) {
    if (threadIdx.x == 0) {
        int off = 0;
        for (int b = kBuckets - 1; b >= 0; b--) {
            s.cursors[b] = off;
            off += s.counts[b];
        }
        *s.next = 0;
    }
}

/* rows into their buckets' ranges of the order; the lanes of a warp that share a
 * bucket take one cursor increment (row lengths are heavily skewed: on the
 * power-law matrices nearly half the rows fall into one bucket) */
template <class Len> __global__ void bucket_scatter(int m, Len lenf, Sched s) {
    const int lane = threadIdx.x & 31;
    for (int r0 = blockIdx.x * blockDim.x; r0 < m; r0 += gridDim.x * blockDim.x) {
        const int r = r0 + (int)threadIdx.x;
        const bool ok = r < m;
        const unsigned act = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const int b = bucket_of(lenf(r));
            const unsigned peers = __match_any_sync(act, b);
            const int leader = __ffs(peers) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&s.cursors[b], __popc(peers));
            base = __shfl_sync(peers, base, leader);
            s.perm[base + __popc(peers & ((1u << lane) - 1))] = r;
        }
    }
}

/* a warp's next chunk of `size` entries of the sorted order (-1 when exhausted) */
__device__ __forceinline__ int next_chunk(int *next, int size) {
    int base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(next, size);
    return __shfl_sync(0xffffffffu, base, 0);
}

/* Chain-bound schedules.  A lane's time is its rows' chain of dependent
 * multiple-precision steps, and a warp that shares its SM sub-partition with
 * others waits for issue slots and the FP64 pipe between its steps.  When the
 * longest chain (the first row of the sorted order, `tpr` lanes to a row) is at
 * least the average work of a lane with one block per SM, that chain bounds the
 * whole call: then only the first block to arrive on each SM works and the
 * others leave at once, so the longest chains run without neighbours (mp_spmv_csr
 * over 2^20 power-law rows, 8 moduli: 7.6 ms against 11-13 ms with every block;
 * the longest chain alone takes 7.3 ms).  Otherwise every block works.  The
 * blocks share the work through one counter, so how many take part never
 * changes a result. */
template <class Len>
__device__ __forceinline__ bool spare_block(const Sched &s, int m, int sms, int tpr, Len lenf) {
    __shared__ int spare;
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        const int slot = smid < (unsigned)kSlots ? atomicAdd(s.slots + smid, 1) : 0;
        bool bound = false;
        if (m > 0 && slot > 0) {
            const long long chain = ((long long)lenf(__ldg(s.perm)) + tpr - 1) / tpr;
            bound = chain * sms * (long long)blockDim.x >= (long long)*s.total;
        }
        spare = bound;
    }
    __syncthreads();
    return spare != 0;
}

template <int N>
__device__ __forceinline__ void csr_row(int row, const int *__restrict__ irp, const int *__restrict__ ja,
                                        const double *__restrict__ as, const void *x, void *y) {
    mp_t<N> sum;
    set_zero<N>(sum);
    const int start = __ldg(irp + row), end = __ldg(irp + row + 1);
    /* the next entry's x record and value are loaded a step ahead: the gather's
     * latency overlaps the current step's arithmetic */
    mp_t<N> xn;
    double an = 0.0;
    if (start < end) {
        load_aos<N>(xn, x, __ldg(ja + start));
        an = __ldg(as + start);
    }
    for (int i = start; i < end; i++) {
        const mp_t<N> xv = xn;
        const double a = an;
        if (i + 1 < end) {
            load_aos<N>(xn, x, __ldg(ja + i + 1));
            an = __ldg(as + i + 1);
        }
        mp_t<N> p, s;
        mp_mul_d<N>(p, xv, a);
        if (i == start && zero_add_keeps<N>(p)) { /* the first step adds p to zero */
            sum = p;
            continue;
        }
        mp_add<N>(s, sum, p);
        sum = s;
    }
    store_aos<N>(sum, y, row);
}

template <int N>
__global__ void __launch_bounds__(256) spmv_csr_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y,
                                                       Sched s, int sms) {
    if (spare_block(s, m, sms, 1, CsrLen{irp})) return;
    const int lane = threadIdx.x & 31;
    for (int base = next_chunk(s.next, 32); base < m; base = next_chunk(s.next, 32)) {
        const int v = base + lane;
        if (v < m) csr_row<N>(__ldg(s.perm + v), irp, ja, as, x, y);
    }
}

template <int N, int TPR>
__global__ void __launch_bounds__(256) spmv_csrv_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                        const double *__restrict__ as, const void *x, void *y,
                                                        Sched s, int sms) {
    if (spare_block(s, m, sms, TPR, CsrLen{irp})) return;
    const int lane = threadIdx.x & 31;
    const int sub = lane & (TPR - 1), group = lane / TPR;
    constexpr int kRows = 32 / TPR;
    for (int base = next_chunk(s.next, kRows); base < m; base = next_chunk(s.next, kRows)) {
        const int v = base + group;
        const bool active = v < m;
        const int row = active ? __ldg(s.perm + v) : 0;
        mp_t<N> sum;
        set_zero<N>(sum);
        bool zero = true; /* sum is still set_zero's zero */
        if (active) {
            const int start = __ldg(irp + row), end = __ldg(irp + row + 1);
            for (int i = start + sub; i < end; i += TPR) {
                mp_t<N> xv, p, t;
                load_aos<N>(xv, x, __ldg(ja + i));
                mp_mul_d<N>(p, xv, __ldg(as + i));
                if (zero && zero_add_keeps<N>(p)) {
                    sum = p;
                } else {
                    mp_add<N>(t, sum, p);
                    sum = t;
                }
                zero = false;
            }
        }
        /* The tree adds zeros wherever a row has fewer entries than lanes (on
         * power-law rows most partial sums are zero); additions that
         * zero_add_keeps shows to return one operand unchanged are skipped.  The
         * levels stay a loop: one copy of mp_add instead of five (unrolled, the
         * kernel's instruction fetch stalled more than it issued). */
#pragma unroll 1
        for (int sft = TPR / 2; sft >= 1; sft >>= 1) {
            mp_t<N> other = shfl_down<N>(sum, sft);
            const bool other_zero = __shfl_down_sync(0xffffffffu, zero, sft);
            if (active && sub < sft) {
                if (other_zero && (zero || zero_add_keeps<N>(sum))) {
                    /* sum + 0 = sum */
                } else if (zero && zero_add_keeps<N>(other)) {
                    sum = other;
                    zero = false;
                } else {
                    mp_t<N> t;
                    mp_add<N>(t, sum, other);
                    sum = t;
                    zero = false;
                }
            }
        }
        if (active && sub == 0) store_aos<N>(sum, y, row);
    }
}

template <int N>
__global__ void __launch_bounds__(256) spmv_ell_kernel(int m, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y,
                                                       Sched s, int sms) {
    if (spare_block(s, m, sms, 1, EllEnd{s.ends})) return;
    const int lane = threadIdx.x & 31;
    for (int base = next_chunk(s.next, 32); base < m; base = next_chunk(s.next, 32)) {
        const int v = base + lane;
        if (v < m) {
            const int row = __ldg(s.perm + v);
            const int end = __ldg(s.ends + row);
            mp_t<N> sum;
            set_zero<N>(sum);
            bool zero = true;
            /* the next slot's value and column are loaded a step ahead (a slot
             * of another column is another cache line); loading its x record
             * ahead as well made the call slower (9.6 against 8.9 ms) */
            double vn = end > 0 ? __ldg(as + row) : 0.0;
            int jn = end > 0 ? __ldg(ja + row) : 0;
            for (int col = 0; col < end; col++) {
                const double val = vn;
                const int j = jn;
                if (col + 1 < end) {
                    const size_t next = (size_t)(col + 1) * m + row;
                    vn = __ldg(as + next);
                    jn = __ldg(ja + next);
                }
                if (dnz(val)) {
                    mp_t<N> xv, p, t;
                    load_aos<N>(xv, x, j);
                    mp_mul_d<N>(p, xv, val);
                    if (zero && zero_add_keeps<N>(p)) {
                        sum = p;
                    } else {
                        mp_add<N>(t, sum, p);
                        sum = t;
                    }
                    zero = false;
                }
            }
            store_aos<N>(sum, y, row);
        }
    }
}

int grid_for(int work, int threads) {
    long long g = ((long long)work + threads - 1) / threads;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

/* persistent grid: as many blocks as fit on the current device, computed once
 * per device and kernel (the kernel is the template argument: kernels of one
 * signature, such as the 8/16/32-moduli instances, must not share a size) */
template <auto Kernel> int persistent_grid(int threads) {
    static PerDevice<int> grids(positive);
    const int dev = current_device();
    const int g = grids.get(dev, 0, [&] {
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kernel, threads, 0) != cudaSuccess)
            return 0;
        return sms * (per_sm > 0 ? per_sm : 1);
    });
    return g > 0 ? g : 152;
}

bool positive_int(const int &v) { return v > 0; }
int sm_count() {
    static PerDevice<int> sms(positive_int);
    const int dev = current_device();
    const int n = sms.get(dev, 0, [&] {
        int v = 0;
        return cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess ? v : 0;
    });
    return n > 0 ? n : 152;
}

Sched carve(Workspace ws, int m) {
    int *w = static_cast<int *>(ws.ptr);
    return Sched{w, w + kBuckets, w + 2 * kBuckets, w + 512, reinterpret_cast<unsigned long long *>(w + 258),
                 w + 260, w + 512 + (size_t)m};
}

/* the workspace header (counts, cursors, counter, total, blocks per SM) is
 * cleared, the rows counted by length bucket and scattered into the sorted
 * order */
template <class Len> cudaError_t sort_rows(int m, Len lenf, Sched sc, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sc.counts, 0, sizeof(int) * 512, st);
    if (e != cudaSuccess) return e;
    bucket_count<<<grid_for(m, 256), 256, 0, st>>>(m, lenf, sc);
    bucket_offsets<<<1, 32, 0, st>>>(sc);
    bucket_scatter<<<grid_for(m, 256), 256, 0, st>>>(m, lenf, sc);
    return cudaGetLastError();
}

template <int N> cudaError_t csr(int m, const csr_t &a, const void *x, void *y, Workspace ws, cudaStream_t st) {
    Sched sc = carve(ws, m);
    cudaError_t e = sort_rows(m, CsrLen{a.irp}, sc, st);
    if (e != cudaSuccess) return e;
    spmv_csr_kernel<N><<<persistent_grid<spmv_csr_kernel<N>>(128), 128, 0, st>>>(m, a.irp, a.ja, a.as, x, y, sc,
                                                                               sm_count());
    return cudaGetLastError();
}

template <int N, int TPR>
cudaError_t csrv_t(int m, const csr_t &a, const void *x, void *y, Workspace ws, cudaStream_t st) {
    Sched sc = carve(ws, m);
    cudaError_t e = sort_rows(m, CsrLen{a.irp}, sc, st);
    if (e != cudaSuccess) return e;
    spmv_csrv_kernel<N, TPR><<<persistent_grid<spmv_csrv_kernel<N, TPR>>(128), 128, 0, st>>>(m, a.irp, a.ja, a.as,
                                                                                            x, y, sc, sm_count());
    return cudaGetLastError();
}

template <int N>
cudaError_t csrv(int m, int tpr, const csr_t &a, const void *x, void *y, Workspace ws, cudaStream_t st) {
    switch (tpr) {
    case 1: return csrv_t<N, 1>(m, a, x, y, ws, st);
    case 2: return csrv_t<N, 2>(m, a, x, y, ws, st);
    case 4: return csrv_t<N, 4>(m, a, x, y, ws, st);
    case 8: return csrv_t<N, 8>(m, a, x, y, ws, st);
    case 16: return csrv_t<N, 16>(m, a, x, y, ws, st);
    case 32: return csrv_t<N, 32>(m, a, x, y, ws, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int N>
cudaError_t ell(int m, int maxnzr, const ell_t &a, const void *x, void *y, Workspace ws, cudaStream_t st) {
    Sched sc = carve(ws, m);
    if (m > 0 && (m % 2) == 0 && (reinterpret_cast<uintptr_t>(a.as) % 16) == 0)
        ell_row_ends2<<<grid_for(m / 2, 256), 256, 0, st>>>(m, maxnzr, a.as, sc.ends);
    else if (m > 0)
        ell_row_ends<<<grid_for(m, 256), 256, 0, st>>>(m, maxnzr, a.as, sc.ends);
    cudaError_t e = sort_rows(m, EllEnd{sc.ends}, sc, st);
    if (e != cudaSuccess) return e;
    spmv_ell_kernel<N><<<persistent_grid<spmv_ell_kernel<N>>(128), 128, 0, st>>>(m, a.ja, a.as, x, y, sc, sm_count());
    return cudaGetLastError();
}

} // namespace

size_t spmv_workspace_bytes(int m) { return sizeof(int) * (2 * (size_t)m + 512); }

cudaError_t launch_spmv_csr(int nmod, int m, const csr_t &a, const void *x, void *y, Workspace ws, cudaStream_t s) {
    if (ws.bytes < spmv_workspace_bytes(m)) return cudaErrorInvalidValue;
    switch (nmod) {
    case 8: return csr<8>(m, a, x, y, ws, s);
    case 16: return csr<16>(m, a, x, y, ws, s);
    case 32: return csr<32>(m, a, x, y, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_spmv_csrv(int nmod, int m, int tpr, const csr_t &a, const void *x, void *y, Workspace ws,
                             cudaStream_t s) {
    if (ws.bytes < spmv_workspace_bytes(m)) return cudaErrorInvalidValue;
    switch (nmod) {
    case 8: return csrv<8>(m, tpr, a, x, y, ws, s);
    case 16: return csrv<16>(m, tpr, a, x, y, ws, s);
    case 32: return csrv<32>(m, tpr, a, x, y, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_spmv_ell(int nmod, int m, int maxnzr, const ell_t &a, const void *x, void *y, Workspace ws,
                            cudaStream_t s) {
    if (ws.bytes < spmv_workspace_bytes(m)) return cudaErrorInvalidValue;
    switch (nmod) {
    case 8: return ell<8>(m, maxnzr, a, x, y, ws, s);
    case 16: return ell<16>(m, maxnzr, a, x, y, ws, s);
    case 32: return ell<32>(m, maxnzr, a, x, y, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
