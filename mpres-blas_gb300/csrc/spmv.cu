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
 * counter, [257] unused, [512, 512 + m) the sorted row order. */
struct Sched {
    int *counts, *cursors, *next, *perm;
};

/* length of row r: CSR from the row pointers, ELL from its last nonzero slot */
struct CsrLen {
    const int *irp;
    __device__ int operator()(int r) const { return __ldg(irp + r + 1) - __ldg(irp + r); }
};
/* ELL: the first empty slot, found by bisection as if the stored entries of a
 * row formed a prefix (true up to explicit zeros); only the schedule uses it */
struct EllLen {
    const double *as;
    int m, maxnzr;
    __device__ int operator()(int r) const {
        int lo = 0, hi = maxnzr;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (dnz(__ldg(as + (size_t)mid * m + r))) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    }
};

template <class Len> __global__ void bucket_count(int m, Len lenf, Sched s) {
    __shared__ int hist[kBuckets];
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        atomicAdd(&hist[bucket_of(lenf(r))], 1);
    __syncthreads();
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
        if (hist[b]) atomicAdd(&s.counts[b], hist[b]);
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

template <class Len> __global__ void bucket_scatter(int m, Len lenf, Sched s) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        s.perm[atomicAdd(&s.cursors[bucket_of(lenf(r))], 1)] = r;
}

/* a warp's next chunk of `size` entries of the sorted order (-1 when exhausted) */
__device__ __forceinline__ int next_chunk(int *next, int size) {
    int base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(next, size);
    return __shfl_sync(0xffffffffu, base, 0);
}

template <int N>
__device__ __forceinline__ void csr_row(int row, const int *__restrict__ irp, const int *__restrict__ ja,
                                        const double *__restrict__ as, const void *x, void *y) {
    mp_t<N> sum;
    set_zero<N>(sum);
    const int start = __ldg(irp + row), end = __ldg(irp + row + 1);
    for (int i = start; i < end; i++) {
        mp_t<N> xv, p, s;
        load_aos<N>(xv, x, __ldg(ja + i));
        mp_mul_d<N>(p, xv, __ldg(as + i));
        mp_add<N>(s, sum, p);
        sum = s;
    }
    store_aos<N>(sum, y, row);
}

template <int N>
__global__ void __launch_bounds__(256) spmv_csr_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y,
                                                       Sched s) {
    const int lane = threadIdx.x & 31;
    for (int base = next_chunk(s.next, 32); base < m; base = next_chunk(s.next, 32)) {
        const int v = base + lane;
        if (v < m) csr_row<N>(__ldg(s.perm + v), irp, ja, as, x, y);
    }
}

template <int N, int TPR>
__global__ void __launch_bounds__(256) spmv_csrv_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                        const double *__restrict__ as, const void *x, void *y,
                                                        Sched s) {
    const int lane = threadIdx.x & 31;
    const int sub = lane & (TPR - 1), group = lane / TPR;
    constexpr int kRows = 32 / TPR;
    for (int base = next_chunk(s.next, kRows); base < m; base = next_chunk(s.next, kRows)) {
        const int v = base + group;
        const bool active = v < m;
        const int row = active ? __ldg(s.perm + v) : 0;
        mp_t<N> sum;
        set_zero<N>(sum);
        if (active) {
            const int start = __ldg(irp + row), end = __ldg(irp + row + 1);
            for (int i = start + sub; i < end; i += TPR) {
                mp_t<N> xv, p, t;
                load_aos<N>(xv, x, __ldg(ja + i));
                mp_mul_d<N>(p, xv, __ldg(as + i));
                mp_add<N>(t, sum, p);
                sum = t;
            }
        }
#pragma unroll
        for (int sft = 16; sft >= 1; sft >>= 1) {
            if (TPR >= 2 * sft) {
                mp_t<N> other = shfl_down<N>(sum, sft);
                if (active && sub < sft) {
                    mp_t<N> t;
                    mp_add<N>(t, sum, other);
                    sum = t;
                }
            }
        }
        if (active && sub == 0) store_aos<N>(sum, y, row);
    }
}

template <int N>
__global__ void __launch_bounds__(256) spmv_ell_kernel(int m, int maxnzr, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y,
                                                       Sched s) {
    const int lane = threadIdx.x & 31;
    for (int base = next_chunk(s.next, 32); base < m; base = next_chunk(s.next, 32)) {
        const int v = base + lane;
        if (v < m) {
            const int row = __ldg(s.perm + v);
            mp_t<N> sum;
            set_zero<N>(sum);
            for (int col = 0; col < maxnzr; col++) {
                const size_t slot = (size_t)col * m + row;
                const double val = __ldg(as + slot);
                if (dnz(val)) {
                    mp_t<N> xv, p, t;
                    load_aos<N>(xv, x, __ldg(ja + slot));
                    mp_mul_d<N>(p, xv, val);
                    mp_add<N>(t, sum, p);
                    sum = t;
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

/* persistent grid: as many blocks as fit on the current device (computed
 * once per device and kernel) */
template <class K> int persistent_grid(K kernel, int threads) {
    static PerDevice<int> grids(positive);
    const int dev = current_device();
    const int g = grids.get(dev, 0, [&] {
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess)
            return 0;
        return sms * (per_sm > 0 ? per_sm : 1);
    });
    return g > 0 ? g : 152;
}

Sched carve(Workspace ws, int m) {
    int *w = static_cast<int *>(ws.ptr);
    return Sched{w, w + kBuckets, w + 2 * kBuckets, w + 512};
}

template <class Len> cudaError_t sort_rows(int m, Len lenf, Sched sc, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sc.counts, 0, sizeof(int) * kBuckets, st);
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
    spmv_csr_kernel<N><<<persistent_grid(spmv_csr_kernel<N>, 128), 128, 0, st>>>(m, a.irp, a.ja, a.as, x, y, sc);
    return cudaGetLastError();
}

template <int N, int TPR>
cudaError_t csrv_t(int m, const csr_t &a, const void *x, void *y, Workspace ws, cudaStream_t st) {
    Sched sc = carve(ws, m);
    cudaError_t e = sort_rows(m, CsrLen{a.irp}, sc, st);
    if (e != cudaSuccess) return e;
    spmv_csrv_kernel<N, TPR><<<persistent_grid(spmv_csrv_kernel<N, TPR>, 128), 128, 0, st>>>(m, a.irp, a.ja, a.as,
                                                                                            x, y, sc);
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
    cudaError_t e = sort_rows(m, EllLen{a.as, m, maxnzr}, sc, st);
    if (e != cudaSuccess) return e;
    spmv_ell_kernel<N><<<persistent_grid(spmv_ell_kernel<N>, 128), 128, 0, st>>>(m, maxnzr, a.ja, a.as, x, y, sc);
    return cudaGetLastError();
}

} // namespace

size_t spmv_workspace_bytes(int m) { return sizeof(int) * ((size_t)m + 512); }

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
