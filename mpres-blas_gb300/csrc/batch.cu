/*
 * Batches of mp_gemv / mp_dot / mp_spmv_csr / csrv / ell in one persistent launch
 * (include/mpres_gb300_batch.h).  No reference counterpart: the reference
 * launches each operation separately (src/blas/gemv.cuh:151-269,
 * src/blas/dot.cuh:85-108, src/sparse/spmv/spmv_csr.cuh:49-63).
 *
 * Every output keeps the summation order of the plain kernels of this library
 * (gemv.cu, dot.cu, spmv.cu), which is the reference's:
 *   GEMV  per output, blockDim3 chains over the inner index (chain c takes
 *         c, c + b3, ...), the shared-memory tree from nextPow2(b3)/2, then
 *         y = beta*y + sum, with buffer1 = alpha*x formed first;
 *   DOT   gridDim3 first-pass blocks of blockDim3 chains (thread p of the
 *         whole grid takes products p, p + K, ...), a tree per block, then one
 *         block of blockDim3 chains and a tree over the block sums;
 *   SpMV  per row, one chain over its nonzeros (CSR; ELL over its slots,
 *         stored zeros skipped), or tpr lane-strided chains and the fixed
 *         16/8/4/2/1 tree (CSR-vector).
 * What the batch chooses -- threads per CTA, CTAs per SM, which CTA runs which
 * tile and when -- never changes a result.
 *
 * Cross-CTA data (DOT block sums) is written before a __threadfence and a
 * counter increment and read by the last CTA with L2 (.cg) loads; no CTA ever
 * waits for another.
 */
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/mpres_gb300_batch.h"
#include "batch.h"
#include "kernels.h"
#include "mp_device.cuh"
#include "gemm_chain.cuh"

MPRES_DEFINE_TABLES(batch)

namespace mpres {

struct BatchArgs {
    const GemvOp *gemv;
    const DotOp *dot;
    const SpmvOp *spmv;
    const GemmOp *gemm;
    const Task *tasks;
    int ntasks;
    int *counters; /* [0] the task counter, [1 + d] finished blocks of DOT d */
    void *buf1;    /* GEMV alpha*x, AoS */
    void *parts;   /* DOT block sums, AoS */
    const int4 *w; /* GEMM W(A), W(B) */
};

namespace {
using namespace dev;

__host__ __device__ inline unsigned next_pow2(unsigned v) {
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    return v + 1;
}

/* an AoS record written by another CTA of this launch: read through L2 */
template <int N> __device__ __forceinline__ void load_aos_cg(mp_t<N> &v, const void *base, long long i) {
    const long long *p = reinterpret_cast<const long long *>((const char *)base + (size_t)i * (4 * N + 40));
#pragma unroll
    for (int q = 0; q < N / 2; q++) {
        long long w = __ldcg(p + q);
        v.d[2 * q] = (int)(w & 0xffffffff);
        v.d[2 * q + 1] = (int)(w >> 32);
    }
    long long se = __ldcg(p + N / 2);
    v.sign = (int)(se & 0xffffffff);
    v.exp = (int)(se >> 32);
    v.ev[0].frac = __longlong_as_double(__ldcg(p + N / 2 + 1));
    v.ev[0].exp = __ldcg(p + N / 2 + 2);
    v.ev[1].frac = __longlong_as_double(__ldcg(p + N / 2 + 3));
    v.ev[1].exp = __ldcg(p + N / 2 + 4);
}

/* The element-wise passes before the persistent kernel, one chunk of one
 * operation per block: GEMV buffer1 = alpha * x, GEMM W(A) and W(B) */
template <int N>
__global__ void __launch_bounds__(256) batch_scale(const GemvOp *ops, const GemmOp *gemms, const ScaleChunk *chunks,
                                                   int nchunks, void *buf1, int4 *w) {
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const ScaleChunk ch = chunks[c];
        if (ch.kind != kChunkAlphaX) {
            const GemmOp &g = gemms[ch.op];
            const long long e = (long long)ch.start + threadIdx.x;
            if ((int)threadIdx.x < ch.count) {
                if (ch.kind == kChunkWA) prescale_element<N, true>(g.Ad, g.As, g.Ae, g.lda, g.m, e, w + g.wa);
                else prescale_element<N, false>(g.Bd, g.Bs, g.Be, g.ldb, g.k, e, w + g.wb);
            }
            continue;
        }
        const GemvOp &g = ops[ch.op];
        const int lx = g.trans ? g.m : g.n;
        const int j = ch.start + (int)threadIdx.x;
        if ((int)threadIdx.x < ch.count) {
            mp_t<N> a, v, r;
            load_soa<N>(a, g.ad, g.as, g.ae, g.av, __ldg(g.alen), 0);
            load_soa<N>(v, g.xd, g.xs, g.xe, g.xv, __ldg(g.xlen), blas_index(j, lx, g.incx));
            mp_mul<N>(r, v, a);
            store_aos<N>(r, buf1, g.buf1_off + j);
        }
    }
}

template <int N> __device__ __forceinline__ void gemv_tile(const GemvOp &g, int o0, const void *buf1, mp_t<N> *sdata) {
    const int t = threadIdx.x;
    const int b3 = g.b3, R = g.R;
    const bool trans = g.trans != 0;
    const bool mine = t < R * b3;
    const int r = trans ? t / b3 : t % R;
    const int c = trans ? t % b3 : t / R;
    const int outs = trans ? g.n : g.m, inner = trans ? g.m : g.n;
    const int o = o0 + r;
    const bool active = mine && o < outs;
    mp_t<N> acc;
    set_zero<N>(acc);
    if (active) {
        const int lena = __ldg(g.Alen);
        for (int j = c; j < inner; j += b3) {
            const long long row = trans ? j : o, col = trans ? o : j;
            mp_t<N> a, xb, p, s;
            load_soa<N>(a, g.Ad, g.As, g.Ae, g.Av, lena, col * g.lda + row);
            load_aos<N>(xb, buf1, g.buf1_off + (trans ? row : col));
            mp_mul<N>(p, a, xb);
            mp_add<N>(s, acc, p);
            acc = s;
        }
    }
    const int slot = trans ? (r * b3 + c) : (c * R + r);
    if (mine) sdata[slot] = acc;
    __syncthreads();
    for (unsigned i = next_pow2((unsigned)b3) >> 1; i >= 1; i >>= 1) {
        if (active && (unsigned)c < i && (unsigned)c + i < (unsigned)b3) {
            const int other = trans ? (r * b3 + c + (int)i) : ((c + (int)i) * R + r);
            mp_t<N> x0 = sdata[slot], x1 = sdata[other], s;
            mp_add<N>(s, x0, x1);
            sdata[slot] = s;
        }
        __syncthreads();
    }
    if (active && c == 0) {
        const int leny = __ldg(g.ylen);
        const long long iy = blas_index(o, outs, g.incy);
        mp_t<N> yv0, bv, yb, res;
        load_soa<N>(yv0, g.yd, g.ys, g.ye, g.yv, leny, iy);
        load_soa<N>(bv, g.bd, g.bs, g.be, g.bv, __ldg(g.blen), 0);
        mp_mul<N>(yb, yv0, bv);
        mp_t<N> sum = sdata[slot];
        mp_add<N>(res, yb, sum);
        store_soa<N>(res, g.yd, g.ys, g.ye, g.yv, leny, iy);
    }
}

/* tree over `len` entries of one group (CTA-wide barriers: every thread calls
 * it); groups that start at a multiple of 32 threads take tree_sum's shuffles
 * below stride 32 */
template <int N> __device__ __forceinline__ void group_tree(mp_t<N> *s, int lt, int len, bool valid, bool aligned) {
    if (aligned) {
        tree_sum<N>(s, lt, len, valid);
        return;
    }
    for (unsigned i = next_pow2((unsigned)len) >> 1; i >= 1; i >>= 1) {
        if (valid && (unsigned)lt < i && (unsigned)lt + i < (unsigned)len) {
            mp_t<N> a = s[lt], b = s[lt + i], r;
            mp_add<N>(r, a, b);
            s[lt] = r;
        }
        __syncthreads();
    }
}

template <int N>
__device__ __forceinline__ void dot_group(const DotOp &d, int dop, int b0, int nblk, void *parts, int *done,
                                          mp_t<N> *sdata, int *flag) {
    const int t = threadIdx.x, b3 = d.b3;
    const int grp = t / b3, lt = t % b3;
    const int blk = b0 + grp;
    const bool valid = grp < nblk;
    const long long K = (long long)d.g3 * b3;
    mp_t<N> acc;
    set_zero<N>(acc);
    if (valid) {
        const int lenx = __ldg(d.xlen), leny = __ldg(d.ylen);
        for (long long i = (long long)blk * b3 + lt; i < d.n; i += K) {
            mp_t<N> a, b, p, s;
            load_soa<N>(a, d.xd, d.xs, d.xe, d.xv, lenx, blas_index(i, d.n, d.incx));
            load_soa<N>(b, d.yd, d.ys, d.ye, d.yv, leny, blas_index(i, d.n, d.incy));
            mp_mul<N>(p, a, b);
            mp_add<N>(s, acc, p);
            acc = s;
        }
        sdata[t] = acc;
    }
    __syncthreads();
    group_tree<N>(sdata + grp * b3, lt, b3, valid, (b3 & 31) == 0);
    if (valid && lt == 0) store_aos<N>(sdata[t], parts, d.part_off + blk);
    __threadfence();
    __syncthreads();
    if (t == 0) *flag = (atomicAdd(done + dop, nblk) + nblk == d.g3);
    __syncthreads();
    if (!*flag) return;
    /* the last group of this DOT: its second pass (dot.cu's dot_pass2) */
    __threadfence();
    const bool in2 = t < b3;
    set_zero<N>(acc);
    if (in2)
        for (int i = t; i < d.g3; i += b3) {
            mp_t<N> b, s;
            load_aos_cg<N>(b, parts, d.part_off + i);
            mp_add<N>(s, acc, b);
            acc = s;
        }
    if (in2) sdata[t] = acc;
    __syncthreads();
    group_tree<N>(sdata, t, b3, in2, true);
    if (t == 0) store_soa<N>(sdata[0], d.rd, d.rs, d.re, d.rv, __ldg(d.rlen), 0);
}

/* shuffle a whole number down by delta lanes */
template <int N> __device__ __forceinline__ mp_t<N> shfl_down(const mp_t<N> &v, int delta) {
    mp_t<N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = __shfl_down_sync(0xffffffffu, v.d[i], delta);
    r.sign = __shfl_down_sync(0xffffffffu, v.sign, delta);
    r.exp = __shfl_down_sync(0xffffffffu, v.exp, delta);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        r.ev[k].frac = __shfl_down_sync(0xffffffffu, v.ev[k].frac, delta);
        r.ev[k].exp = __shfl_down_sync(0xffffffffu, v.ev[k].exp, delta);
    }
    return r;
}

/* `rows` rows of the length-sorted order from `first`, in the operation's form
 * (spmv.cu: spmv_csr_kernel, spmv_csrv_kernel, spmv_ell_kernel); every thread of
 * the CTA calls it (the CSR-vector tree shuffles across whole warps) */
template <int N> __device__ __forceinline__ void spmv_chunk(const SpmvOp &s, int first, int rows) {
    const int t = threadIdx.x;
    if (s.form == kCsrv) {
        const int tpr = s.tpr, group = t / tpr, sub = t % tpr;
        const bool active = group < rows;
        const int row = active ? __ldg(s.perm + first + group) : 0;
        mp_t<N> sum;
        set_zero<N>(sum);
        bool zero = true; /* sum is still set_zero's zero (see zero_add_keeps) */
        if (active) {
            const int start = __ldg(s.irp + row), end = __ldg(s.irp + row + 1);
            for (int i = start + sub; i < end; i += tpr) {
                mp_t<N> xv, p, q;
                load_aos<N>(xv, s.x, __ldg(s.ja + i));
                mp_mul_d<N>(p, xv, __ldg(s.as + i));
                if (zero && zero_add_keeps<N>(p)) {
                    sum = p;
                } else {
                    mp_add<N>(q, sum, p);
                    sum = q;
                }
                zero = false;
            }
        }
        /* the fixed tree of src/sparse/spmv/spmv_csrv.cuh:70-84; additions of a
         * zero that return the other operand unchanged are skipped (a loop, so
         * that one copy of mp_add serves every level) */
#pragma unroll 1
        for (int sft = 16; sft >= 1; sft >>= 1) {
            if (tpr >= 2 * sft) {
                mp_t<N> other = shfl_down<N>(sum, sft);
                const bool other_zero = __shfl_down_sync(0xffffffffu, zero, sft);
                if (active && sub < sft) {
                    if (other_zero && (zero || zero_add_keeps<N>(sum))) {
                    } else if (zero && zero_add_keeps<N>(other)) {
                        sum = other;
                        zero = false;
                    } else {
                        mp_t<N> q;
                        mp_add<N>(q, sum, other);
                        sum = q;
                        zero = false;
                    }
                }
            }
        }
        if (active && sub == 0) store_aos<N>(sum, s.y, row);
        return;
    }
    if (t >= rows) return;
    const int row = __ldg(s.perm + first + t);
    mp_t<N> sum;
    set_zero<N>(sum);
    bool zero = true;
    if (s.form == kEll) {
        for (int col = 0; col < s.maxnzr; col++) {
            const size_t slot = (size_t)col * s.m + row;
            const double val = __ldg(s.as + slot);
            if (dnz(val)) {
                mp_t<N> xv, p, q;
                load_aos<N>(xv, s.x, __ldg(s.ja + slot));
                mp_mul_d<N>(p, xv, val);
                if (zero && zero_add_keeps<N>(p)) {
                    sum = p;
                } else {
                    mp_add<N>(q, sum, p);
                    sum = q;
                }
                zero = false;
            }
        }
    } else {
        const int start = __ldg(s.irp + row), end = __ldg(s.irp + row + 1);
        for (int i = start; i < end; i++) {
            mp_t<N> xv, p, q;
            load_aos<N>(xv, s.x, __ldg(s.ja + i));
            mp_mul_d<N>(p, xv, __ldg(s.as + i));
            if (zero && zero_add_keeps<N>(p)) {
                sum = p;
            } else {
                mp_add<N>(q, sum, p);
                sum = q;
            }
            zero = false;
        }
    }
    store_aos<N>(sum, s.y, row);
}

/* ELL row lengths for the schedule: the first empty slot, by bisection as if
 * the stored entries of a row formed a prefix (spmv.cu's EllLen) */
__global__ void ell_row_lengths(const double *as, int m, int maxnzr, int *len) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        int lo = 0, hi = maxnzr;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (dnz(__ldg(as + (size_t)mid * m + r))) lo = mid + 1;
            else hi = mid;
        }
        len[r] = lo;
    }
}

/* a 32 x (threads / 32) tile of a GEMM: one output per thread, the lazy-residue
 * chain of gemm_chain.cuh (the k order is the reference's, so the tile shape
 * never enters a result) */
template <int N> __device__ __forceinline__ void gemm_tile(const GemmOp &g, int r0, int c0, const int4 *w) {
    const int row = r0 + (int)(threadIdx.x & 31), col = c0 + (int)(threadIdx.x >> 5);
    if (row >= g.m || col >= g.n) return;
    const MatSoA al{g.ad, g.as, g.ae, g.av, g.alen}, A{g.Ad, g.As, g.Ae, g.Av, g.Alen};
    const MatSoA B{g.Bd, g.Bs, g.Be, g.Bv, g.Blen}, be{g.bd, g.bs, g.be, g.bv, g.blen};
    gemm_lazy_output<N>(g.m, g.k, al, A, g.lda, B, g.ldb, be, g.Cd, g.Cs, g.Ce, g.Cv, g.Clen, g.ldc, w + g.wa,
                        w + g.wb, row, col);
}

/* The persistent kernel.  Variants with GEMM tiles (GEMM = true) are separate
 * instantiations: the k chain's registers would otherwise lower the occupancy
 * of batches without GEMMs.  They exist for 128 threads (three CTAs an SM, as
 * the plain GEMM kernel) and 256. */
template <int N, int MAXT, bool GEMM>
__global__ void __launch_bounds__(MAXT, (GEMM && MAXT == 128) ? 3 : 1) batch_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    __shared__ int s_task, s_flag;
    for (;;) {
        if (threadIdx.x == 0) s_task = atomicAdd(a.counters, 1);
        __syncthreads();
        const int ti = s_task;
        if (ti >= a.ntasks) break;
        const Task tk = a.tasks[ti];
        if (tk.kind == kGemvTile) gemv_tile<N>(a.gemv[tk.op], tk.a, a.buf1, sdata);
        else if (tk.kind == kDotGroup) dot_group<N>(a.dot[tk.op], tk.op, tk.a, tk.b, a.parts, a.counters + 1, sdata, &s_flag);
        else if (GEMM && tk.kind == kGemmTile) gemm_tile<N>(a.gemm[tk.op], tk.a, tk.b, a.w);
        else spmv_chunk<N>(a.spmv[tk.op], tk.a, tk.b);
        __syncthreads();
    }
}

/* snapshot / restore of every GEMM output C (column-major, ldc), for autotuning */
template <int N> __global__ void gemm_c_copy(const GemmOp *ops, int nops, const long long *offs, void *save, int dir) {
    const int op = blockIdx.y;
    if (op >= nops) return;
    const GemmOp &g = ops[op];
    const long long outs = (long long)g.m * g.n;
    const int lenc = __ldg(g.Clen);
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < outs; o += (long long)gridDim.x * blockDim.x) {
        const long long ic = (o / g.m) * g.ldc + o % g.m;
        mp_t<N> v;
        if (dir == 0) {
            load_soa<N>(v, g.Cd, g.Cs, g.Ce, g.Cv, lenc, ic);
            store_aos<N>(v, save, offs[op] + o);
        } else {
            load_aos<N>(v, save, offs[op] + o);
            store_soa<N>(v, g.Cd, g.Cs, g.Ce, g.Cv, lenc, ic);
        }
    }
}

/* snapshot / restore of every GEMV output, for autotuning on the batch itself */
template <int N> __global__ void gemv_y_copy(const GemvOp *ops, int nops, const long long *offs, void *save, int dir) {
    const int op = blockIdx.y;
    if (op >= nops) return;
    const GemvOp &g = ops[op];
    const int outs = g.trans ? g.n : g.m;
    const int leny = __ldg(g.ylen);
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < outs; o += gridDim.x * blockDim.x) {
        const long long iy = blas_index(o, outs, g.incy);
        mp_t<N> v;
        if (dir == 0) {
            load_soa<N>(v, g.yd, g.ys, g.ye, g.yv, leny, iy);
            store_aos<N>(v, save, offs[op] + o);
        } else {
            load_aos<N>(v, save, offs[op] + o);
            store_soa<N>(v, g.yd, g.ys, g.ye, g.yv, leny, iy);
        }
    }
}

} // namespace

/* ------------------------------ host helpers ------------------------------ */

namespace {

er_t *ev(const mp_array_t &a) { return reinterpret_cast<er_t *>(a.eval); }

/* autotuned shapes per (moduli set, device): {threads per CTA, CTAs per SM} */
std::vector<int> g_shape_cache[3 * 64];
std::mutex g_shape_mu;

int shape_slot(int nmod) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int si = nmod == 8 ? 0 : nmod == 16 ? 1 : 2;
    return si * 64 + (dev >= 0 && dev < 64 ? dev : 0);
}

/* the kernel's shared-memory limit, raised on each device that runs a variant */
template <int N, int MAXT, bool GEMM> cudaError_t set_attr() {
    static PerDevice<cudaError_t> attrs(cuda_ok);
    return attrs.get(current_device(), cudaErrorInvalidDevice, [] {
        return cudaFuncSetAttribute(batch_kernel<N, MAXT, GEMM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    MAXT * (int)sizeof(mp_t<N>));
    });
}

template <int N, int MAXT, bool GEMM> int occupancy(int threads) {
    int per_sm = 0;
    if (set_attr<N, MAXT, GEMM>() != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<N, MAXT, GEMM>, threads,
                                                      (size_t)threads * sizeof(mp_t<N>)) != cudaSuccess)
        return 0;
    return per_sm;
}

template <int N, int MAXT, bool GEMM>
cudaError_t launch_variant(const BatchArgs &a, int threads, int ctas, cudaStream_t s) {
    cudaError_t e = set_attr<N, MAXT, GEMM>();
    if (e != cudaSuccess) return e;
    batch_kernel<N, MAXT, GEMM><<<ctas, threads, (size_t)threads * sizeof(mp_t<N>), s>>>(a);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_n(const BatchHost &b, const BatchDev &d, int threads, int ctas, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d.counters, 0, sizeof(int) * (1 + b.dot.size()), s);
    if (e != cudaSuccess) return e;
    if (!b.chunks.empty()) {
        const int g = (int)std::min<size_t>(b.chunks.size(), 152 * 16);
        batch_scale<N><<<g, 256, 0, s>>>(d.gemv, d.gemm, d.chunks, (int)b.chunks.size(), d.buf1,
                                         static_cast<int4 *>(d.w));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (b.tasks.empty()) return cudaSuccess;
    BatchArgs a{d.gemv, d.dot, d.spmv, d.gemm, d.tasks, (int)b.tasks.size(), d.counters, d.buf1, d.parts,
                static_cast<const int4 *>(d.w)};
    /* register budgets: 128-thread GEMM CTAs up to 168 registers a thread,
     * 256-thread CTAs up to 255, 512 up to 128, 1024 up to 64 */
    if (!b.gemm.empty()) {
        if (threads <= 128) return launch_variant<N, 128, true>(a, threads, ctas, s);
        if (threads <= 256) return launch_variant<N, 256, true>(a, threads, ctas, s);
        return cudaErrorInvalidConfiguration;
    }
    if (threads <= 256) return launch_variant<N, 256, false>(a, threads, ctas, s);
    if (threads <= 512) return launch_variant<N, 512, false>(a, threads, ctas, s);
    return launch_variant<N, 1024, false>(a, threads, ctas, s);
}

template <class T> size_t bytes_of(const std::vector<T> &v) { return sizeof(T) * v.size(); }
size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

} // namespace

bool batch_add_gemv(BatchHost &b, int trans, int m, int n, const mp_array_t &alpha, const mp_array_t &A, int lda,
                    const mp_array_t &x, int incx, const mp_array_t &beta, const mp_array_t &y, int incy, int b3) {
    /* the quick returns of src/blas/gemv.cuh:155-161 */
    if (m <= 0 || n <= 0 || incx == 0 || incy == 0 || lda < (m > 1 ? m : 1)) return false;
    GemvOp g{};
    g.Ad = A.digits; g.As = A.sign; g.Ae = A.exp; g.Av = ev(A); g.Alen = A.len;
    g.xd = x.digits; g.xs = x.sign; g.xe = x.exp; g.xv = ev(x); g.xlen = x.len;
    g.ad = alpha.digits; g.as = alpha.sign; g.ae = alpha.exp; g.av = ev(alpha); g.alen = alpha.len;
    g.bd = beta.digits; g.bs = beta.sign; g.be = beta.exp; g.bv = ev(beta); g.blen = beta.len;
    g.yd = y.digits; g.ys = y.sign; g.ye = y.exp; g.yv = ev(y); g.ylen = y.len;
    g.m = m; g.n = n; g.lda = lda; g.incx = incx; g.incy = incy;
    g.trans = trans != MPRES_NO_TRANS;
    g.b3 = b3;
    g.buf1_off = b.buf1_elems;
    b.buf1_elems += g.trans ? m : n;
    b.gemv.push_back(g);
    return true;
}

bool batch_add_dot(BatchHost &b, int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy,
                   const mp_array_t &r, int g3, int b3) {
    if (n <= 0) return false; /* src/blas/dot.cuh:88-90 */
    DotOp d{};
    d.xd = x.digits; d.xs = x.sign; d.xe = x.exp; d.xv = ev(x); d.xlen = x.len;
    d.yd = y.digits; d.ys = y.sign; d.ye = y.exp; d.yv = ev(y); d.ylen = y.len;
    d.rd = r.digits; d.rs = r.sign; d.re = r.exp; d.rv = ev(r); d.rlen = r.len;
    d.n = n; d.incx = incx; d.incy = incy; d.g3 = g3; d.b3 = b3;
    d.part_off = b.part_elems;
    b.part_elems += g3;
    b.dot.push_back(d);
    return true;
}

void batch_add_spmv(BatchHost &b, int m, const csr_t &csr, const void *x, void *y, const int *perm,
                    std::vector<int> lens, int form, int tpr) {
    SpmvOp sp{};
    sp.irp = csr.irp; sp.ja = csr.ja; sp.as = csr.as; sp.x = x; sp.y = y; sp.m = m; sp.perm = perm;
    sp.form = form;
    sp.tpr = tpr;
    b.spmv.push_back(sp);
    b.spmv_len.push_back(std::move(lens));
}

void batch_add_spmv_ell(BatchHost &b, int m, int maxnzr, const ell_t &ell, const void *x, void *y) {
    SpmvOp sp{};
    sp.ja = ell.ja; sp.as = ell.as; sp.x = x; sp.y = y; sp.m = m;
    sp.form = kEll;
    sp.tpr = 1;
    sp.maxnzr = maxnzr;
    b.spmv.push_back(sp);
    b.spmv_len.push_back({});
}

bool batch_add_gemm(BatchHost &b, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                    const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc, int nmod) {
    /* the quick returns of src/blas/gemm.cuh:77-96 (no transposition) */
    if (m <= 0 || n <= 0 || k <= 0 || lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
        return false;
    GemmOp g{};
    g.ad = alpha.digits; g.as = alpha.sign; g.ae = alpha.exp; g.av = ev(alpha); g.alen = alpha.len;
    g.Ad = A.digits; g.As = A.sign; g.Ae = A.exp; g.Av = ev(A); g.Alen = A.len;
    g.Bd = B.digits; g.Bs = B.sign; g.Be = B.exp; g.Bv = ev(B); g.Blen = B.len;
    g.bd = beta.digits; g.bs = beta.sign; g.be = beta.exp; g.bv = ev(beta); g.blen = beta.len;
    g.Cd = C.digits; g.Cs = C.sign; g.Ce = C.exp; g.Cv = ev(C); g.Clen = C.len;
    g.m = m; g.n = n; g.k = k; g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    const long long q = nmod / 4;
    g.wa = b.w_elems;
    b.w_elems += (long long)m * k * q;
    g.wb = b.w_elems;
    b.w_elems += (long long)k * n * q;
    b.gemm.push_back(g);
    return true;
}

void spmv_row_order(const int *irp, int m, std::vector<int> &order, std::vector<int> &lens) {
    /* counting sort by length, longest first, rows of equal length in order */
    int maxlen = 0;
    for (int r = 0; r < m; r++) maxlen = std::max(maxlen, irp[r + 1] - irp[r]);
    std::vector<int> start((size_t)maxlen + 2, 0);
    for (int r = 0; r < m; r++) start[(size_t)(maxlen - (irp[r + 1] - irp[r])) + 1]++;
    for (int k = 1; k <= maxlen + 1; k++) start[k] += start[k - 1];
    order.assign((size_t)m, 0);
    for (int r = 0; r < m; r++) order[start[(size_t)(maxlen - (irp[r + 1] - irp[r]))]++] = r;
    lens.resize((size_t)m);
    for (int r = 0; r < m; r++) lens[r] = irp[order[r] + 1] - irp[order[r]];
}

bool batch_plan(BatchHost &b, int threads) {
    struct Item {
        long long cost;
        Task t;
    };
    std::vector<Item> items;
    b.chunks.clear();
    for (size_t i = 0; i < b.gemv.size(); i++) {
        GemvOp &g = b.gemv[i];
        if (g.b3 > threads) return false;
        g.R = threads / g.b3;
        const int outs = g.trans ? g.n : g.m, inner = g.trans ? g.m : g.n;
        /* chain length in multiply-add steps, plus the tree */
        const long long cost = (inner + g.b3 - 1) / g.b3 + 2 * (32 - __builtin_clz((unsigned)g.b3));
        for (int o = 0; o < outs; o += g.R) items.push_back({cost, {kGemvTile, (int)i, o, 0}});
        for (int j = 0; j < inner; j += 256) b.chunks.push_back({(int)i, j, std::min(256, inner - j), kChunkAlphaX});
    }
    for (size_t i = 0; i < b.dot.size(); i++) {
        DotOp &d = b.dot[i];
        if (d.b3 > threads) return false;
        d.groups = threads / d.b3;
        const long long K = (long long)d.g3 * d.b3;
        const long long cost = (d.n + K - 1) / K + 2 * (32 - __builtin_clz((unsigned)d.b3));
        for (int blk = 0; blk < d.g3; blk += d.groups)
            items.push_back({cost, {kDotGroup, (int)i, blk, std::min(d.groups, d.g3 - blk)}});
    }
    for (size_t i = 0; i < b.spmv.size(); i++) {
        const SpmvOp &sp = b.spmv[i];
        const std::vector<int> &len = b.spmv_len[i];
        if (sp.form == kCsrv && sp.tpr > threads) return false;
        /* rows per task: one thread per row, or tpr threads per row */
        const int rows = sp.form == kCsrv ? threads / sp.tpr : threads;
        for (int r = 0; r < sp.m; r += rows) {
            long long cost = (long long)len[r] + 1;
            if (sp.form == kCsrv) cost = (len[r] + sp.tpr - 1) / sp.tpr + (32 - __builtin_clz((unsigned)sp.tpr));
            items.push_back({cost, {kSpmvChunk, (int)i, r, std::min(rows, sp.m - r)}});
        }
    }
    for (size_t i = 0; i < b.gemm.size(); i++) {
        const GemmOp &g = b.gemm[i];
        if (threads > 256) return false;
        const int cols = threads / 32;
        /* cost in chain steps: the k chain, then the epilogue's products and addition */
        const long long cost = g.k + 8;
        for (int r = 0; r < g.m; r += 32)
            for (int c = 0; c < g.n; c += cols) items.push_back({cost, {kGemmTile, (int)i, r, c}});
        const long long na = (long long)g.m * g.k, nb = (long long)g.k * g.n;
        for (long long e = 0; e < na; e += 256)
            b.chunks.push_back({(int)i, (int)e, (int)std::min<long long>(256, na - e), kChunkWA});
        for (long long e = 0; e < nb; e += 256)
            b.chunks.push_back({(int)i, (int)e, (int)std::min<long long>(256, nb - e), kChunkWB});
    }
    std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) { return x.cost > y.cost; });
    b.tasks.resize(items.size());
    for (size_t i = 0; i < items.size(); i++) b.tasks[i] = items[i].t;
    return true;
}

TableLayout batch_layout(const BatchHost &b) {
    TableLayout l;
    l.gemv = 0;
    l.dot = align256(l.gemv + bytes_of(b.gemv));
    l.spmv = align256(l.dot + bytes_of(b.dot));
    l.gemm = align256(l.spmv + bytes_of(b.spmv));
    l.tasks = align256(l.gemm + bytes_of(b.gemm));
    l.chunks = align256(l.tasks + bytes_of(b.tasks));
    l.counters = align256(l.chunks + bytes_of(b.chunks));
    l.total = align256(l.counters + sizeof(int) * (1 + b.dot.size()));
    return l;
}

void batch_pack(const BatchHost &b, const TableLayout &l, void *host_buf) {
    char *p = static_cast<char *>(host_buf);
    if (!b.gemv.empty()) std::memcpy(p + l.gemv, b.gemv.data(), bytes_of(b.gemv));
    if (!b.dot.empty()) std::memcpy(p + l.dot, b.dot.data(), bytes_of(b.dot));
    if (!b.spmv.empty()) std::memcpy(p + l.spmv, b.spmv.data(), bytes_of(b.spmv));
    if (!b.gemm.empty()) std::memcpy(p + l.gemm, b.gemm.data(), bytes_of(b.gemm));
    if (!b.tasks.empty()) std::memcpy(p + l.tasks, b.tasks.data(), bytes_of(b.tasks));
    if (!b.chunks.empty()) std::memcpy(p + l.chunks, b.chunks.data(), bytes_of(b.chunks));
}

BatchDev batch_dev_at(const BatchHost &b, const TableLayout &l, void *dev_buf, void *buf1, void *parts, void *w) {
    (void)b;
    char *p = static_cast<char *>(dev_buf);
    BatchDev d;
    d.gemv = reinterpret_cast<GemvOp *>(p + l.gemv);
    d.dot = reinterpret_cast<DotOp *>(p + l.dot);
    d.spmv = reinterpret_cast<SpmvOp *>(p + l.spmv);
    d.gemm = reinterpret_cast<GemmOp *>(p + l.gemm);
    d.w = w;
    d.tasks = reinterpret_cast<Task *>(p + l.tasks);
    d.chunks = reinterpret_cast<ScaleChunk *>(p + l.chunks);
    d.counters = reinterpret_cast<int *>(p + l.counters);
    d.buf1 = buf1;
    d.parts = parts;
    return d;
}

cudaError_t batch_launch(int nmod, const BatchHost &b, const BatchDev &d, int threads, int ctas, cudaStream_t s) {
    switch (nmod) {
    case 8: return launch_n<8>(b, d, threads, ctas, s);
    case 16: return launch_n<16>(b, d, threads, ctas, s);
    case 32: return launch_n<32>(b, d, threads, ctas, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int N> int ctas_per_sm_n(int threads, bool gemm) {
    if (gemm) return threads <= 128 ? occupancy<N, 128, true>(threads)
                                    : (threads <= 256 ? occupancy<N, 256, true>(threads) : 0);
    return threads <= 256 ? occupancy<N, 256, false>(threads)
                          : (threads <= 512 ? occupancy<N, 512, false>(threads) : occupancy<N, 1024, false>(threads));
}

int batch_ctas_per_sm(int nmod, int threads, bool gemm) {
    if (nmod == 8) return ctas_per_sm_n<8>(threads, gemm);
    if (nmod == 16) return ctas_per_sm_n<16>(threads, gemm);
    if (nmod == 32) return ctas_per_sm_n<32>(threads, gemm);
    return 0;
}

bool batch_cached_shape(int nmod, int &threads, int &per_sm) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    const std::vector<int> &c = g_shape_cache[shape_slot(nmod)];
    if (c.empty()) return false;
    threads = c[0];
    per_sm = c[1];
    return true;
}

static void cache_shape(int nmod, int threads, int per_sm) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_shape_cache[shape_slot(nmod)] = {threads, per_sm};
}

/* snapshot (dir 0) or restore (dir 1) of every output a run accumulates into
 * (GEMV y, GEMM C): offs[op] for the GEMVs, then for the GEMMs */
static cudaError_t gemv_outputs(int nmod, const BatchHost &b, const BatchDev &d, const long long *offs, void *save,
                                int dir, cudaStream_t s) {
    if (!b.gemv.empty()) {
        dim3 grid(8, (unsigned)b.gemv.size());
        const int nops = (int)b.gemv.size();
        switch (nmod) {
        case 8: gemv_y_copy<8><<<grid, 256, 0, s>>>(d.gemv, nops, offs, save, dir); break;
        case 16: gemv_y_copy<16><<<grid, 256, 0, s>>>(d.gemv, nops, offs, save, dir); break;
        case 32: gemv_y_copy<32><<<grid, 256, 0, s>>>(d.gemv, nops, offs, save, dir); break;
        default: return cudaErrorInvalidValue;
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (!b.gemm.empty()) {
        dim3 grid(64, (unsigned)b.gemm.size());
        const int nops = (int)b.gemm.size();
        const long long *go = offs + b.gemv.size();
        switch (nmod) {
        case 8: gemm_c_copy<8><<<grid, 256, 0, s>>>(d.gemm, nops, go, save, dir); break;
        case 16: gemm_c_copy<16><<<grid, 256, 0, s>>>(d.gemm, nops, go, save, dir); break;
        case 32: gemm_c_copy<32><<<grid, 256, 0, s>>>(d.gemm, nops, go, save, dir); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    return cudaSuccess;
}

} // namespace mpres

/* ------------------------------- C entry points --------------------------- */

using namespace mpres;

struct mpres_batch {
    int nmod = 0, device = 0;
    bool committed = false;
    BatchHost host;
    void *tables = nullptr; /* device tables (batch_layout) */
    void *buf1 = nullptr, *parts = nullptr, *w = nullptr;
    int *perm = nullptr;
    BatchDev dev;
    int threads = 256, ctas = 0, candidates = 0;
    bool autotuned = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static void release(mpres_batch *b) {
    for (void *p : {b->tables, b->buf1, b->parts, b->w, (void *)b->perm})
        if (p) cudaFree(p);
    b->tables = b->buf1 = b->parts = b->w = nullptr;
    b->perm = nullptr;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

/* plans for `threads` and uploads the tables (reallocating them if they grew) */
static cudaError_t plan_and_upload(mpres_batch *b, int threads, size_t &cap) {
    batch_plan(b->host, threads);
    const TableLayout l = batch_layout(b->host);
    cudaError_t e;
    if (l.total > cap) {
        if (b->tables) cudaFree(b->tables);
        b->tables = nullptr;
        cap = 0;
        if ((e = cudaMalloc(&b->tables, l.total)) != cudaSuccess) return e;
        cap = l.total;
    }
    std::vector<char> staging(l.total);
    batch_pack(b->host, l, staging.data());
    if ((e = cudaMemcpy(b->tables, staging.data(), l.total, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    b->dev = batch_dev_at(b->host, l, b->tables, b->buf1, b->parts, b->w);
    return cudaSuccess;
}

extern "C" {

int mpres_batch_create(int nmod, mpres_batch_t **batch) {
    if (!batch) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_create: null handle");
    if (int st = status_require(nmod)) return st;
    mpres_batch *b = new (std::nothrow) mpres_batch;
    if (!b) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_create: out of host memory");
    b->nmod = nmod;
    cudaGetDevice(&b->device);
    *batch = b;
    return status_ok();
}

int mpres_batch_destroy(mpres_batch_t *b) {
    if (!b) return status_ok();
    release(b);
    delete b;
    return status_ok();
}

static int check_open(mpres_batch *b, const char *what) {
    if (!b) return status_fail(MPRES_ERR_INVALID_VALUE, "%s: null batch", what);
    if (b->committed) return status_fail(MPRES_ERR_INVALID_VALUE, "%s: the batch is committed", what);
    return MPRES_SUCCESS;
}

int mpres_batch_add_gemv(mpres_batch_t *b, int trans, int m, int n, const mp_array_t *alpha, const mp_array_t *A,
                         int lda, const mp_array_t *x, int incx, const mp_array_t *beta, const mp_array_t *y, int incy,
                         int blockDim3) {
    if (int st = check_open(b, "mpres_batch_add_gemv")) return st;
    if (m <= 0 || n <= 0 || incx == 0 || incy == 0 || lda < (m > 1 ? m : 1)) return status_ok();
    if (!alpha || !A || !x || !beta || !y) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_gemv: null array");
    if (blockDim3 <= 0 || blockDim3 > 1024)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_gemv: blockDim3 %d out of range", blockDim3);
    batch_add_gemv(b->host, trans, m, n, *alpha, *A, lda, *x, incx, *beta, *y, incy, blockDim3);
    return status_ok();
}

int mpres_batch_add_dot(mpres_batch_t *b, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy,
                        const mp_array_t *r, int gridDim3, int blockDim3) {
    if (int st = check_open(b, "mpres_batch_add_dot")) return st;
    if (n <= 0) return status_ok();
    if (!x || !y || !r) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_dot: null array");
    if (gridDim3 <= 0 || blockDim3 <= 0 || blockDim3 > 1024)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_dot: gridDim3 %d / blockDim3 %d out of range",
                           gridDim3, blockDim3);
    batch_add_dot(b->host, n, *x, incx, *y, incy, *r, gridDim3, blockDim3);
    return status_ok();
}

int mpres_batch_add_spmv_csr(mpres_batch_t *b, int m, const csr_t *csr, const void *x, void *y) {
    if (int st = check_open(b, "mpres_batch_add_spmv_csr")) return st;
    if (m <= 0) return status_ok();
    if (!csr || !x || !y) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_spmv_csr: null argument");
    batch_add_spmv(b->host, m, *csr, x, y, nullptr, {});
    return status_ok();
}

int mpres_batch_add_spmv_csrv(mpres_batch_t *b, int m, const csr_t *csr, const void *x, void *y, int threadsPerRow) {
    if (int st = check_open(b, "mpres_batch_add_spmv_csrv")) return st;
    if (threadsPerRow < 1 || threadsPerRow > 32 || (threadsPerRow & (threadsPerRow - 1)))
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_spmv_csrv: threadsPerRow %d not a power of two <= 32",
                           threadsPerRow);
    if (m <= 0) return status_ok();
    if (!csr || !x || !y) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_spmv_csrv: null argument");
    batch_add_spmv(b->host, m, *csr, x, y, nullptr, {}, kCsrv, threadsPerRow);
    return status_ok();
}

int mpres_batch_add_spmv_ell(mpres_batch_t *b, int m, int maxnzr, const ell_t *ell, const void *x, void *y) {
    if (int st = check_open(b, "mpres_batch_add_spmv_ell")) return st;
    if (m <= 0) return status_ok();
    if (maxnzr < 0 || !ell || !x || !y) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_spmv_ell: bad argument");
    batch_add_spmv_ell(b->host, m, maxnzr, *ell, x, y);
    return status_ok();
}

int mpres_batch_add_gemm(mpres_batch_t *b, int transa, int transb, int m, int n, int k, const mp_array_t *alpha,
                         const mp_array_t *A, int lda, const mp_array_t *B, int ldb, const mp_array_t *beta,
                         mp_array_t *C, int ldc) {
    if (int st = check_open(b, "mpres_batch_add_gemm")) return st;
    if (m <= 0 || n <= 0 || k <= 0) return status_ok();
    if (transa != MPRES_NO_TRANS || transb != MPRES_NO_TRANS)
        return status_fail(MPRES_ERR_NOT_SUPPORTED, "mpres_batch_add_gemm: only non-transposed matrices are supported");
    if (!alpha || !A || !B || !beta || !C) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_add_gemm: null array");
    if ((long long)m * k >= (1ll << 31) || (long long)k * n >= (1ll << 31))
        return status_fail(MPRES_ERR_NOT_SUPPORTED, "mpres_batch_add_gemm: m*k and k*n must stay below 2^31");
    batch_add_gemm(b->host, m, n, k, *alpha, *A, lda, *B, ldb, *beta, *C, ldc, b->nmod);
    return status_ok();
}

int mpres_batch_commit(mpres_batch_t *b, unsigned flags, void *stream) {
    if (int st = check_open(b, "mpres_batch_commit")) return st;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != b->device)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_commit: batch made on device %d", b->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t rec = 4 * (size_t)b->nmod + 40;
    cudaError_t e;
    BatchHost &h = b->host;
    /* SpMV: rows by length, longest first, from the row pointers */
    std::vector<int> perm_all;
    std::vector<size_t> perm_off;
    for (size_t i = 0; i < h.spmv.size(); i++) {
        SpmvOp &sp = h.spmv[i];
        std::vector<int> irp((size_t)sp.m + 1), order;
        if (sp.form == kEll) {
            /* ELL: row lengths found on the device, as row pointers for the order */
            int *dlen = nullptr;
            std::vector<int> len((size_t)sp.m);
            if ((e = cudaMalloc(&dlen, sizeof(int) * (size_t)sp.m)) != cudaSuccess)
                return status_cuda(e, "mpres_batch_commit (ELL row lengths)");
            ell_row_lengths<<<std::min(4096, (sp.m + 255) / 256), 256, 0, s>>>(sp.as, sp.m, sp.maxnzr, dlen);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e == cudaSuccess) e = cudaMemcpy(len.data(), dlen, sizeof(int) * len.size(), cudaMemcpyDeviceToHost);
            cudaFree(dlen);
            if (e != cudaSuccess) return status_cuda(e, "mpres_batch_commit (ELL row lengths)");
            irp[0] = 0;
            for (int r = 0; r < sp.m; r++) irp[(size_t)r + 1] = irp[r] + len[r];
        } else if ((e = cudaMemcpy(irp.data(), sp.irp, sizeof(int) * irp.size(), cudaMemcpyDeviceToHost)) !=
                   cudaSuccess) {
            return status_cuda(e, "mpres_batch_commit (row pointers)");
        }
        spmv_row_order(irp.data(), sp.m, order, h.spmv_len[i]);
        perm_off.push_back(perm_all.size());
        perm_all.insert(perm_all.end(), order.begin(), order.end());
    }
    if (!perm_all.empty()) {
        if ((e = cudaMalloc(&b->perm, sizeof(int) * perm_all.size())) != cudaSuccess ||
            (e = cudaMemcpy(b->perm, perm_all.data(), sizeof(int) * perm_all.size(), cudaMemcpyHostToDevice)) !=
                cudaSuccess)
            return status_cuda(e, "mpres_batch_commit (row order)");
        for (size_t i = 0; i < h.spmv.size(); i++) h.spmv[i].perm = b->perm + perm_off[i];
    }
    if (h.buf1_elems && (e = cudaMalloc(&b->buf1, rec * h.buf1_elems)) != cudaSuccess)
        return status_cuda(e, "mpres_batch_commit (alpha*x)");
    if (h.part_elems && (e = cudaMalloc(&b->parts, rec * h.part_elems)) != cudaSuccess)
        return status_cuda(e, "mpres_batch_commit (block sums)");
    if (h.w_elems && (e = cudaMalloc(&b->w, sizeof(int4) * (size_t)h.w_elems)) != cudaSuccess)
        return status_cuda(e, "mpres_batch_commit (GEMM W(A), W(B))");
    const bool gemm = !h.gemm.empty();
    /* launch shape: the largest blockDim3 (or threadsPerRow) is the least threads per CTA */
    int min_threads = 32;
    for (const GemvOp &g : h.gemv) min_threads = std::max(min_threads, g.b3);
    for (const DotOp &d : h.dot) min_threads = std::max(min_threads, d.b3);
    for (const SpmvOp &sp : h.spmv) min_threads = std::max(min_threads, sp.tpr);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    std::vector<std::pair<int, int>> cand; /* threads, CTAs per SM */
    int ct = 0, cp = 0;
    /* batches with GEMM tiles run 128 or 256 threads per CTA */
    if (gemm && min_threads > 256)
        return status_fail(MPRES_ERR_NOT_SUPPORTED,
                           "mpres_batch_commit: a batch with GEMMs takes blockDim3 and threadsPerRow <= 256");
    if (flags & MPRES_BATCH_AUTOTUNE) {
        for (int t : {128, 256, 512, 1024}) {
            if (t < min_threads || (gemm && t > 256)) continue;
            const int occ = batch_ctas_per_sm(b->nmod, t, gemm);
            for (int p : {1, 2, 4, occ})
                if (p >= 1 && p <= occ && std::find(cand.begin(), cand.end(), std::make_pair(t, p)) == cand.end())
                    cand.push_back({t, p});
        }
    } else if (!gemm && batch_cached_shape(b->nmod, ct, cp) && ct >= min_threads) {
        cand.push_back({ct, cp});
    }
    if (cand.empty()) {
        int t = gemm ? 128 : 256;
        while (t < min_threads) t *= 2;
        const int occ = batch_ctas_per_sm(b->nmod, t, gemm);
        if (occ < 1) return status_fail(MPRES_ERR_NOT_SUPPORTED, "mpres_batch_commit: no launch shape fits");
        cand.push_back({t, occ});
    }
    size_t cap = 0;
    int best = 0;
    if (cand.size() > 1) {
        /* time every shape on this batch; GEMV outputs are restored after every run */
        long long outs_total = 0;
        std::vector<long long> offs;
        for (const GemvOp &g : h.gemv) {
            offs.push_back(outs_total);
            outs_total += g.trans ? g.n : g.m;
        }
        for (const GemmOp &g : h.gemm) {
            offs.push_back(outs_total);
            outs_total += (long long)g.m * g.n;
        }
        void *save = nullptr;
        long long *d_offs = nullptr;
        if (outs_total) {
            if ((e = cudaMalloc(&save, rec * outs_total)) != cudaSuccess ||
                (e = cudaMalloc(&d_offs, sizeof(long long) * offs.size())) != cudaSuccess ||
                (e = cudaMemcpy(d_offs, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice)) !=
                    cudaSuccess)
                return status_cuda(e, "mpres_batch_commit (autotune scratch)");
        }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best_ms = 1e30f;
        bool saved = false;
        for (size_t c = 0; c < cand.size() && e == cudaSuccess; c++) {
            const int t = cand[c].first, ctas = cand[c].second * sms;
            if ((e = plan_and_upload(b, t, cap)) != cudaSuccess) break;
            if (!saved && outs_total) {
                if ((e = gemv_outputs(b->nmod, h, b->dev, d_offs, save, 0, s)) != cudaSuccess) break;
                saved = true;
            }
            float ms_min = 1e30f;
            for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {
                cudaEventRecord(e0, s);
                e = batch_launch(b->nmod, h, b->dev, t, ctas, s);
                cudaEventRecord(e1, s);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) ms_min = std::min(ms_min, ms); /* the first run warms up */
                if (e == cudaSuccess && outs_total) e = gemv_outputs(b->nmod, h, b->dev, d_offs, save, 1, s);
            }
            if (ms_min < best_ms) {
                best_ms = ms_min;
                best = (int)c;
            }
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (save) cudaFree(save);
        if (d_offs) cudaFree(d_offs);
        if (e != cudaSuccess) return status_cuda(e, "mpres_batch_commit (autotune)");
        b->autotuned = true;
        if (!gemm) cache_shape(b->nmod, cand[best].first, cand[best].second);
    }
    b->candidates = cand.size() > 1 ? (int)cand.size() : 0;
    b->threads = cand[best].first;
    b->ctas = cand[best].second * sms;
    if ((e = plan_and_upload(b, b->threads, cap)) != cudaSuccess) return status_cuda(e, "mpres_batch_commit (tables)");
    batch_ctas_per_sm(b->nmod, b->threads, gemm); /* raises the shared-memory limit before any capture */
    if (flags & MPRES_BATCH_GRAPH) {
        cudaStream_t cs;
        if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess)
            return status_cuda(e, "mpres_batch_commit (capture stream)");
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = batch_launch(b->nmod, h, b->dev, b->threads, b->ctas, cs);
            e = cudaStreamEndCapture(cs, &b->graph);
            if (e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return status_cuda(e, "mpres_batch_commit (graph capture)");
    }
    b->committed = true;
    return status_ok();
}

int mpres_batch_run(mpres_batch_t *b, void *stream) {
    if (!b) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_run: null batch");
    if (!b->committed) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_run: batch not committed");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = b->exec ? cudaGraphLaunch(b->exec, s) : batch_launch(b->nmod, b->host, b->dev, b->threads, b->ctas, s);
    return e == cudaSuccess ? status_ok() : status_cuda(e, "mpres_batch_run");
}

int mpres_batch_info(const mpres_batch_t *b, long long *out) {
    if (!b || !out) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_batch_info: null argument");
    const size_t rec = 4 * (size_t)b->nmod + 40;
    const BatchHost &h = b->host;
    out[0] = (long long)(h.gemv.size() + h.dot.size() + h.spmv.size() + h.gemm.size());
    out[1] = (long long)h.tasks.size();
    out[2] = b->threads;
    out[3] = b->ctas;
    out[4] = b->exec != nullptr;
    out[5] = b->autotuned;
    out[6] = (long long)(rec * (h.buf1_elems + h.part_elems) + sizeof(int4) * h.w_elems);
    out[7] = b->candidates;
    return status_ok();
}

} // extern "C"
