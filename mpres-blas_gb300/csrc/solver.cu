/*
 * Conjugate gradients over a double CSR matrix with multiple-precision vectors
 * (AoS mp_float_t, src/types.cuh:69-74): the reference's mp_cg_csr and
 * mp_pcg_csr (src/sparse/solver/cg_csr.cuh, pcg_csr.cuh) and the "v2" vector
 * kernels they call (src/blas/v2/{diff,axpy,maxpy,prod,dot,norm2}_v2.cuh).
 *
 * Every step is the reference's, in the reference's order, so x and the
 * residual history are bit-identical:
 *   r = b - A x; norm0 = ||r||; eps = norm0 * tol;
 *   while ||r|| > eps and k < maxit:
 *     [PCG: z = r .* M]; rho_{k-1} = rho; rho = r.r [r.z];
 *     p = r [z] at k = 0, else beta = rho / rho_{k-1} (host, MPFR rounding), p = beta p + r [z];
 *     q = A p; alpha = rho / (p.q); x = alpha p + x; r = -alpha q + r; ||r||.
 * The dot products and norms use the reference's two-pass reductions with
 * `blocks_reduce` blocks of `threads` chains; norms take the square root on the
 * host (mp_dsqrt).  The SpMV is this library's (spmv.cu; per-row chains, so
 * any schedule gives the reference's result).
 */
#include <algorithm>
#include <vector>

#include "../../include/mpres_gb300.h"
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(solver)

namespace mpres {

bool host_mp_div(const HostTables &t, const void *x, const void *y, void *r);
bool host_mp_dsqrt(const HostTables &t, const void *x, double &out);

namespace {
using namespace dev;

__host__ __device__ inline unsigned next_pow2(unsigned v) {
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    return v + 1;
}

enum VecOp { kDiff = 0, kAxpy = 1, kMaxpy = 2 };

/* r = x - y (mp_diff), r = alpha x + y (mp_axpy), r = -alpha x + y (mp_maxpy) */
template <int N>
__global__ void __launch_bounds__(256) vec_kernel(int op, int n, const void *alpha, const void *x, const void *y,
                                                  void *r) {
    mp_t<N> a;
    if (op != kDiff) {
        load_aos<N>(a, alpha, 0);
        if (op == kMaxpy) a.sign ^= 1;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mp_t<N> xv, yv, res;
        load_aos<N>(xv, x, i);
        load_aos<N>(yv, y, i);
        if (op == kDiff) {
            yv.sign ^= 1; /* mp_sub: x + (-y) */
            mp_add<N>(res, xv, yv);
        } else {
            mp_t<N> ax;
            mp_mul<N>(ax, a, xv);
            mp_add<N>(res, ax, yv);
        }
        store_aos<N>(res, r, i);
    }
}

/* r = x .* M (mp_prod_d) */
template <int N> __global__ void __launch_bounds__(256) prod_d_kernel(int n, const void *x, const double *M, void *r) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mp_t<N> xv, res;
        load_aos<N>(xv, x, i);
        mp_mul_d<N>(res, xv, __ldg(M + i));
        store_aos<N>(res, r, i);
    }
}

template <int N> __device__ __forceinline__ void block_tree(mp_t<N> *s, unsigned tid, unsigned bsize, bool abs) {
    for (unsigned i = next_pow2(bsize) >> 1; i >= 1; i >>= 1) {
        if (tid < i && tid + i < bsize) {
            mp_t<N> a = s[tid], b = s[tid + i], r;
            if (abs) mp_add_abs<N>(r, a, b);
            else mp_add<N>(r, a, b);
            s[tid] = r;
        }
        __syncthreads();
    }
}

/* first pass of mp_dot_kernel1 (dot_v2.cuh) / mp_sumsq_kernel1 (norm2_v2.cuh):
 * thread p of the grid sums x_i*y_i (x_i*x_i) for i = p, p + K, ...; a tree per block */
template <int N>
__global__ void __launch_bounds__(256) reduce1(int n, const void *x, const void *y, bool sumsq, void *parts) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    const unsigned tid = threadIdx.x, bsize = blockDim.x;
    const unsigned K = gridDim.x * bsize;
    mp_t<N> acc;
    set_zero<N>(acc);
    for (unsigned i = blockIdx.x * bsize + tid; i < (unsigned)n; i += K) {
        mp_t<N> a, b, p, s;
        load_aos<N>(a, x, i);
        if (sumsq) {
            mp_mul<N>(p, a, a);
            mp_add_abs<N>(s, acc, p);
        } else {
            load_aos<N>(b, y, i);
            mp_mul<N>(p, a, b);
            mp_add<N>(s, acc, p);
        }
        acc = s;
    }
    sdata[tid] = acc;
    __syncthreads();
    block_tree<N>(sdata, tid, bsize, sumsq);
    if (tid == 0) store_aos<N>(sdata[0], parts, blockIdx.x);
}

/* second pass (mp_dot_kernel2 / mp_sumsq_kernel2): one block over the block sums */
template <int N>
__global__ void __launch_bounds__(256) reduce2_kernel(int count, const void *parts, bool sumsq, void *r) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    const unsigned tid = threadIdx.x, bsize = blockDim.x;
    mp_t<N> acc;
    set_zero<N>(acc);
    for (unsigned i = tid; i < (unsigned)count; i += bsize) {
        mp_t<N> b, s;
        load_aos<N>(b, parts, i);
        if (sumsq) mp_add_abs<N>(s, acc, b);
        else mp_add<N>(s, acc, b);
        acc = s;
    }
    sdata[tid] = acc;
    __syncthreads();
    block_tree<N>(sdata, tid, bsize, sumsq);
    if (tid == 0) store_aos<N>(sdata[0], r, 0);
}

int grid_for(int n, int threads) { return n / threads + 1; }

template <int N> struct Ops {
    static cudaError_t vec(int op, int n, int threads, const void *a, const void *x, const void *y, void *r,
                           cudaStream_t s) {
        vec_kernel<N><<<grid_for(n, threads), threads, 0, s>>>(op, n, a, x, y, r);
        return cudaGetLastError();
    }
    static cudaError_t prod_d(int n, int threads, const void *x, const double *M, void *r, cudaStream_t s) {
        prod_d_kernel<N><<<grid_for(n, threads), threads, 0, s>>>(n, x, M, r);
        return cudaGetLastError();
    }
    static cudaError_t reduce(int n, int blocks, int threads, const void *x, const void *y, bool sumsq, void *parts,
                              void *r, cudaStream_t s) {
        const size_t smem = (size_t)threads * sizeof(mp_t<N>);
        reduce1<N><<<blocks, threads, smem, s>>>(n, x, y, sumsq, parts);
        reduce2_kernel<N><<<1, threads, smem, s>>>(blocks, parts, sumsq, r);
        return cudaGetLastError();
    }
};

struct Solver {
    int nmod, n, threads, blocks;
    const HostTables *t;
    cudaStream_t s;
    size_t rec;
    cudaError_t vec(int op, const void *a, const void *x, const void *y, void *r) {
        switch (nmod) {
        case 8: return Ops<8>::vec(op, n, threads, a, x, y, r, s);
        case 16: return Ops<16>::vec(op, n, threads, a, x, y, r, s);
        default: return Ops<32>::vec(op, n, threads, a, x, y, r, s);
        }
    }
    cudaError_t prod_d(const void *x, const double *M, void *r) {
        switch (nmod) {
        case 8: return Ops<8>::prod_d(n, threads, x, M, r, s);
        case 16: return Ops<16>::prod_d(n, threads, x, M, r, s);
        default: return Ops<32>::prod_d(n, threads, x, M, r, s);
        }
    }
    cudaError_t reduce(const void *x, const void *y, bool sumsq, void *parts, void *r) {
        switch (nmod) {
        case 8: return Ops<8>::reduce(n, blocks, threads, x, y, sumsq, parts, r, s);
        case 16: return Ops<16>::reduce(n, blocks, threads, x, y, sumsq, parts, r, s);
        default: return Ops<32>::reduce(n, blocks, threads, x, y, sumsq, parts, r, s);
        }
    }
    /* a record from the device after the stream's work */
    cudaError_t fetch(const void *d, char *h) {
        cudaError_t e = cudaMemcpyAsync(h, d, rec, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    /* ||x|| (mp_norm2): sum of squares on the device, root on the host */
    cudaError_t norm2(const void *x, void *parts, void *scratch, double &out, bool &ok) {
        cudaError_t e = reduce(x, nullptr, true, parts, scratch);
        char h[168];
        if (e == cudaSuccess) e = fetch(scratch, h);
        ok = e == cudaSuccess && host_mp_dsqrt(*t, h, out);
        return e;
    }
    /* r = a / b (cuda::mp_div: host MPFR rounding) */
    cudaError_t div(const void *a, const void *b, void *r, bool &ok) {
        char ha[168], hb[168], hr[168];
        cudaError_t e = fetch(a, ha);
        if (e == cudaSuccess) e = fetch(b, hb);
        ok = e == cudaSuccess && host_mp_div(*t, ha, hb, hr);
        if (e == cudaSuccess && ok) e = cudaMemcpyAsync(r, hr, rec, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e;
    }
};

} // namespace

/* mp_cg_csr / mp_pcg_csr; M == nullptr: no preconditioner */
int solve_cg(int nmod, const HostTables &t, int n, const csr_t &A, const void *b, double tol, int maxit,
             const double *M, void *x, double *resvec, int resvec_cap, int *iters, int threads, int blocks_reduce,
             cudaStream_t s) {
    Solver sv{nmod, n, threads, blocks_reduce, &t, s, 4 * (size_t)nmod + 40};
    const size_t rec = sv.rec;
    const size_t vecs = (M ? 4 : 3) * (size_t)n;
    const size_t scal = 6; /* rho, rhop, alpha, beta, pqDot, norm scratch */
    const size_t sched = spmv_workspace_bytes(n);
    char *mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, rec * (vecs + scal + blocks_reduce) + sched + 256);
    if (e != cudaSuccess) return status_cuda(e, "mpres_cg_csr (scratch)");
    char *r = mem, *p = r + rec * n, *q = p + rec * n, *z = M ? q + rec * n : r;
    char *rho = mem + rec * vecs, *rhop = rho + rec, *alpha = rhop + rec, *beta = alpha + rec, *pq = beta + rec,
         *nrm = pq + rec;
    char *parts = nrm + rec;
    Workspace ws;
    ws.ptr = reinterpret_cast<void *>(((uintptr_t)(parts + rec * blocks_reduce) + 255) & ~(uintptr_t)255);
    ws.bytes = sched;
    int status = MPRES_SUCCESS;
    bool ok = true;
    int k = 0, nres = 0;
    double norm0 = 0, normk = 0;
    auto fail_on = [&](cudaError_t err, const char *what) {
        if (err != cudaSuccess && status == MPRES_SUCCESS) status = status_cuda(err, what);
        return err != cudaSuccess;
    };
    do {
        /* r = b - A x; norm0 */
        if (fail_on(launch_spmv_csr(nmod, n, A, x, r, ws, s), "mpres_cg_csr (spmv)")) break;
        if (fail_on(sv.vec(kDiff, nullptr, b, r, r), "mpres_cg_csr (diff)")) break;
        if (fail_on(sv.norm2(r, parts, nrm, norm0, ok), "mpres_cg_csr (norm)") || !ok) break;
        const double eps = norm0 * tol;
        normk = norm0;
        if (nres < resvec_cap) resvec[nres] = normk / norm0;
        nres++;
        while (normk > eps && k < maxit) {
            if (M && fail_on(sv.prod_d(r, M, z), "mpres_cg_csr (precondition)")) break;
            if (fail_on(cudaMemcpyAsync(rhop, rho, rec, cudaMemcpyDeviceToDevice, s), "mpres_cg_csr (copy)")) break;
            if (fail_on(sv.reduce(r, z, false, parts, rho), "mpres_cg_csr (dot)")) break;
            if (k == 0) {
                if (fail_on(cudaMemcpyAsync(p, z, rec * n, cudaMemcpyDeviceToDevice, s), "mpres_cg_csr (copy)")) break;
            } else {
                if (fail_on(sv.div(rho, rhop, beta, ok), "mpres_cg_csr (div)") || !ok) break;
                if (fail_on(sv.vec(kAxpy, beta, p, z, p), "mpres_cg_csr (axpy)")) break;
            }
            if (fail_on(launch_spmv_csr(nmod, n, A, p, q, ws, s), "mpres_cg_csr (spmv)")) break;
            if (fail_on(sv.reduce(p, q, false, parts, pq), "mpres_cg_csr (dot)")) break;
            if (fail_on(sv.div(rho, pq, alpha, ok), "mpres_cg_csr (div)") || !ok) break;
            if (fail_on(sv.vec(kAxpy, alpha, p, x, x), "mpres_cg_csr (axpy)")) break;
            if (fail_on(sv.vec(kMaxpy, alpha, q, r, r), "mpres_cg_csr (maxpy)")) break;
            if (fail_on(sv.norm2(r, parts, nrm, normk, ok), "mpres_cg_csr (norm)") || !ok) break;
            if (nres < resvec_cap) resvec[nres] = normk / norm0;
            nres++;
            k++;
        }
    } while (false);
    if (status == MPRES_SUCCESS && !ok)
        status = status_fail(MPRES_ERR_INVALID_VALUE, "mpres_cg_csr: division by zero or root of a negative number");
    cudaStreamSynchronize(s);
    cudaFree(mem);
    if (iters) *iters = k;
    return status == MPRES_SUCCESS ? status_ok() : status;
}

cudaError_t launch_vec_v2(int nmod, int op, int n, int threads, const void *alpha, const void *x, const void *y,
                          void *r, cudaStream_t s) {
    Solver sv{nmod, n, threads, 0, nullptr, s, 4 * (size_t)nmod + 40};
    return sv.vec(op, alpha, x, y, r);
}

cudaError_t launch_reduce_v2(int nmod, bool sumsq, int n, int blocks, int threads, const void *x, const void *y,
                             void *parts, void *r, cudaStream_t s) {
    Solver sv{nmod, n, threads, blocks, nullptr, s, 4 * (size_t)nmod + 40};
    return sv.reduce(x, y, sumsq, parts, r);
}

} // namespace mpres
