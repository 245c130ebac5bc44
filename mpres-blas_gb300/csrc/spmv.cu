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
 * fixed tree 16, 8, 4, 2, 1.  Those orders are kept exactly.  The reference
 * stages each thread's running sum and product in shared memory; here they stay
 * in registers and the csrv tree moves partial sums with warp shuffles.
 */
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(spmv)

namespace mpres {
namespace {
using namespace dev;

template <int N>
__global__ void __launch_bounds__(256) spmv_csr_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < m; row += gridDim.x * blockDim.x) {
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

template <int N, int TPR>
__global__ void __launch_bounds__(256) spmv_csrv_kernel(int m, const int *__restrict__ irp, const int *__restrict__ ja,
                                                        const double *__restrict__ as, const void *x, void *y) {
    const int lane = threadIdx.x & (TPR - 1);
    const int groups_per_grid = (gridDim.x * blockDim.x) / TPR;
    const int first = (blockIdx.x * blockDim.x + threadIdx.x) / TPR;
    /* every lane of a warp runs the same number of iterations (shuffles below) */
    const int rounds = (m + groups_per_grid - 1) / groups_per_grid;
    for (int it = 0; it < rounds; it++) {
        const int row = first + it * groups_per_grid;
        const bool active = row < m;
        mp_t<N> sum;
        set_zero<N>(sum);
        if (active) {
            const int start = __ldg(irp + row), end = __ldg(irp + row + 1);
            for (int i = start + lane; i < end; i += TPR) {
                mp_t<N> xv, p, s;
                load_aos<N>(xv, x, __ldg(ja + i));
                mp_mul_d<N>(p, xv, __ldg(as + i));
                mp_add<N>(s, sum, p);
                sum = s;
            }
        }
#pragma unroll
        for (int sft = 16; sft >= 1; sft >>= 1) {
            if (TPR >= 2 * sft) {
                mp_t<N> other = shfl_down<N>(sum, sft);
                if (active && lane < sft) {
                    mp_t<N> s;
                    mp_add<N>(s, sum, other);
                    sum = s;
                }
            }
        }
        if (active && lane == 0) store_aos<N>(sum, y, row);
    }
}

template <int N>
__global__ void __launch_bounds__(256) spmv_ell_kernel(int m, int maxnzr, const int *__restrict__ ja,
                                                       const double *__restrict__ as, const void *x, void *y) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < m; row += gridDim.x * blockDim.x) {
        mp_t<N> sum;
        set_zero<N>(sum);
        for (int col = 0; col < maxnzr; col++) {
            const size_t slot = (size_t)col * m + row;
            const double val = __ldg(as + slot);
            if (dnz(val)) {
                mp_t<N> xv, p, s;
                load_aos<N>(xv, x, __ldg(ja + slot));
                mp_mul_d<N>(p, xv, val);
                mp_add<N>(s, sum, p);
                sum = s;
            }
        }
        store_aos<N>(sum, y, row);
    }
}

int grid_for(int work, int threads) {
    long long g = ((long long)work + threads - 1) / threads;
    return (int)(g < 1 ? 1 : (g > (1 << 30) ? (1 << 30) : g));
}

template <int N> cudaError_t csr(int m, const csr_t &a, const void *x, void *y, cudaStream_t s) {
    spmv_csr_kernel<N><<<grid_for(m, 128), 128, 0, s>>>(m, a.irp, a.ja, a.as, x, y);
    return cudaGetLastError();
}

template <int N, int TPR> cudaError_t csrv_t(int m, const csr_t &a, const void *x, void *y, cudaStream_t s) {
    const int threads = 128;
    spmv_csrv_kernel<N, TPR><<<grid_for(m, threads / TPR), threads, 0, s>>>(m, a.irp, a.ja, a.as, x, y);
    return cudaGetLastError();
}

template <int N> cudaError_t csrv(int m, int tpr, const csr_t &a, const void *x, void *y, cudaStream_t s) {
    switch (tpr) {
    case 1: return csrv_t<N, 1>(m, a, x, y, s);
    case 2: return csrv_t<N, 2>(m, a, x, y, s);
    case 4: return csrv_t<N, 4>(m, a, x, y, s);
    case 8: return csrv_t<N, 8>(m, a, x, y, s);
    case 16: return csrv_t<N, 16>(m, a, x, y, s);
    case 32: return csrv_t<N, 32>(m, a, x, y, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int N> cudaError_t ell(int m, int maxnzr, const ell_t &a, const void *x, void *y, cudaStream_t s) {
    spmv_ell_kernel<N><<<grid_for(m, 128), 128, 0, s>>>(m, maxnzr, a.ja, a.as, x, y);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_spmv_csr(int nmod, int m, const csr_t &a, const void *x, void *y, cudaStream_t s) {
    switch (nmod) {
    case 8: return csr<8>(m, a, x, y, s);
    case 16: return csr<16>(m, a, x, y, s);
    case 32: return csr<32>(m, a, x, y, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_spmv_csrv(int nmod, int m, int tpr, const csr_t &a, const void *x, void *y, cudaStream_t s) {
    switch (nmod) {
    case 8: return csrv<8>(m, tpr, a, x, y, s);
    case 16: return csrv<16>(m, tpr, a, x, y, s);
    case 32: return csrv<32>(m, tpr, a, x, y, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_spmv_ell(int nmod, int m, int maxnzr, const ell_t &a, const void *x, void *y, cudaStream_t s) {
    switch (nmod) {
    case 8: return ell<8>(m, maxnzr, a, x, y, s);
    case 16: return ell<16>(m, maxnzr, a, x, y, s);
    case 32: return ell<32>(m, maxnzr, a, x, y, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
