/*
 * Throughput probes for the roofline of the compute-bound kernels.
 *
 * The HBM and bf16 peaks of this machine are measured elsewhere; the RNS kernels
 * are bound by two other units, so their ceilings are measured here with the
 * exact instruction sequences the kernels use:
 *   - the 32-bit Barrett modular product of mp_device.cuh (integer pipes);
 *   - the directed-rounding double addition (__dadd_rd, FP64 pipe).
 * Each thread runs 8 independent chains so that issue, not latency, limits.
 */
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mpres_gb300.h"
#include "../../include/mpres_gb300_probe.h"

namespace {

__device__ __forceinline__ uint32_t mulmod(uint32_t x, uint32_t y, uint32_t m, uint32_t mu) {
    uint64_t p = (uint64_t)x * y;
    uint32_t q = __umulhi((uint32_t)(p >> 30), mu);
    uint32_t r = (uint32_t)p - q * m;
    r = min(r, r - m);
    r = min(r, r - m);
    return r;
}

__global__ void probe_mulmod_kernel(long long iters, uint32_t m, uint32_t mu, uint32_t *sink) {
    uint32_t a[8];
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] = (tid * 2654435761u + c * 40503u) % m;
    const uint32_t y = (tid ^ 0x5bd1e995u) % m;
    for (long long i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) a[c] = mulmod(a[c], y, m, mu);
    }
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s ^= a[c];
    if (s == 0x9e3779b9u) sink[0] = s; /* keeps the chains live */
}

__global__ void probe_dadd_kernel(long long iters, double step, double *sink) {
    double a[8];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] = 1.0 + tid * 1e-9 + c;
    for (long long i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) a[c] = __dadd_rd(a[c], step);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += a[c];
    if (s == -1.0) sink[0] = s;
}

/* latency of one dependent operation, in SM clock cycles (one thread) */
__global__ void probe_latency_kernel(int which, long long iters, uint32_t m, uint32_t mu, double *out) {
    const long long t0 = clock64();
    double d = 1.0 + threadIdx.x;
    uint32_t a = 12345u + threadIdx.x;
    uint64_t u = 0x9e3779b97f4a7c15ull + threadIdx.x;
    for (long long i = 0; i < iters; i++) {
        if (which == 0) d = __dadd_rd(d, 1e-3);
        else if (which == 1) a = mulmod(a, 48271u, m, mu);
        else u = (u << 3) + (u >> 7) + 1;
    }
    const long long t1 = clock64();
    out[0] = (double)(t1 - t0) / (double)iters;
    if (d == -1.0 || a == 0xffffffffu || u == 0) out[1] = d + a + (double)u; /* keeps the chains live */
}

__global__ void probe_ceil_log2_kernel(const double *x, double *out, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = ceil(log2(x[i]));
}

} // namespace

extern "C" {

int mpres_probe_ceil_log2(const double *x, double *out, size_t count, void *stream) {
    if (!x || !out) return MPRES_ERR_INVALID_VALUE;
    if (count == 0) return MPRES_SUCCESS;
    long long blocks = ((long long)count + 255) / 256;
    probe_ceil_log2_kernel<<<(int)(blocks > 65535 ? 65535 : blocks), 256, 0, (cudaStream_t)stream>>>(
        x, out, (long long)count);
    return cudaGetLastError() == cudaSuccess ? MPRES_SUCCESS : MPRES_ERR_CUDA;
}

int mpres_probe_latency(int which, long long iters, void *out, void *stream) {
    if (which < 0 || which > 2 || iters <= 0 || !out) return MPRES_ERR_INVALID_VALUE;
    probe_latency_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(which, iters, 1073741827u,
                                                           (uint32_t)((1ull << 62) / 1073741827ull), (double *)out);
    return cudaGetLastError() == cudaSuccess ? MPRES_SUCCESS : MPRES_ERR_CUDA;
}

int mpres_probe_mulmod(int blocks, int threads, long long iters, void *sink, void *stream) {
    if (blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0 || !sink) return MPRES_ERR_INVALID_VALUE;
    const uint32_t m = 1283742825u; /* first modulus of the 8-moduli set */
    const uint32_t mu = (uint32_t)((((unsigned __int128)1) << 62) / m);
    probe_mulmod_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, m, mu, (uint32_t *)sink);
    return cudaGetLastError() == cudaSuccess ? MPRES_SUCCESS : MPRES_ERR_CUDA;
}

int mpres_probe_dadd(int blocks, int threads, long long iters, void *sink, void *stream) {
    if (blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0 || !sink) return MPRES_ERR_INVALID_VALUE;
    probe_dadd_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, 1e-12, (double *)sink);
    return cudaGetLastError() == cudaSuccess ? MPRES_SUCCESS : MPRES_ERR_CUDA;
}

} // extern "C"
