/*
 * Element-wise entry points over AoS mp_float_t vectors in device memory.
 *
 * They expose the device arithmetic the BLAS kernels are built from -- the
 * reference's cuda::mp_add (src/arith/add.cuh:190), cuda::mp_mul
 * (src/arith/mul.cuh:71), cuda::mp_mul_d (src/arith/muld.cuh:59),
 * cuda::rns_scale2pow (src/rns.cuh:1132) and cuda::rns_eval_compute[_fast]
 * (src/rns.cuh:797, :878) -- one element per thread, so each primitive can be
 * checked on its own against the reference's golden vectors.
 */
#include "../../include/mpres_gb300_probe.h"
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(elementwise)

namespace mpres {
namespace {
using namespace dev;

template <int N>
__global__ void __launch_bounds__(256) vec_op(int op, const void *x, const void *y, void *r, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        mp_t<N> a, b, c;
        load_aos<N>(a, x, i);
        if (op == MPRES_OP_MUL_D) {
            mp_mul_d<N>(c, a, __ldg(reinterpret_cast<const double *>(y) + i));
        } else {
            load_aos<N>(b, y, i);
            if (op == MPRES_OP_ADD) mp_add<N>(c, a, b);
            else mp_mul<N>(c, a, b);
        }
        store_aos<N>(c, r, i);
    }
}

template <int N>
__global__ void __launch_bounds__(256) scale_op(const int *digits, const unsigned *D, int *out, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        int d[N];
#pragma unroll
        for (int k = 0; k < N; k++) d[k] = digits[i * N + k];
        scale2pow<N>(d, D[i]);
#pragma unroll
        for (int k = 0; k < N; k++) out[i * N + k] = d[k];
    }
}

template <int N> __device__ __noinline__ void eval_full(er_t &low, er_t &upp, const int *x);

template <int N>
__global__ void __launch_bounds__(256) eval_op(int fast, const int *digits, er_t *low, er_t *upp, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        int d[N];
#pragma unroll
        for (int k = 0; k < N; k++) d[k] = digits[i * N + k];
        er_t lo, up;
        if (fast) eval_fast<N>(lo, up, d);
        else eval_full<N>(lo, up, d);
        low[i] = lo;
        upp[i] = up;
    }
}

/* cuda::rns_eval_compute, src/rns.cuh:797-868 (used by no BLAS kernel; exposed for checking) */
template <int N> __device__ __noinline__ void eval_full(er_t &low, er_t &upp, const int *x) {
    const Tables<N> &t = T<N>();
    int s[N];
    for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(x[i], t.part_inv[i], i);
    double suml = psum<N, false>([&](int i) { return __dmul_rd((double)s[i], t.recip_rd[i]); });
    double sumu = psum<N, true>([&](int i) { return __dmul_ru((double)s[i], t.recip_ru[i]); });
    if (!dnz(suml) && !dnz(sumu)) {
        low.frac = 0.0; low.exp = 0;
        upp.frac = 0.0; upp.exp = 0;
        return;
    }
    const unsigned int whl = (unsigned int)suml, whu = (unsigned int)sumu;
    suml = __dsub_rd(suml, (double)whl);
    sumu = __dsub_ru(sumu, (double)whu);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    int mr = -1;
    if (whl != whu) mr = mrd<N>(x);
    if (mr > 0) {
        upp = t.inv_unit_upp;
        return;
    }
    if (mr == 0) low = t.unit_low;
    if (sumu >= t.eval_acc) return;
    eval_refine<N>(s, sumu, low, upp);
}

int blocks_for(long long count) {
    long long b = (count + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

} // namespace

cudaError_t launch_elementwise(int nmod, int op, const void *x, const void *y, void *r, long long count,
                               cudaStream_t s) {
    const int g = blocks_for(count);
    switch (nmod) {
    case 8: vec_op<8><<<g, 256, 0, s>>>(op, x, y, r, count); break;
    case 16: vec_op<16><<<g, 256, 0, s>>>(op, x, y, r, count); break;
    case 32: vec_op<32><<<g, 256, 0, s>>>(op, x, y, r, count); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_scale2pow(int nmod, const int *digits, const unsigned *D, int *out, long long count,
                             cudaStream_t s) {
    const int g = blocks_for(count);
    switch (nmod) {
    case 8: scale_op<8><<<g, 256, 0, s>>>(digits, D, out, count); break;
    case 16: scale_op<16><<<g, 256, 0, s>>>(digits, D, out, count); break;
    case 32: scale_op<32><<<g, 256, 0, s>>>(digits, D, out, count); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_eval(int nmod, int fast, const int *digits, er_t *low, er_t *upp, long long count,
                        cudaStream_t s) {
    const int g = blocks_for(count);
    switch (nmod) {
    case 8: eval_op<8><<<g, 256, 0, s>>>(fast, digits, low, upp, count); break;
    case 16: eval_op<16><<<g, 256, 0, s>>>(fast, digits, low, upp, count); break;
    case 32: eval_op<32><<<g, 256, 0, s>>>(fast, digits, low, upp, count); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace mpres
