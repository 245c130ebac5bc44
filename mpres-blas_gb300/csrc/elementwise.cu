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
#include "chain_probe.cuh"

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
    const fx sl = fx_fraction_sum<N, false>(s), su = fx_fraction_sum<N, true>(s);
    if (fx_zero(sl) && fx_zero(su)) {
        low.frac = 0.0; low.exp = 0;
        upp.frac = 0.0; upp.exp = 0;
        return;
    }
    const unsigned int whl = fx_whole(sl), whu = fx_whole(su);
    const fx fl = fx_frac(sl), fu = fx_frac(su);
    fx_er_set(low, fl);
    fx_er_set(upp, fu);
    int mr = -1;
    if (whl != whu) mr = mrd<N>(x);
    if (mr > 0) {
        upp = t.inv_unit_upp;
        return;
    }
    if (mr == 0) low = t.unit_low;
    if (fx_ge_acc<N>(fu)) return;
    eval_refine<N>(s, fu, low, upp);
}

/* self-checks of the replacements for CUDA operations (see the probe header) */
template <int N>
__global__ void check_div_kernel(const double *p, double *out, long long count) {
    const Tables<N> &t = T<N>();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = p[i];
        out[4 * i + 0] = div_by_const<false>(v, t.unit_upp.frac, t.unit_upp_recip);
        out[4 * i + 1] = __ddiv_rd(v, t.unit_upp.frac);
        out[4 * i + 2] = div_by_const<true>(v, t.unit_low.frac, t.unit_low_recip);
        out[4 * i + 3] = __ddiv_ru(v, t.unit_low.frac);
    }
}

__global__ void check_scale2_kernel(const double *x, const int *n, double *out, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        out[2 * i] = scale2(x[i], n[i]);
        out[2 * i + 1] = scalbn(x[i], n[i]);
    }
}

/* x must be F * 2^-83 with F < 2^83 holding at most 53 significant bits */
template <int N>
__global__ void check_ceil_log2_kernel(const double *x, int *out, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = x[i];
        const uint64_t u = dbits(v);
        const int e = (int)((u >> 52) & 2047) - 1023;
        const uint64_t m = (u & ((1ull << 52) - 1)) | (1ull << 52); /* v = m * 2^(e-52) */
        const int sh = e - 52 + kFixShift;                             /* F = m * 2^sh */
        fx f;
        if (sh >= 0) {
            f.lo = sh >= 64 ? 0 : m << sh;
            f.hi = sh == 0 ? 0 : (sh >= 64 ? m << (sh - 64) : m >> (64 - sh));
        } else {
            f.lo = m >> -sh;
            f.hi = 0;
        }
        out[2 * i] = fx_ceil_log2<N>(f);
        out[2 * i + 1] = (int)ceil(log2(v));
    }
}

template <int N> __global__ void check_ceil_log2_double_kernel(const double *x, int *out, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        out[2 * i] = ceil_log2_d<N>(x[i]);
        out[2 * i + 1] = (int)ceil(log2(x[i]));
    }
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

cudaError_t launch_check(int which, int nmod, const void *a, const void *b, void *out, long long count,
                         cudaStream_t s) {
    const int g = blocks_for(count);
    if (which == 0) {
        if (nmod == 8) check_div_kernel<8><<<g, 256, 0, s>>>((const double *)a, (double *)out, count);
        else if (nmod == 16) check_div_kernel<16><<<g, 256, 0, s>>>((const double *)a, (double *)out, count);
        else if (nmod == 32) check_div_kernel<32><<<g, 256, 0, s>>>((const double *)a, (double *)out, count);
        else return cudaErrorInvalidValue;
    } else if (which == 1) {
        check_scale2_kernel<<<g, 256, 0, s>>>((const double *)a, (const int *)b, (double *)out, count);
    } else if (which == 2) {
        check_ceil_log2_kernel<8><<<g, 256, 0, s>>>((const double *)a, (int *)out, count);
    } else if (which == 3) {
        check_ceil_log2_double_kernel<8><<<g, 256, 0, s>>>((const double *)a, (int *)out, count);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

MPRES_CHAIN_PROBE_LAUNCHER(launch_chain_probe_fp64)
MPRES_ROUND_PROBE_LAUNCHER(launch_round_probe)
MPRES_PSUM_PROBE_LAUNCHER(launch_psum_probe)
MPRES_EVAL_PHASE_LAUNCHER(launch_eval_phase_probe)

} // namespace mpres
