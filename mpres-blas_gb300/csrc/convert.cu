/*
 * Double -> mp_float_t conversion on the device, bit for bit the host
 * conversion: the reference's mp_set_d (src/arith/assign.cuh:54-81) with its
 * HOST interval evaluation rns_eval_compute (src/rns.cuh:645-716), which is
 * what every converted input of the reference carries.
 *
 * The host evaluation is not the device one.  It rounds "downward" and
 * "upward" by c -/+ (PHI1*|c| + ETA) computed in round-to-nearest
 * (src/dinterval.cuh:113-154), multiplies residues through a double quotient
 * that may leave a residue one modulus off (src/modular.cuh:88-93), divides by
 * the moduli in its refinement loop, and takes ceil(log2(.)) with the host's
 * log2.  Every one of those steps is an IEEE operation in round-to-nearest,
 * repeated here with the _rn intrinsics; the host log2 is replayed from
 * host_ceil_log2_table(), measured on the host at mpres_init: it differs from
 * the exact ceiling only just above powers of two.
 *
 * One thread per element; the digits of the 53-bit significand come from the
 * Barrett reduction used everywhere else.
 */
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(convert)

namespace mpres {
namespace {
using namespace dev;

/* src/dinterval.cuh emulated directed rounding, evaluated without fusing:
 * PHI1 = 2^-53 (1 + 2 * 2^-53) (exact in double), ETA = 2^-1074 */
constexpr double kPhi1 = 0x1.0000000000001p-53;
constexpr double kEta = 0x1p-1074;
__device__ __forceinline__ double emu_rd(double c) { return __dsub_rn(c, __dadd_rn(__dmul_rn(kPhi1, fabs(c)), kEta)); }
__device__ __forceinline__ double emu_ru(double c) { return __dadd_rn(c, __dadd_rn(__dmul_rn(kPhi1, fabs(c)), kEta)); }

/* the host pairwise tree (src/pairwise.cuh:401-479): same shape as the device
 * one, every node one emulated-rounding addition (missing leaves read 0) */
template <int SPAN, int LEN, bool UP, class F> __device__ __forceinline__ double htree(const F &leaf, int base) {
    if constexpr (SPAN == 2) {
        const double a = leaf(base), b = LEN > 1 ? leaf(base + 1) : 0.0;
        return UP ? emu_ru(__dadd_rn(a, b)) : emu_rd(__dadd_rn(a, b));
    } else {
        const double s1 = htree<SPAN / 2, LEN, UP>(leaf, base);
        double s2 = 0.0;
        if constexpr (LEN > SPAN / 2) s2 = htree<SPAN / 2, LEN - SPAN / 2, UP>(leaf, base + SPAN / 2);
        return UP ? emu_ru(__dadd_rn(s1, s2)) : emu_rd(__dadd_rn(s1, s2));
    }
}
template <int N, bool UP, class F> __device__ __forceinline__ double hsum(const F &leaf) {
    return htree<psum_span(N), N, UP>(leaf, 0);
}

/* src/modular.cuh:88-93: x*y mod m through the quotient (double)(x*y) * (1/m),
 * truncated; the result may be off by one modulus either way */
__device__ __forceinline__ int mulmod_dq(int x, int y, int m, double d) {
    const long long r = (long long)x * (long long)y;
    const int q = __double2int_rz(__dmul_rn(__ll2double_rn(r), d));
    return (int)(r - (long long)q * (long long)m);
}

/* (unsigned) c for the fractions here (c < 2^32; truncation toward zero) */
__device__ __forceinline__ double drop_whole(double c, unsigned &whole) {
    whole = __double2uint_rz(c);
    return __dsub_rn(c, (double)whole);
}

/* ceil(log2(x)) as the host's log2 gives it.  NaN for x < 0 or NaN (log2 of a
 * negative number); `bad` is set for 0, subnormal x and x >= 2, which the
 * refinement loop does not meet (its argument is a fraction below
 * RNS_EVAL_ACCURACY rounded upward from a sum of terms of at least 2^-83). */
template <int N> __device__ __forceinline__ double host_ceil_log2(double x, bool &bad) {
    const uint64_t u = dbits(x);
    if (x < 0 || x != x) return __longlong_as_double(0x7ff8000000000000ll);
    const int E = (int)((u >> 52) & 2047);
    if (E == 0 || E > 1023) {
        bad = true;
        return 0.0;
    }
    const int e = E - 1023;
    const uint64_t frac = u & ((1ull << 52) - 1);
    const int j = frac > 0x7fffffffull ? 0x7fffffff : (int)frac;
    const int *row = T<N>().host_ceil_log2 + 2 * (e + 1022);
    if (j == 0) return (double)__ldg(row);
    return (double)(j < __ldg(row + 1) ? e : e + 1);
}

/* host mrd, src/rns.cuh:514-531 (operands non-negative below the modulus) */
template <int N> __device__ __noinline__ int host_mrd(const int *x) {
    const Tables<N> &t = T<N>();
    int mixed[N];
    for (int i = 0; i < N; i++) {
        int v = x[i];
        for (int j = 0; j < i; j++) {
            if (v < mixed[j]) v = t.moduli[i] - mixed[j] + v;
            else v = v - mixed[j];
            v = mulmod_i<N>(v, t.mrc_inv[j][i], i);
        }
        mixed[i] = v;
    }
    return mixed[N - 1];
}

/* host rns_eval_compute, src/rns.cuh:645-716 */
template <int N> __device__ __noinline__ void host_eval(const int *x, er_t &low, er_t &upp, bool &bad) {
    const Tables<N> &t = T<N>();
    bool zero = true;
    for (int i = 0; i < N; i++) zero = zero && x[i] == 0;
    if (zero) {
        low.frac = upp.frac = 0.0;
        low.exp = upp.exp = 0;
        return;
    }
    int s[N];
#pragma unroll
    for (int i = 0; i < N; i++) s[i] = mulmod_dq(x[i], t.part_inv[i], t.moduli[i], t.recip_rn[i]);
    double suml = hsum<N, false>([&](int i) { return emu_rd(__dmul_rn((double)s[i], t.recip_rd[i])); });
    double sumu = hsum<N, true>([&](int i) { return emu_ru(__dmul_rn((double)s[i], t.recip_ru[i])); });
    unsigned whl, whu;
    suml = drop_whole(suml, whl);
    sumu = drop_whole(sumu, whu);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    int mr = -1;
    if (whl != whu) mr = host_mrd<N>(x);
    if (mr > 0) {
        upp = t.inv_unit_upp;
        return;
    }
    if (mr == 0) low = t.unit_low;
    if (sumu >= t.eval_acc) return;
    long long K = 0;
    for (int guard = 0; sumu < t.eval_acc && guard < 4096; guard++) {
        const double a = -__dadd_rn(host_ceil_log2<N>(sumu, bad), 1.0);
        const double kr = a > (double)t.ref_factor ? a : (double)t.ref_factor;
        int k = __double2int_rz(kr);
        if (k > t.log2m) k = t.log2m;
        if (k < 0) { /* unreachable: ref_factor >= 0 */
            bad = true;
            return;
        }
        const int *row = t.pow2 + (size_t)k * N;
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = mulmod_dq(s[i], __ldg(row + i), t.moduli[i], t.recip_rn[i]);
        sumu = hsum<N, true>([&](int i) { return emu_ru(__ddiv_rn((double)s[i], (double)t.moduli[i])); });
        sumu = drop_whole(sumu, whu);
        K += k;
    }
    suml = hsum<N, false>([&](int i) { return emu_rd(__ddiv_rn((double)s[i], (double)t.moduli[i])); });
    suml = drop_whole(suml, whl);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    low.exp -= K;
    upp.exp -= K;
}

/* mp_set_d, src/arith/assign.cuh:54-81 */
template <int N> __device__ __forceinline__ void set_d(mp_t<N> &r, double x, bool &bad) {
    const Tables<N> &t = T<N>();
    const uint64_t u = dbits(x);
    r.sign = (int)(u >> 63);
    const int field = (int)((u >> 52) & 2047);
    uint64_t sig = u & ((1ull << 52) - 1);
    if (field != 0) sig |= 1ull << 52;
    int exp = field - 1023 - 52; /* as the reference: -1075 for subnormals */
    if (sig != 0) {
        const int tz = __ffsll((long long)sig) - 1;
        sig >>= tz;
        exp += tz;
    } else {
        exp = 0;
    }
    r.exp = exp;
    const uint32_t hi = (uint32_t)(sig >> 30), lo = (uint32_t)(sig & ((1u << 30) - 1));
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i];
        const uint32_t h = mulmod(hi, 1u << 30, m, t.mu[i]);
        r.d[i] = (int)reduce2(h + reduce2(lo, m), m);
    }
    host_eval<N>(r.d, r.ev[0], r.ev[1], bad);
}

template <int N>
__global__ void __launch_bounds__(256) set_d_aos(const double *x, long long count, void *out, int *flag) {
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        mp_t<N> r;
        set_d<N>(r, __ldg(x + i), bad);
        store_aos<N>(r, out, i);
    }
    if (bad) atomicOr(flag, 1);
}

template <int N>
__global__ void __launch_bounds__(256) set_d_soa(const double *x, long long count, int *digits, int *sign, int *exp,
                                                 er_t *eval, const int *lenp, long long offset, int *flag) {
    bool bad = false;
    const int len = __ldg(lenp);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        mp_t<N> r;
        set_d<N>(r, __ldg(x + i), bad);
        store_soa<N>(r, digits, sign, exp, eval, len, offset + i);
    }
    if (bad) atomicOr(flag, 1);
}

/* AoS mp_float_t records <-> SoA mp_array_t elements [offset, offset + count);
 * the SoA's upper bounds sit at eval + layout_len */
template <int N>
__global__ void __launch_bounds__(256) aos_to_soa(const void *aos, int *digits, int *sign, int *exp, er_t *eval,
                                                  long long layout_len, long long offset, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        mp_t<N> v;
        load_aos<N>(v, aos, i);
        store_soa<N>(v, digits, sign, exp, eval, (int)layout_len, offset + i);
    }
}
template <int N>
__global__ void __launch_bounds__(256) soa_to_aos(const int *digits, const int *sign, const int *exp, const er_t *eval,
                                                  long long layout_len, long long offset, long long count, void *aos) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        mp_t<N> v;
        load_soa<N>(v, digits, sign, exp, eval, (int)layout_len, offset + i);
        store_aos<N>(v, aos, i);
    }
}

int blocks_for(long long count) {
    long long b = (count + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

} // namespace

cudaError_t launch_pack(int nmod, bool to_soa, void *aos, const mp_array_t &a, long long layout_len, long long offset,
                        long long count, cudaStream_t s) {
    const int g = blocks_for(count);
    er_t *ev = reinterpret_cast<er_t *>(a.eval);
#define MPRES_PACK(NN)                                                                                      \
    if (to_soa) aos_to_soa<NN><<<g, 256, 0, s>>>(aos, a.digits, a.sign, a.exp, ev, layout_len, offset, count); \
    else soa_to_aos<NN><<<g, 256, 0, s>>>(a.digits, a.sign, a.exp, ev, layout_len, offset, count, aos);
    switch (nmod) {
    case 8: MPRES_PACK(8) break;
    case 16: MPRES_PACK(16) break;
    case 32: MPRES_PACK(32) break;
    default: return cudaErrorInvalidValue;
    }
#undef MPRES_PACK
    return cudaGetLastError();
}

cudaError_t launch_set_d(int nmod, const double *x, long long count, void *out_aos, const mp_array_t *out_soa,
                         long long offset, int *flag, cudaStream_t s) {
    const int g = blocks_for(count);
#define MPRES_SET_D(NN)                                                                                    \
    if (out_aos) set_d_aos<NN><<<g, 256, 0, s>>>(x, count, out_aos, flag);                                 \
    else set_d_soa<NN><<<g, 256, 0, s>>>(x, count, out_soa->digits, out_soa->sign, out_soa->exp,           \
                                         reinterpret_cast<er_t *>(out_soa->eval), out_soa->len, offset, flag);
    switch (nmod) {
    case 8: MPRES_SET_D(8) break;
    case 16: MPRES_SET_D(16) break;
    case 32: MPRES_SET_D(32) break;
    default: return cudaErrorInvalidValue;
    }
#undef MPRES_SET_D
    return cudaGetLastError();
}

} // namespace mpres
