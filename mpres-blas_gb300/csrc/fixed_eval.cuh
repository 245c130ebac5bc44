/*
 * The reference's RNS interval evaluation and rank computation on the integer
 * pipes, bit for bit.
 *
 * src/rns.cuh computes, for residues s_i, the fractions s_i/m_i as directed-
 * rounding products s_i * RECIP_{RD,RU}[i] (__dmul_rd/__dmul_ru), sums them with
 * the directed-rounding pairwise tree of src/pairwise.cuh, and drops the whole
 * part.  On GB300 each of those double operations occupies the FP64 pipe, the
 * binding unit of every kernel here.  The same values are obtained exactly with
 * integers:
 *   - every recip is R * 2^-83 with a 53-bit integer R (2^30 < m_i < 2^31), so
 *     the exact product s_i * recip is the integer s_i*R (< 2^84) times 2^-83;
 *   - rounding a non-negative value to 53 significant bits downward is
 *     truncation, upward is truncation plus one unit if any dropped bit is set;
 *     every rounded leaf and every tree node is therefore a multiple of 2^-83
 *     below 2^5 (N <= 32 leaves below 2), i.e. an integer below 2^88;
 *   - subtracting the whole part from such a sum is exact (the reference's
 *     __dsub_rd/__dsub_ru of it return the fraction unchanged), so the fraction
 *     is the low 83 bits.
 * Doubles are formed only where the reference stores one (er_set_d) or where
 * ceil(log2(sumu)) must follow CUDA's log2 (see ceil_log2 below).
 */
#ifndef MPRES_FIXED_EVAL_CUH
#define MPRES_FIXED_EVAL_CUH

#include <cstdint>

namespace mpres {
namespace dev {

constexpr int kFixShift = 83; /* value = F * 2^-83 */

struct fx {
    uint64_t lo, hi; /* F = hi * 2^64 + lo, hi < 2^24 */
};

__device__ __forceinline__ int fx_bitlen(const fx &a) {
    return a.hi ? 128 - __clzll((long long)a.hi) : 64 - __clzll((long long)a.lo);
}

/* round to 53 significant bits, downward (UP = false) or upward (UP = true);
 * at most 35 bits are dropped (F < 2^88), all from the low word */
template <bool UP> __device__ __forceinline__ fx fx_round53(fx a) {
    const int L = fx_bitlen(a);
    if (L > 53) {
        const int drop = L - 53;
        const uint64_t mask = (1ull << drop) - 1;
        const uint64_t dropped = a.lo & mask;
        a.lo &= ~mask;
        if (UP && dropped) {
            const uint64_t inc = 1ull << drop;
            const uint64_t lo = a.lo + inc;
            a.hi += (lo < a.lo);
            a.lo = lo;
        }
    }
    return a;
}

/* exact s * R for s < 2^31, R < 2^53 (result < 2^84) */
__device__ __forceinline__ fx fx_mul(uint32_t s, uint64_t R) {
    const uint64_t p0 = (uint64_t)s * (uint32_t)R;          /* < 2^63 */
    const uint64_t p1 = (uint64_t)s * (uint32_t)(R >> 32);  /* < 2^52 */
    fx r;
    r.lo = p0 + (p1 << 32);
    r.hi = (p1 >> 32) + (r.lo < p0);
    return r;
}

template <bool UP> __device__ __forceinline__ fx fx_add(const fx &a, const fx &b) {
    fx s;
    s.lo = a.lo + b.lo;
    s.hi = a.hi + b.hi + (s.lo < a.lo);
    return fx_round53<UP>(s);
}

/* the pairwise tree of src/pairwise.cuh:855-929 in fixed point; leaf(i) on demand */
template <int SPAN, int LEN, bool UP, class F> __device__ __forceinline__ fx fx_node(const F &leaf, int base) {
    if constexpr (SPAN == 2) {
        if constexpr (LEN > 1) return fx_add<UP>(leaf(base), leaf(base + 1));
        else return leaf(base); /* x + 0 */
    } else {
        fx s1 = fx_node<SPAN / 2, LEN, UP>(leaf, base);
        if constexpr (LEN > SPAN / 2) return fx_add<UP>(s1, fx_node<SPAN / 2, LEN - SPAN / 2, UP>(leaf, base + SPAN / 2));
        else return s1; /* s1 + 0 is exact */
    }
}
template <int N, bool UP, class F> __device__ __forceinline__ fx fx_psum(const F &leaf) {
    return fx_node<psum_span(N), N, UP>(leaf, 0);
}

/* sum over i of RD/RU(s_i * recip_i), rounded as the reference's tree */
template <int N, bool UP> __device__ __forceinline__ fx fx_fraction_sum(const int *s) {
    const Tables<N> &t = T<N>();
    return fx_psum<N, UP>([&](int i) { return fx_round53<UP>(fx_mul((uint32_t)s[i], UP ? t.recip_ru_m[i] : t.recip_rd_m[i])); });
}

__device__ __forceinline__ uint32_t fx_whole(const fx &a) { return (uint32_t)(a.hi >> (kFixShift - 64)); }
__device__ __forceinline__ fx fx_frac(fx a) {
    a.hi &= (1ull << (kFixShift - 64)) - 1;
    return a;
}
__device__ __forceinline__ bool fx_zero(const fx &a) { return (a.lo | a.hi) == 0; }

/* the double F * 2^-83 (F has at most 53 significant bits, so it is exact) */
__device__ __forceinline__ double fx_to_double(const fx &a) {
    const int L = fx_bitlen(a);
    if (L == 0) return 0.0;
    uint64_t m = (L > 64) ? ((a.lo >> (L - 53)) | (a.hi << (64 - (L - 53)))) : (L > 53 ? a.lo >> (L - 53) : a.lo << (53 - L));
    const int e = L - 1 - kFixShift; /* value in [2^e, 2^(e+1)) */
    return __longlong_as_double((long long)(((uint64_t)(e + 1023) << 52) | (m & ((1ull << 52) - 1))));
}

/* er_set_d of the value (src/extrange.cuh:93-107): frac in [1,2), exp */
__device__ __forceinline__ void fx_er_set(er_t &r, const fx &a) {
    if (fx_zero(a)) {
        r.frac = 0.0;
        r.exp = 0;
        return;
    }
    const int L = fx_bitlen(a);
    uint64_t m = (L > 64) ? ((a.lo >> (L - 53)) | (a.hi << (64 - (L - 53)))) : (L > 53 ? a.lo >> (L - 53) : a.lo << (53 - L));
    r.exp = (long long)(L - 1 - kFixShift);
    r.frac = __longlong_as_double((long long)((1023ull << 52) | (m & ((1ull << 52) - 1))));
}

/* value >= eval_acc, i.e. F >= ceil(eval_acc * 2^83) */
template <int N> __device__ __forceinline__ bool fx_ge_acc(const fx &a) {
    const uint64_t lo = T<N>().eval_acc_fx[0], hi = T<N>().eval_acc_fx[1];
    return a.hi > hi || (a.hi == hi && a.lo >= lo);
}

/* ceil(log2(x)) as CUDA's log2 gives it, x = F * 2^-83 > 0 (ceil_log2_d on the
 * exact double) */
template <int N> __device__ __forceinline__ int fx_ceil_log2(const fx &a) { return ceil_log2_d<N>(fx_to_double(a)); }

} // namespace dev
} // namespace mpres

#endif
