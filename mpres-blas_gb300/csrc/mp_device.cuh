/*
 * Device arithmetic of RNS multiple-precision numbers, one number per thread.
 *
 * Semantics are those of the reference's device code (namespace cuda of
 * src/modular.cuh, src/extrange.cuh, src/pairwise.cuh, src/rns.cuh and
 * src/arith/{arith_utils,add,mul,muld}.cuh), bit for bit: same residues, sign,
 * exponent and interval evaluation.  The implementation is this library's own:
 *  - residues are reduced with a 32-bit Barrett step (one IMAD.WIDE, one
 *    IMAD.HI, one IMAD and two min-subtractions) instead of 64-bit `%`;
 *  - multiplications of doubles by 0/1/-1 factors, the exponent/significand
 *    splits and the zero tests are bit operations on the integer pipes, and
 *    give exactly the double the reference's multiplications give;
 *  - the directed-rounding operations the interval bounds need (the
 *    __dadd_rd/__dmul_ru/__ddiv_rd... intrinsics) are kept: they are IEEE
 *    correctly rounded, so any exact method gives the same bits;
 *  - pairwise sums evaluate the reference's tree depth first, computing leaves
 *    on demand, so register use stays logarithmic in the set size.
 *
 * The number of moduli N is a template parameter; each translation unit that
 * includes this header owns a __constant__ copy of the tables of N = 8, 16, 32
 * (MPRES_DEFINE_TABLES), uploaded by mpres_init().
 */
#ifndef MPRES_MP_DEVICE_CUH
#define MPRES_MP_DEVICE_CUH

#include <cstdint>

#include "tables.h"

namespace mpres {

template <int N>
struct mp_t {
    int d[N];
    int sign;
    int exp;
    er_t ev[2];
};

namespace dev {

constexpr uint64_t kSign = 1ull << 63;
constexpr uint64_t kZeroExpMask = ((1ull << 52) - 1) | kSign;
constexpr uint64_t kBiasExpMask = 1023ull << 52;

template <int N> __device__ __forceinline__ const Tables<N> &T();

/* The bits of a double, through a move the optimiser cannot see through: tests
 * written on the bits (zero, sign) stay integer instructions instead of being
 * folded back into double comparisons, which occupy GB300's narrow FP64 pipe. */
__device__ __forceinline__ uint64_t dbits(double d) {
    uint64_t u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(d));
    return u;
}
__device__ __forceinline__ double bdbl(uint64_t u) { return __longlong_as_double((long long)u); }
/* x != 0 for a double (false for +0 and -0) */
__device__ __forceinline__ bool dnz(double d) { return (dbits(d) << 1) != 0; }
/* x < 0 for a non-NaN double */
__device__ __forceinline__ bool dneg(double d) { return (dbits(d) >> 63) && dnz(d); }
/* x > 0 for a non-NaN double */
__device__ __forceinline__ bool dpos(double d) { return !(dbits(d) >> 63) && dnz(d); }
/* The high word of the sign bit, read from constant memory.  A flip of a
 * double's sign written with a literal mask is compiled as a double negation,
 * an instruction of the FP64 pipe (ncu counted 5 double additions a step in a
 * loop whose code has 2); an XOR with an operand the compiler cannot know stays
 * on the integer pipes.  Same bits either way. */
static __constant__ uint32_t kSignHiWord = 0x80000000u;
/* -x: the sign bit flipped (what IEEE negation does), on the integer pipes */
__device__ __forceinline__ double dflip(double x) {
    const uint64_t u = dbits(x);
    return __hiloint2double((int)((uint32_t)(u >> 32) ^ kSignHiWord), (int)(uint32_t)u);
}
/* x * f for f in {-1, 0, 1}: exactly the IEEE product, computed on bits */
__device__ __forceinline__ double dscale_sign(double x, int f) {
    if (f == 0) return bdbl(dbits(x) & kSign);
    return f < 0 ? dflip(x) : x;
}

/* Conversions between integers and doubles on the integer pipes.  On GB300 a
 * conversion instruction (I2F.F64, F2I.F64) or a double comparison occupies the
 * FP64 pipe like an arithmetic operation: one warp instruction per 64 cycles of
 * each SM sub-partition, measured, with no overlap between independent ones.
 * These bit forms give the same values exactly. */

/* (double)v for 0 <= v < 2^31 (exact: v has at most 31 significant bits),
 * assembled from two 32-bit words */
__device__ __forceinline__ double u31_to_double(uint32_t v) {
    const int lz = __clz(v | 1u);
    const uint32_t f = v << (lz + 1); /* the fraction bits below the leading 1 */
    const uint32_t hi = ((uint32_t)(1054 - lz) << 20) | (f >> 12);
    return v ? __hiloint2double((int)hi, (int)(f << 20)) : 0.0;
}
/* (unsigned int)x, truncating, for +0 <= x < 2^32 */
__device__ __forceinline__ uint32_t d_trunc_u32(double x) {
    const uint64_t a = dbits(x);
    const int e = (int)(a >> 52) - 1023;
    const uint64_t m = (a & ((1ull << 52) - 1)) | (1ull << 52);
    return e < 0 ? 0u : (uint32_t)(m >> (52 - e));
}
/* x - (double)(unsigned int)x with the subtraction rounded downward (UP =
 * false) or upward, for +0 <= x < 2^32.  The difference is exact, so only a
 * zero result depends on the direction: -0 downward, +0 upward. */
template <bool UP> __device__ __forceinline__ double d_frac(double x) {
    const uint64_t a = dbits(x);
    const int e = (int)(a >> 52) - 1023;
    const double zero = UP ? 0.0 : -0.0;
    if (e < 0) return a ? x : zero;
    const uint64_t f = a & ((1ull << (52 - e)) - 1); /* the bits below the binary point */
    if (!f) return zero;
    const int L = 64 - __clzll((long long)f);
    const uint64_t m = (f << (53 - L)) & ((1ull << 52) - 1);
    return bdbl(((uint64_t)(L + e + 970) << 52) | m); /* f * 2^(e-52): exponent L-1+e-52 */
}

template <bool UP> __device__ __forceinline__ double dadd(double a, double b) {
    return UP ? __dadd_ru(a, b) : __dadd_rd(a, b);
}
template <bool UP> __device__ __forceinline__ double dsub(double a, double b) {
    return UP ? __dsub_ru(a, b) : __dsub_rd(a, b);
}
template <bool UP> __device__ __forceinline__ double dmul(double a, double b) {
    return UP ? __dmul_ru(a, b) : __dmul_rd(a, b);
}
template <bool UP> __device__ __forceinline__ double ddiv(double a, double b) {
    return UP ? __ddiv_ru(a, b) : __ddiv_rd(a, b);
}

/* ---------------------------- residues ---------------------------------- */

/* x*y mod m for 0 <= x, y < 2^31, 2^30 < m < 2^32/3, mu = floor(2^62/m):
 * the Barrett quotient is at most 2 short, so r < 3m < 2^32. */
__device__ __forceinline__ uint32_t mulmod(uint32_t x, uint32_t y, uint32_t m, uint32_t mu) {
    uint64_t p = (uint64_t)x * y;
    uint32_t q = __umulhi((uint32_t)(p >> 30), mu);
    uint32_t r = (uint32_t)p - q * m;
    r = min(r, r - m);
    r = min(r, r - m);
    return r;
}
/* a mod m for 0 <= a < 2m */
__device__ __forceinline__ uint32_t reduce2(uint32_t a, uint32_t m) { return min(a, a - m); }

template <int N> __device__ __forceinline__ int mulmod_i(int x, int y, int i) {
    const Tables<N> &t = T<N>();
    return (int)mulmod((uint32_t)x, (uint32_t)y, (uint32_t)t.moduli[i], t.mu[i]);
}

/* ------------------------ extended-range floats ------------------------- */

/* er_adjust, src/extrange.cuh:412-421 */
__device__ __forceinline__ void er_adjust(er_t &x) {
    uint64_t u = dbits(x.frac);
    bool nz = (u << 1) != 0;
    long long e = (long long)((uint64_t)x.exp + ((u & ~kSign) >> 52) - 1023ull);
    x.exp = nz ? e : 0;
    x.frac = nz ? bdbl((u & kZeroExpMask) | kBiasExpMask) : bdbl(u & kSign);
}

/* er_set_d, src/extrange.cuh:93-107 */
__device__ __forceinline__ void er_set_d(er_t &r, double x) {
    uint64_t u = dbits(x);
    if (dnz(x)) {
        r.exp = (long long)((u & ~kSign) >> 52) - 1023;
        r.frac = bdbl((u & kZeroExpMask) | kBiasExpMask);
    } else {
        r.exp = 0;
        r.frac = 0.0;
    }
}

/* scalbn(x, n): for a normal x whose result stays normal, adding n to the
 * exponent field is the exact result; other cases (zero, subnormal, overflow)
 * go to CUDA's scalbn, which the reference calls in every case. */
__device__ __forceinline__ double scale2(double x, int n) {
    const uint64_t u = dbits(x);
    const int e = (int)((u >> 52) & 2047);
    if (n == 0 || (e != 0 && e != 2047 && e + n >= 1 && e + n <= 2046))
        return bdbl(u + ((uint64_t)(int64_t)n << 52));
    return scalbn(x, n);
}

/* er_add_rd / er_add_ru, src/extrange.cuh:451-490: the operand with the larger
 * exponent keeps its fraction, the other is scaled to it, one directed addition.
 * Written with selects rather than the reference's three branches: a branch
 * costs a single warp about as much as several integer instructions. */
template <bool UP> __device__ __forceinline__ er_t er_add(const er_t &x, const er_t &y) {
    const bool xnz = dnz(x.frac), ynz = dnz(y.frac);
    const long long xe = xnz ? x.exp : 0, ye = ynz ? y.exp : 0;
    const long long dexp = (xnz && ynz) ? xe - ye : 0;
    const bool swap = dexp < 0;
    const double big = swap ? y.frac : x.frac, small = swap ? x.frac : y.frac;
    er_t r;
    r.exp = dexp != 0 ? (swap ? ye : xe) : (xe == 0 ? ye : xe);
    r.frac = dadd<UP>(big, scale2(small, (int)(swap ? dexp : -dexp)));
    er_adjust(r);
    return r;
}

/* Directed division p / z by a positive constant z with zr = RN(1/z): the
 * classical quotient correction.  q0 = RN(p * zr) is within two ulps of p/z; the
 * sign of the remainder p - q*z, obtained exactly from one FMA (it is rounded
 * once, and a nonzero remainder of this size cannot round to zero), decides
 * whether q*z lies below or above p, so stepping q by ulps until the sign flips
 * gives the correctly rounded quotient in the requested direction -- the value
 * __ddiv_rd / __ddiv_ru return.  Inputs outside the normal range where those
 * bounds hold are passed to the intrinsics. */
__device__ __forceinline__ double next_up(double q) {
    const int64_t u = (int64_t)dbits(q);
    if (u == 0 || u == (int64_t)kSign) return bdbl(1); /* +-0 -> smallest subnormal */
    return bdbl((uint64_t)(u >= 0 ? u + 1 : u - 1));
}
__device__ __forceinline__ double next_down(double q) { return -next_up(-q); }

template <bool UP> __device__ __forceinline__ double div_by_const(double p, double z, double zr) {
    const uint64_t ep = (dbits(p) >> 52) & 2047;
    if (ep < 64 || ep > 1984) return ddiv<UP>(p, z); /* zero, subnormal, huge: exact intrinsic */
    double q = __dmul_rn(p, zr);
    if (!UP) {
        /* largest q with q*z <= p */
        if (dneg(__fma_rn(-q, z, p))) {
            q = next_down(q);
            if (dneg(__fma_rn(-q, z, p))) q = next_down(q);
        } else {
            double qn = next_up(q);
            if (!dneg(__fma_rn(-qn, z, p))) {
                q = qn;
                qn = next_up(q);
                if (!dneg(__fma_rn(-qn, z, p))) q = qn;
            }
        }
    } else {
        /* smallest q with q*z >= p */
        if (dpos(__fma_rn(-q, z, p))) {
            q = next_up(q);
            if (dpos(__fma_rn(-q, z, p))) q = next_up(q);
        } else {
            double qn = next_down(q);
            if (!dpos(__fma_rn(-qn, z, p))) {
                q = qn;
                qn = next_down(q);
                if (!dpos(__fma_rn(-qn, z, p))) q = qn;
            }
        }
    }
    return q;
}

/* er_md_rd / er_md_ru (x*y/z), src/extrange.cuh:627-644: the fractions'
 * product rounded in the direction, divided by z.frac rounded in the direction,
 * then er_adjust.  z is RNS_EVAL_UNIT's upper (RD) or lower (RU) bound, zr the
 * nearest double to 1/z.frac and zinv = floor(2^116 / Z), Z the 53-bit
 * significand of z.frac.
 *
 * For fractions with |frac| in [1, 2) (as er_adjust leaves them) and for zeros,
 * both roundings run on the integer pipes.  The 106-bit product P of the
 * significands is cut to 53 bits p (plus one unit when rounding the magnitude
 * up and a dropped bit is set).  With k = 52 if p >= Z, else 53, the quotient
 * Q = floor(p * 2^k / Z) lies in [2^52, 2^53); q0 = floor(p * zinv / 2^(116-k))
 * is Q or Q - 1 (the error of zinv contributes less than 2^-10), the remainder
 * p * 2^k - q0 * Z < 2Z fits 64 bits, and one comparison with Z corrects q0 and
 * yields the remainder that decides the directed rounding.  Other operands use
 * the FP64 intrinsics. */
/* a * b = hi * 2^64 + lo for a, b < 2^53, from four 32-bit partial products
 * that the high and the low half share */
__device__ __forceinline__ void mul_wide53(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
    const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
    const uint64_t p00 = (uint64_t)a0 * b0;
    const uint64_t mid = (uint64_t)a0 * b1 + (uint64_t)a1 * b0 + (p00 >> 32); /* < 2^55 */
    lo = (mid << 32) | (p00 & 0xffffffffull);
    hi = (uint64_t)a1 * b1 + (mid >> 32);
}
/* the same for a < 2^53 and any 64-bit b: the middle sum may carry out of 64 bits */
__device__ __forceinline__ void mul_wide53x64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
    const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
    const uint64_t p00 = (uint64_t)a0 * b0, p10 = (uint64_t)a1 * b0;
    const uint64_t mid = (uint64_t)a0 * b1 + (p00 >> 32); /* at most 2^64 - 2^32 */
    const uint64_t mid2 = mid + p10;
    const uint64_t carry = mid2 < p10 ? (1ull << 32) : 0ull;
    lo = (mid2 << 32) | (p00 & 0xffffffffull);
    hi = (uint64_t)a1 * b1 + (mid2 >> 32) + carry;
}

template <bool UP>
__device__ __forceinline__ er_t er_md(const er_t &x, const er_t &y, const er_t &z, double zr, uint64_t zinv) {
    constexpr uint64_t kMant = (1ull << 52) - 1, kHidden = 1ull << 52;
    const uint64_t bx = dbits(x.frac), by = dbits(y.frac);
    const uint32_t ex = (uint32_t)(bx >> 52) & 2047u, ey = (uint32_t)(by >> 52) & 2047u;
    const uint64_t sgn = (bx ^ by) & kSign;
    er_t r;
    if (ex == 1023u && ey == 1023u) {
        const bool up = UP != (sgn != 0); /* round the magnitude up */
        const uint64_t mx = (bx & kMant) | kHidden, my = (by & kMant) | kHidden;
        uint64_t hi, lo;
        mul_wide53(mx, my, hi, lo); /* P in [2^104, 2^106) */
        const int sh = (hi >> 41) ? 53 : 52;
        uint64_t p = (hi << (64 - sh)) | (lo >> sh);
        p += (up && (lo & ((1ull << sh) - 1))) ? 1u : 0u;
        int e = sh; /* the product is p * 2^(e - 104) */
        if (p >> 53) {
            p >>= 1;
            e++;
        }
        const uint64_t bz = dbits(z.frac);
        const uint64_t mz = (bz & kMant) | kHidden;
        const int ez = (int)((bz >> 52) & 2047) - 1023;
        const bool k52 = p >= mz;
        uint64_t thi, tlo;
        mul_wide53x64(p, zinv, thi, tlo);
        uint64_t q = k52 ? thi : ((thi << 1) | (tlo >> 63));
        uint64_t rem = (k52 ? (p << 52) : (p << 53)) - q * mz;
        if (rem >= mz) {
            q++;
            rem -= mz;
        }
        q += (up && rem) ? 1u : 0u;
        int E = e - 52 - ez - (k52 ? 52 : 53); /* the quotient is q * 2^E */
        if (q >> 53) {
            q >>= 1;
            E++;
        }
        r.exp = x.exp + y.exp - z.exp + (long long)(E + 52);
        r.frac = bdbl(sgn | kBiasExpMask | (q & kMant));
        return r;
    }
    if (((bx << 1) == 0 && ey != 2047u) || ((by << 1) == 0 && ex != 2047u)) {
        /* a zero factor: a signed zero, which er_adjust leaves with exponent 0 */
        r.exp = 0;
        r.frac = bdbl(sgn);
        return r;
    }
    r.exp = x.exp + y.exp - z.exp;
    r.frac = div_by_const<UP>(dmul<UP>(x.frac, y.frac), z.frac, zr);
    er_adjust(r);
    return r;
}

/* ---------------------------- pairwise sums ------------------------------ */

/* The balanced tree of src/pairwise.cuh:855-929 over a power-of-two SPAN with
 * LEN real leaves (missing leaves read 0); leaf(i) is evaluated on demand. */
template <int SPAN, int LEN, bool UP, class F>
__device__ __forceinline__ double psum_node(const F &leaf, int base) {
    /* The leaves are directed-rounding products of non-negative residues and
     * positive reciprocals, so every node is +0 or positive; adding the +0 of
     * a missing subtree is then exact in either direction and is skipped. */
    if constexpr (SPAN == 2) {
        if constexpr (LEN > 1) return dadd<UP>(leaf(base), leaf(base + 1));
        else return leaf(base);
    } else {
        double s1 = psum_node<SPAN / 2, LEN, UP>(leaf, base);
        if constexpr (LEN > SPAN / 2) return dadd<UP>(s1, psum_node<SPAN / 2, LEN - SPAN / 2, UP>(leaf, base + SPAN / 2));
        else return s1;
    }
}
__host__ __device__ constexpr int psum_span(int len) {
    int s = 8;
    while (s <= len) s *= 2;
    return s;
}
template <int N, bool UP, class F> __device__ __forceinline__ double psum(const F &leaf) {
    static_assert(N >= 4, "moduli sets have at least 4 moduli");
    return psum_node<psum_span(N), N, UP>(leaf, 0);
}

/* ceil(log2(x)) exactly as CUDA's log2 gives it, for x > 0.  The exact ceiling
 * follows from the bits; CUDA's log2 is within one ulp of the exact logarithm,
 * which can only move the ceiling for x within a few ulps of a power of two.  At
 * an exact power of two the answer comes from a table filled at mpres_init by
 * evaluating ceil(log2(2^e)) with CUDA's log2 on the device; for any other x
 * within 4096 ulps of a power of two (and for subnormal x) CUDA's log2 is
 * called; beyond that the logarithm is at least 4096 ulps of x away from an
 * integer -- well over two ulps of the result for every exponent -- and the
 * exact ceiling is the answer. */
template <int N> __device__ __forceinline__ int ceil_log2_d(double x) {
    const uint64_t u = dbits(x);
    const int E = (int)((u >> 52) & 2047);
    const uint64_t j = u & ((1ull << 52) - 1);
    if (E != 0 && j == 0) return T<N>().ceil_log2_pow2[E - 1023 + 1074];
    if (E == 0 || j < 4096 || j >= (1ull << 52) - 4096) return (int)ceil(log2(x));
    return E - 1023 + 1;
}

} // namespace dev
} // namespace mpres

#include "fixed_eval.cuh"

namespace mpres {
namespace dev {

/* --------------------------- RNS algorithms ------------------------------ */

/* One step of the mixed-radix conversion (cuda::mrc / cuda::mrd,
 * src/rns.cuh:570-603): digit i less the finished digit j (mod_psub when it is
 * the smaller), times m_j^-1 mod m_i. */
template <int N> __device__ __forceinline__ int mrc_step(int v, int pivot, int j, int i) {
    const Tables<N> &t = T<N>();
    const uint32_t m = (uint32_t)t.moduli[i];
    const uint32_t d = v < pivot ? reduce2((uint32_t)v - (uint32_t)pivot + m, m) : (uint32_t)(v - pivot);
    return (int)mulmod(d, (uint32_t)t.mrc_inv[j][i], m, t.mu[i]);
}

/* The mixed-radix digits of x, in place.  The reference forms digit i by the
 * steps j = 0 .. i-1 in that order, one digit after another: a chain of
 * N(N-1)/2 dependent modular products (measured on one warp: 3.4k cycles for
 * 8 moduli, 15k for 16, 62k for 32).  Here every finished digit j updates all
 * later digits at once: each digit still takes the steps j = 0 .. i-1 in order,
 * so the values are the same, but the chain is N - 1 rounds of independent
 * products.  Up to 16 moduli every index is a constant; for 32 the rounds are
 * a loop and the next round's finished digit is carried in a scalar, so no
 * digit is addressed by a runtime index (which would move them to local
 * memory).  Unrolling the 496 products for 32 moduli as well made the one
 * warp's mixed-radix digit faster (42k against 104k cycles) but mp_gemm 1024^3
 * slower (43.0 against 38.2 ms: its kernel, which calls the rounding out of
 * line, spilled more). */
template <int N> __device__ __forceinline__ void mrc_digits(int (&v)[N]) {
    if constexpr (N <= 16) {
#pragma unroll
        for (int j = 0; j < N - 1; j++) {
#pragma unroll
            for (int i = j + 1; i < N; i++) v[i] = mrc_step<N>(v[i], v[j], j, i);
        }
    } else {
        int pivot = v[0];
#pragma unroll 1
        for (int j = 0; j < N - 1; j++) {
            int next = 0;
#pragma unroll
            for (int i = 1; i < N; i++) {
                if (i > j) {
                    v[i] = mrc_step<N>(v[i], pivot, j, i);
                    if (i == j + 1) next = v[i];
                }
            }
            pivot = next;
        }
    }
}

/* Most significant mixed-radix digit, src/rns.cuh:587-603 (cuda::mrd); out of
 * line so that its N registers of digits do not add to the caller's (mp_dot
 * 2^20 with 8 moduli: 0.82 against 0.92 ms inline) */
template <int N> __device__ __noinline__ int mrd_digits(const int *x) {
    int v[N];
#pragma unroll
    for (int i = 0; i < N; i++) v[i] = x[i];
    mrc_digits<N>(v);
    return v[N - 1];
}
template <int N> __device__ __forceinline__ int mrd(const int *x) {
    int v[N]; /* a copy: see round_if_needed */
#pragma unroll
    for (int i = 0; i < N; i++) v[i] = x[i];
    return mrd_digits<N>(v);
}

/* mrc_compare_rns, src/rns.cuh:570-630 (rare path: ambiguous signs) */
template <int N> __device__ __noinline__ int mrc_compare(const int *x, const int *y) {
    int mx[N], my[N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        mx[i] = x[i];
        my[i] = y[i];
    }
    mrc_digits<N>(mx);
    mrc_digits<N>(my);
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
        if (mx[i] > my[i]) return 1;
        if (my[i] > mx[i]) return -1;
    }
    return 0;
}

template <int N> __device__ __forceinline__ int pow2_row_index(int r) {
    /* out-of-table rows only occur for an operand whose digits are all zero,
     * where any row gives the same product (the reference reads past the end) */
    return r > T<N>().log2m ? T<N>().log2m : r;
}

/* The interval evaluation and the rank come in two forms with identical
 * results: on the FP64 pipe, as the reference computes them (directed-rounding
 * products and pairwise sums), and in fixed point on the integer pipes
 * (fixed_eval.cuh).  The fixed-point form issues about twice the instructions
 * and makes a longer dependency chain, but takes the work off the FP64 pipe,
 * GB300's narrowest.  Measured on GB300: fixed point is 5% faster in mp_gemm
 * (32 moduli, every SM full of warps, FP64 pipe bound) and slower everywhere
 * else -- 2.4x slower in mp_gemv, 3x in mp_dot's reduction -- where few warps
 * per SM make latency and instruction fetch bind.  A translation unit picks one
 * with MPRES_EVAL_FIXED_POINT (0 = FP64, the default) before including this
 * header. */
#ifndef MPRES_EVAL_FIXED_POINT
#define MPRES_EVAL_FIXED_POINT 0
#endif

/* Refinement loop of rns_eval_compute[_fast], src/rns.cuh:843-867 / :908-932,
 * on the FP64 pipe: sumu is the current upper fraction, below RNS_EVAL_ACCURACY.
 * Inlined: it is reached from the out-of-line rounding (round_slow) and from
 * the element-wise evaluation, and inline the residues stay in registers
 * instead of local memory. */
template <int N>
__device__ __forceinline__ void eval_refine(int *s, double sumu, er_t &low, er_t &upp) {
    const Tables<N> &t = T<N>();
    int K = 0;
    for (int guard = 0; dbits(sumu) < dbits(t.eval_acc) && guard < 4096; guard++) {
        int k;
        if (!dnz(sumu)) {
            k = t.log2m; /* log2(0): the reference's index saturates past the table */
        } else {
            const int c = ceil_log2_d<N>(sumu);
            k = -(c + 1) > t.ref_factor ? -(c + 1) : t.ref_factor;
            k = pow2_row_index<N>(k < 0 ? 0 : k);
        }
        const int *row = t.pow2 + (size_t)k * N;
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(s[i], __ldg(row + i), i);
        sumu = psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); });
        sumu = d_frac<true>(sumu);
        K += k;
    }
    double suml = psum<N, false>([&](int i) { return __dmul_rd(u31_to_double((uint32_t)s[i]), t.recip_rd[i]); });
    suml = d_frac<false>(suml);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    low.exp -= K;
    upp.exp -= K;
}

/* the same loop in fixed point: fu is the current upper fraction */
template <int N>
__device__ __forceinline__ void eval_refine(int *s, fx fu, er_t &low, er_t &upp) {
    const Tables<N> &t = T<N>();
    int K = 0;
    for (int guard = 0; !fx_ge_acc<N>(fu) && guard < 4096; guard++) {
        int k;
        if (fx_zero(fu)) {
            k = t.log2m; /* log2(0): the reference's index saturates past the table */
        } else {
            const int c = fx_ceil_log2<N>(fu);
            k = -(c + 1) > t.ref_factor ? -(c + 1) : t.ref_factor;
            k = pow2_row_index<N>(k);
        }
        const int *row = t.pow2 + (size_t)k * N;
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(s[i], __ldg(row + i), i);
        fu = fx_frac(fx_fraction_sum<N, true>(s));
        K += k;
    }
    const fx fl = fx_frac(fx_fraction_sum<N, false>(s));
    fx_er_set(low, fl);
    fx_er_set(upp, fu);
    low.exp -= K;
    upp.exp -= K;
}

/* cuda::rns_eval_compute_fast, src/rns.cuh:878-933 */
template <int N> __device__ __forceinline__ void eval_fast(er_t &low, er_t &upp, const int *x) {
    const Tables<N> &t = T<N>();
    int s[N];
#pragma unroll
    for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(x[i], t.part_inv[i], i);
#if !MPRES_EVAL_FIXED_POINT
    /* The lower sum is formed only when it is used: the refinement recomputes it
     * from the refined residues.  Every leaf rounded down is at most the same
     * leaf rounded up, so the lower sum is zero whenever the upper one is, and
     * the reference's test that both are zero is the upper sum's. */
    double sumu = psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); });
    if (!dnz(sumu)) {
        low.frac = 0.0; low.exp = 0;
        upp.frac = 0.0; upp.exp = 0;
        return;
    }
    sumu = d_frac<true>(sumu);
    if (dbits(sumu) >= dbits(t.eval_acc)) {
        const double suml =
            d_frac<false>(psum<N, false>([&](int i) { return __dmul_rd(u31_to_double((uint32_t)s[i]), t.recip_rd[i]); }));
        er_set_d(low, suml);
        er_set_d(upp, sumu);
        return;
    }
    eval_refine<N>(s, sumu, low, upp);
#else
    const fx sl = fx_fraction_sum<N, false>(s);
    const fx su = fx_fraction_sum<N, true>(s);
    if (fx_zero(sl) && fx_zero(su)) {
        low.frac = 0.0; low.exp = 0;
        upp.frac = 0.0; upp.exp = 0;
        return;
    }
    const fx fl = fx_frac(sl), fu = fx_frac(su);
    if (fx_ge_acc<N>(fu)) {
        fx_er_set(low, fl);
        fx_er_set(upp, fu);
        return;
    }
    eval_refine<N>(s, fu, low, upp);
#endif
}

/* The rank of a number X -- floor(V) for V = sum_i s_i / m_i, where
 * V = rank + X/M -- the way the reference obtains it: the whole parts whl, whu
 * of the directed-rounding pairwise sums PD <= V <= PU of the leaves
 * RD/RU(s_i * recip_i); rank_fast takes whu, rank_full takes whl if whl == whu
 * and otherwise whu when the top mixed-radix digit mrd(x) is 0, whl when not.
 * The sums bracket V within 2^-41.9 (each of the N <= 32 leaves errs by less
 * than 2^-51, each of the N - 1 additions of partial sums below 32 by less
 * than 2^-47), so whenever frac(V) <= 1 - 2^-40:
 *   whu = floor(V), as PU < V + 2^-41.9 < floor(V) + 1;
 *   whl = floor(V) when frac(V) >= 2^-40, and otherwise whl is floor(V) or
 *   floor(V) - 1; in that case X/M = frac(V) < 2^-40 < 1 / m_(N-1), so X is
 *   below the product of the other moduli, mrd(x) = 0, and rank_full returns
 *   whu = floor(V) as well.
 * Both ranks are floor(V) then.  rank_shortcut decides it from the exact
 * integer sum S = sum_i s_i * floor(2^94 / m_i), V - 2^-58 < S / 2^94 <= V:
 * when the top 42 fraction bits of S stay 2^-39 below the next integer it
 * returns true with floor(V) = floor(S / 2^94) in `rank`; otherwise (frac(V)
 * just below an integer) the FP64 sums decide, as in the reference.  In a
 * rounding X/M is tiny, so the shortcut holds; it costs about 40 integer
 * instructions instead of one or two 2N-1-operation FP64 sums. */
template <int N> __device__ __forceinline__ bool rank_shortcut(const int *s, unsigned int &rank) {
    const Tables<N> &t = T<N>();
    unsigned __int128 S = 0;
#pragma unroll
    for (int i = 0; i < N; i++) S += (unsigned __int128)(uint32_t)s[i] * t.inv94[i];
    const uint64_t top = (uint64_t)(S >> 52) & ((1ull << 42) - 1); /* fraction bits 2^-1 .. 2^-42 */
    rank = (unsigned int)(S >> 94);
    return top <= (1ull << 42) - 9;
}

/* floor(S / 2^94) for S = sum_i s_i * ceil(2^94 / m_i): V <= S / 2^94 < V + 2^-58 */
template <int N> __device__ __forceinline__ unsigned int rank_from_above(const int *s) {
    const Tables<N> &t = T<N>();
    unsigned __int128 S = 0;
#pragma unroll
    for (int i = 0; i < N; i++) S += (unsigned __int128)(uint32_t)s[i] * (t.inv94[i] + 1);
    return (unsigned int)(S >> 94);
}

/* cuda::rns_rank_compute, src/rns.cuh:1061-1079.  When rank_shortcut cannot
 * decide, frac(V) = X/M is within 2^-39 of an integer: in a rounding it is
 * almost always tiny, and the directed sums straddle the integer.  The
 * reference then takes whu when the top mixed-radix digit mrd(x) is 0 and whl
 * otherwise.  mrd(x) = 0 means X < M / m_(N-1), so X/M < 2^-30: whu is floor(V)
 * and floor(V) = floor(S / 2^94) with the ceiling inverses.  Otherwise
 * (frac(V) just below 1) both branches of the reference give whl, from the
 * downward sum. */
template <int N> __device__ __forceinline__ int rank_full(const int *x, const int *s) {
    unsigned int fast;
    if (rank_shortcut<N>(s, fast)) return (int)fast;
    if (mrd<N>(x) == 0) return (int)rank_from_above<N>(s);
#if MPRES_EVAL_FIXED_POINT
    return (int)fx_whole(fx_fraction_sum<N, false>(s));
#else
    const Tables<N> &t = T<N>();
    return (int)d_trunc_u32(psum<N, false>([&](int i) { return __dmul_rd(u31_to_double((uint32_t)s[i]), t.recip_rd[i]); }));
#endif
}
/* cuda::rns_rank_compute_fast, src/rns.cuh:1088-1096: whu.  With mrd(x) = 0,
 * X/M < 2^-30 and whu = floor(V) as above; up to 16 moduli the mixed-radix
 * digit is cheaper than the FP64 sum, for 32 the sum is taken directly. */
template <int N> __device__ __forceinline__ int rank_fast(const int *x, const int *s) {
    unsigned int fast;
    if (rank_shortcut<N>(s, fast)) return (int)fast;
    if constexpr (N <= 16) {
        if (mrd<N>(x) == 0) return (int)rank_from_above<N>(s);
    }
#if MPRES_EVAL_FIXED_POINT
    return (int)fx_whole(fx_fraction_sum<N, true>(s));
#else
    const Tables<N> &t = T<N>();
    return (int)d_trunc_u32(psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); }));
#endif
}

/* cuda::make_scaling_step, src/rns.cuh:1101-1124, for 1 <= j <= 30.  Residues
 * modulo 2^j are low bits, so the sum runs in wrapping 32-bit arithmetic. */
template <int N>
__device__ __forceinline__ void scaling_step(int *y, int k, int j, const int *x, const int *c) {
    const Tables<N> &t = T<N>();
    const uint32_t mask = (j >= 32) ? 0xffffffffu : ((1u << j) - 1);
    uint32_t residue = 0;
#pragma unroll
    for (int i = 0; i < N; i++) residue += ((uint32_t)t.part_pow2_res30[i] & mask) * (uint32_t)c[i];
    residue -= (uint32_t)k * ((uint32_t)t.m_pow2_res30 & mask);
    residue &= mask;
    const int *inv = t.pow2_inv + (size_t)(j - 1) * N;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i];
        /* residue < 2^30 < m, so residue mod m_i is residue */
        uint32_t multiple = reduce2((uint32_t)x[i] - residue + m, m);
        y[i] = (int)mulmod(multiple, (uint32_t)__ldg(inv + i), m, t.mu[i]);
    }
}

/* cuda::rns_scale2pow, src/rns.cuh:1132-1158; in place */
template <int N> __device__ __forceinline__ void scale2pow(int *x, unsigned int D) {
    const Tables<N> &t = T<N>();
    int c[N];
    int steps = (int)(D / kScaleBits);
    if (steps > 0) {
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(x[i], t.part_inv[i], i);
        int k = rank_full<N>(x, c);
        scaling_step<N>(x, k, kScaleBits, x, c);
        steps -= 1;
    }
    for (; steps > 0; steps--) {
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(x[i], t.part_inv[i], i);
        int k = rank_fast<N>(x, c);
        scaling_step<N>(x, k, kScaleBits, x, c);
    }
    unsigned int d = D % kScaleBits;
    if (d > 0) {
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(x[i], t.part_inv[i], i);
        int k = (d < D) ? rank_full<N>(x, c) : rank_fast<N>(x, c);
        scaling_step<N>(x, k, (int)d, x, c);
    }
}

/* Rounding after an operation: src/arith/arith_utils.cuh:172-190 (mp_round with
 * mp_get_rnd_bits), also mp_vector_round_kernel (src/mpvector.cuh:669-688) and
 * mp_matrix_round_kernel (src/mpmatrix.cuh:410-428). */
template <int N> __device__ __noinline__ void round_slow(mp_t<N> &r, int bits) {
    r.exp += bits;
    scale2pow<N>(r.d, (unsigned int)bits);
    eval_fast<N>(r.ev[0], r.ev[1], r.d);
}
/* The out-of-line calls of the rare paths take their operands through a copy:
 * a variable whose address reaches a call lives in local memory, so passing
 * the caller's own number would keep every number of the hot loop there. */
template <int N> __device__ __forceinline__ void round_if_needed(mp_t<N> &r) {
    if (dnz(r.ev[1].frac) && r.ev[1].exp >= T<N>().mp_h) {
        int bits = (int)(r.ev[1].exp - T<N>().mp_h + 1);
        if (bits > 0) {
            mp_t<N> tmp = r;
            round_slow<N>(tmp, bits);
            r = tmp;
        }
    }
}

/* cuda::sign_estimate, src/arith/arith_utils.cuh:197-206 (rare path) */
template <int N>
__device__ __noinline__ int sign_estimate(const int *dx, const int *dy, int sx, int sy, int gamma, int theta, int nzx,
                                          int nzy) {
    const Tables<N> &t = T<N>();
    int lx[N], ly[N];
    const int *pg = t.pow2 + (size_t)pow2_row_index<N>(gamma) * N;
    const int *pt = t.pow2 + (size_t)pow2_row_index<N>(theta) * N;
    for (int i = 0; i < N; i++) {
        lx[i] = nzx * mulmod_i<N>(dx[i], __ldg(pg + i), i);
        ly[i] = nzy * mulmod_i<N>(dy[i], __ldg(pt + i), i);
    }
    int cmp = mrc_compare<N>(lx, ly);
    return (cmp < 0 ? sy : sx) * (cmp != 0);
}

/* ------------------------ multiple-precision ops ------------------------- */

template <int N> __device__ __forceinline__ void set_zero(mp_t<N> &z) {
#pragma unroll
    for (int i = 0; i < N; i++) z.d[i] = 0;
    z.sign = 0;
    z.exp = 0;
    z.ev[0].frac = 0.0; z.ev[0].exp = 0;
    z.ev[1].frac = 0.0; z.ev[1].exp = 0;
}

/* RNS_POW2 rows 0 .. kPow2Rows-1 staged in shared memory for the aligned
 * additions of a kernel.  The lanes of a warp align by different shifts, so a
 * load of RNS_POW2[shift][i] from the global table touches up to 32 cache lines
 * per instruction; measured with the rows made uniform (a timing-only copy),
 * those loads were a third of mp_gemm 1024^3.  The copy (pow2_stage, then a
 * barrier) has a row stride of N+4 words and is read four words at a time; lanes
 * on different rows mostly read different banks.  Larger shifts read the global
 * table. */
constexpr int kPow2Rows = 256;
template <int N> __host__ __device__ constexpr int pow2_cache_words() { return kPow2Rows * (N + 4); }
template <int N> __device__ __forceinline__ void pow2_stage(int *cache, int tid, int nthreads) {
    const Tables<N> &t = T<N>();
    const int rows = t.log2m + 1 < kPow2Rows ? t.log2m + 1 : kPow2Rows;
    for (int w = tid; w < rows * N; w += nthreads) cache[(w / N) * (N + 4) + w % N] = __ldg(t.pow2 + w);
}
/* every thread of the block stages the copy, then a barrier; returns its
 * shared-memory address for mp_add */
template <int N> __device__ __forceinline__ uint32_t pow2_cache_setup(int *cache) {
    pow2_stage<N>(cache, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y);
    __syncthreads();
    return (uint32_t)__cvta_generic_to_shared(cache);
}
/* four consecutive words of shared memory at a 16-byte aligned address */
__device__ __forceinline__ void lds_v4(uint32_t addr, uint32_t (&v)[4]) {
    asm("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "r"(addr));
}

/* cuda::mp_add: mp_add_common (src/arith/add.cuh:126-188) and the rounding of
 * its overloads (:190-271).  cache: the shared-memory address of a pow2_stage
 * copy, or 0 for the global table. */
template <int N>
__device__ __forceinline__ void mp_add(mp_t<N> &r, const mp_t<N> &x, const mp_t<N> &y, uint32_t cache = 0) {
    const Tables<N> &t = T<N>();
    int ex = x.exp, ey = y.exp, sx = x.sign, sy = y.sign;
    const int dexp = ex - ey;
    int gamma = dexp > 0 ? dexp : 0;
    int theta = dexp < 0 ? -dexp : 0;
    const int nzx = (!dnz(y.ev[1].frac) || (theta + y.ev[1].exp) < t.mp_j);
    const int nzy = (!dnz(x.ev[1].frac) || (gamma + x.ev[1].exp) < t.mp_j);
    gamma *= nzy;
    theta *= nzx;
    ex = (ex - gamma) * nzx;
    ey = (ey - theta) * nzy;
    sx *= nzx;
    sy *= nzy;
    const int fx = (1 - 2 * sx) * nzx;
    const int fy = (1 - 2 * sy) * nzy;
    er_t ax[2], ay[2];
    ax[0].exp = x.ev[0].exp + gamma; ax[1].exp = x.ev[1].exp + gamma;
    ay[0].exp = y.ev[0].exp + theta; ay[1].exp = y.ev[1].exp + theta;
    ax[0].frac = dscale_sign(x.ev[0].frac, fx); ax[1].frac = dscale_sign(x.ev[1].frac, fx);
    ay[0].frac = dscale_sign(y.ev[0].frac, fy); ay[1].frac = dscale_sign(y.ev[1].frac, fy);
    er_t ev[2];
    ev[0] = er_add<false>(sx ? ax[1] : ax[0], sy ? ay[1] : ay[0]);
    ev[1] = er_add<true>(sx ? ax[0] : ax[1], sy ? ay[0] : ay[1]);
    int sign = dneg(ev[0].frac);
    if (sign != (int)dneg(ev[1].frac)) {
        int dx[N], dy[N]; /* copies: see round_if_needed */
#pragma unroll
        for (int i = 0; i < N; i++) {
            dx[i] = x.d[i];
            dy[i] = y.d[i];
        }
        sign = sign_estimate<N>(dx, dy, sx, sy, gamma, theta, nzx, nzy);
        er_t u = t.unit_low;
        /* ev[sign] = +-unit_low, without indexing ev by a runtime value (which
         * would place ev in local memory) */
        if (sign) {
            u.frac = dflip(u.frac);
            ev[1] = u;
        } else {
            ev[0] = u;
        }
    }
    r.sign = sign;
    r.exp = (ex == 0) ? ey : ex;
    /* cuda::rns_axby_cd, src/modular.cuh:306-314: (2^gamma*x*fx + 2^theta*y*fy) mod m.
     * At most one of gamma, theta is nonzero, so one modular product per
     * residue scales the operand that needs it (row 0 holds 2^0 = 1). */
    const bool gx = gamma != 0;
    const int row = pow2_row_index<N>(gx ? gamma : theta);
    const int *pw = t.pow2 + (size_t)row * N;
    const bool cached = cache != 0 && row < kPow2Rows;
    const uint32_t srow = cache + (uint32_t)((cached ? row : 0) * (N + 4)) * 4u;
    uint32_t pv[4];
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i];
        if (i % 4 == 0) {
            if (cache != 0) {
                lds_v4(srow + 4u * i, pv);
                if (!cached)
                    for (int e = 0; e < 4; e++) pv[e] = (uint32_t)__ldg(pw + i + e);
            } else {
                for (int e = 0; e < 4; e++) pv[e] = (uint32_t)__ldg(pw + i + e);
            }
        }
        const uint32_t w = mulmod(pv[i % 4], (uint32_t)(gx ? x.d[i] : y.d[i]), m, t.mu[i]);
        const uint32_t u = gx ? w : (uint32_t)x.d[i];
        const uint32_t v = gx ? (uint32_t)y.d[i] : w;
        uint32_t a = fx > 0 ? u : (fx < 0 ? (u ? m - u : 0u) : 0u);
        uint32_t b = fy > 0 ? v : (fy < 0 ? (v ? m - v : 0u) : 0u);
        uint32_t s = reduce2(a + b, m);
        if (sign) s = s ? m - s : 0u;
        r.d[i] = (int)s;
    }
    if (sign) {
        er_t lo = ev[0];
        ev[0].frac = dflip(ev[1].frac);
        ev[0].exp = ev[1].exp;
        ev[1].frac = dflip(lo.frac);
        ev[1].exp = lo.exp;
    }
    r.ev[0] = ev[0];
    r.ev[1] = ev[1];
    round_if_needed<N>(r);
}

/* Whether mp_add(x, 0) and mp_add(0, x) return x unchanged, 0 being the
 * number set_zero leaves (sign 0, exp 0, residues 0, bounds 0.0 with exponent
 * 0): when x.exp <= 0 the alignment shifts only the zero operand (or drops it),
 * the zero operand's residues and bounds add nothing, an interval addition of a
 * bound with a zero returns the bound normalised -- unchanged when both of x's
 * bounds are normalised (1 <= |frac| < 2) -- the bounds decide the sign, and the
 * sum needs no rounding when x needs none.  Checked on the oracle over 1.2 M
 * values of 8, 16 and 32 moduli (set_d values with exponents up to +-300 and
 * 2% zeros, then generations of products, sums with exact cancellations and
 * products by doubles with 5% zeros): every x this accepts gave x both ways;
 * the three kinds it rejects (a positive exponent, an unnormalised bound left
 * by an exact cancellation, a bound that needs rounding) do change.  0 + 0 gives
 * the same zero. */
template <int N> __device__ __forceinline__ bool zero_add_keeps(const mp_t<N> &x) {
    const uint64_t b0 = dbits(x.ev[0].frac), b1 = dbits(x.ev[1].frac);
    return x.exp <= 0 && ((b0 >> 52) & 2047) == 1023 && ((b1 >> 52) & 2047) == 1023 && x.ev[1].exp < T<N>().mp_h;
}

/* cuda::mp_add_abs: |x| + |y|, mp_add_abs_common (src/arith/addabs.cuh:81-127):
 * the aligned residues added with 0/1 factors, no signs, bounds added as stored */
template <int N> __device__ __forceinline__ void mp_add_abs(mp_t<N> &r, const mp_t<N> &x, const mp_t<N> &y) {
    const Tables<N> &t = T<N>();
    int ex = x.exp, ey = y.exp;
    const int dexp = ex - ey;
    int gamma = dexp > 0 ? dexp : 0;
    int theta = dexp < 0 ? -dexp : 0;
    const int nzx = (!dnz(y.ev[1].frac) || (theta + y.ev[1].exp) < t.mp_j);
    const int nzy = (!dnz(x.ev[1].frac) || (gamma + x.ev[1].exp) < t.mp_j);
    gamma *= nzy;
    theta *= nzx;
    ex = (ex - gamma) * nzx;
    ey = (ey - theta) * nzy;
    r.exp = (ex == 0) ? ey : ex;
    r.sign = 0;
    er_t ax[2], ay[2];
    ax[0].exp = x.ev[0].exp + gamma; ax[1].exp = x.ev[1].exp + gamma;
    ay[0].exp = y.ev[0].exp + theta; ay[1].exp = y.ev[1].exp + theta;
    ax[0].frac = dscale_sign(x.ev[0].frac, nzx); ax[1].frac = dscale_sign(x.ev[1].frac, nzx);
    ay[0].frac = dscale_sign(y.ev[0].frac, nzy); ay[1].frac = dscale_sign(y.ev[1].frac, nzy);
    r.ev[0] = er_add<false>(ax[0], ay[0]);
    r.ev[1] = er_add<true>(ax[1], ay[1]);
    const int *pg = t.pow2 + (size_t)pow2_row_index<N>(gamma) * N;
    const int *pt = t.pow2 + (size_t)pow2_row_index<N>(theta) * N;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i];
        const uint32_t u = nzx ? mulmod((uint32_t)__ldg(pg + i), (uint32_t)x.d[i], m, t.mu[i]) : 0u;
        const uint32_t v = nzy ? mulmod((uint32_t)__ldg(pt + i), (uint32_t)y.d[i], m, t.mu[i]) : 0u;
        r.d[i] = (int)reduce2(u + v, m);
    }
    round_if_needed<N>(r);
}

/* cuda::mp_mul: mp_mul_common + rounding (src/arith/mul.cuh:53-113); also the
 * split kernels mp_*_mul_esi/digits + round of src/mpvector.cuh, src/mpmatrix.cuh */
template <int N> __device__ __forceinline__ void mp_mul(mp_t<N> &r, const mp_t<N> &x, const mp_t<N> &y) {
    const Tables<N> &t = T<N>();
    r.exp = x.exp + y.exp;
    r.sign = x.sign ^ y.sign;
    r.ev[0] = er_md<false>(x.ev[0], y.ev[0], t.unit_upp, t.unit_upp_recip, t.unit_upp_inv);
    r.ev[1] = er_md<true>(x.ev[1], y.ev[1], t.unit_low, t.unit_low_recip, t.unit_low_inv);
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = mulmod_i<N>(x.d[i], y.d[i], i);
    round_if_needed<N>(r);
}

/* cuda::mp_mul_d, src/arith/muld.cuh:59-74 */
template <int N> __device__ __forceinline__ void mp_mul_d(mp_t<N> &r, const mp_t<N> &x, double y) {
    const Tables<N> &t = T<N>();
    const uint64_t u = dbits(y);
    const bool ynz = dnz(y);
    const uint64_t significand = ynz ? ((u & ((1ull << 52) - 1)) | (1ull << 52)) : 0ull;
    const int yexp = (int)(((u >> 52) & 2047) - (ynz ? (uint64_t)(1023 + 52) : 0ull));
    r.exp = x.exp + yexp;
    r.sign = x.sign ^ (int)(u >> 63);
    r.ev[0].exp = x.ev[0].exp;
    r.ev[1].exp = x.ev[1].exp;
    /* (double)significand: 2^52 <= significand < 2^53, or 0 */
    const double sd = ynz ? bdbl((1075ull << 52) | (significand & ((1ull << 52) - 1))) : 0.0;
    r.ev[0].frac = __dmul_rd(x.ev[0].frac, sd);
    r.ev[1].frac = __dmul_ru(x.ev[1].frac, sd);
    er_adjust(r.ev[0]);
    er_adjust(r.ev[1]);
    /* significand < 2^53: reduce it once per modulus, then multiply */
    const uint32_t hi = (uint32_t)(significand >> 30), lo = (uint32_t)(significand & ((1u << 30) - 1));
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i];
        /* significand mod m = (hi * 2^30 + lo) mod m, with hi < 2^23 */
        uint32_t h = mulmod(hi, (uint32_t)(1u << 30), m, t.mu[i]);
        uint32_t ym = reduce2(h + reduce2(lo, m), m);
        r.d[i] = (int)mulmod((uint32_t)x.d[i], ym, m, t.mu[i]);
    }
    round_if_needed<N>(r);
}

/* ---------------------------- memory access ------------------------------ */

/* element i of an SoA mp_array_t (src/types.cuh:85-92); len = *a.len */
template <int N>
__device__ __forceinline__ void load_soa(mp_t<N> &v, const int *digits, const int *sign, const int *exp,
                                         const er_t *eval, int len, long long i) {
    static_assert(N % 4 == 0, "vector loads of digits");
    const int4 *dp = reinterpret_cast<const int4 *>(digits + (size_t)i * N);
#pragma unroll
    for (int q = 0; q < N / 4; q++) {
        int4 w = __ldg(dp + q);
        v.d[4 * q] = w.x; v.d[4 * q + 1] = w.y; v.d[4 * q + 2] = w.z; v.d[4 * q + 3] = w.w;
    }
    v.sign = __ldg(sign + i);
    v.exp = __ldg(exp + i);
    const longlong2 *ep = reinterpret_cast<const longlong2 *>(eval);
    longlong2 lo = __ldg(ep + i), up = __ldg(ep + len + i);
    v.ev[0].frac = __longlong_as_double(lo.x); v.ev[0].exp = lo.y;
    v.ev[1].frac = __longlong_as_double(up.x); v.ev[1].exp = up.y;
}
template <int N>
__device__ __forceinline__ void store_soa(const mp_t<N> &v, int *digits, int *sign, int *exp, er_t *eval, int len,
                                          long long i) {
    int4 *dp = reinterpret_cast<int4 *>(digits + (size_t)i * N);
#pragma unroll
    for (int q = 0; q < N / 4; q++) dp[q] = make_int4(v.d[4 * q], v.d[4 * q + 1], v.d[4 * q + 2], v.d[4 * q + 3]);
    sign[i] = v.sign;
    exp[i] = v.exp;
    longlong2 *ep = reinterpret_cast<longlong2 *>(eval);
    ep[i] = make_longlong2(__double_as_longlong(v.ev[0].frac), v.ev[0].exp);
    ep[len + i] = make_longlong2(__double_as_longlong(v.ev[1].frac), v.ev[1].exp);
}

/* AoS mp_float_t (src/types.cuh:69-74): digits[N], sign, exp, eval[2]; 4N+40 bytes,
 * 8-byte aligned.  Loaded as 8-byte words. */
template <int N> __device__ __forceinline__ void load_aos(mp_t<N> &v, const void *base, long long i) {
    const long long *p = reinterpret_cast<const long long *>((const char *)base + (size_t)i * (4 * N + 40));
#pragma unroll
    for (int q = 0; q < N / 2; q++) {
        long long w = __ldg(p + q);
        v.d[2 * q] = (int)(w & 0xffffffff);
        v.d[2 * q + 1] = (int)(w >> 32);
    }
    long long se = __ldg(p + N / 2);
    v.sign = (int)(se & 0xffffffff);
    v.exp = (int)(se >> 32);
    v.ev[0].frac = __longlong_as_double(__ldg(p + N / 2 + 1));
    v.ev[0].exp = __ldg(p + N / 2 + 2);
    v.ev[1].frac = __longlong_as_double(__ldg(p + N / 2 + 3));
    v.ev[1].exp = __ldg(p + N / 2 + 4);
}
template <int N> __device__ __forceinline__ void store_aos(const mp_t<N> &v, void *base, long long i) {
    long long *p = reinterpret_cast<long long *>((char *)base + (size_t)i * (4 * N + 40));
#pragma unroll
    for (int q = 0; q < N / 2; q++)
        p[q] = (long long)(uint32_t)v.d[2 * q] | ((long long)(uint32_t)v.d[2 * q + 1] << 32);
    p[N / 2] = (long long)(uint32_t)v.sign | ((long long)(uint32_t)v.exp << 32);
    p[N / 2 + 1] = __double_as_longlong(v.ev[0].frac);
    p[N / 2 + 2] = v.ev[0].exp;
    p[N / 2 + 3] = __double_as_longlong(v.ev[1].frac);
    p[N / 2 + 4] = v.ev[1].exp;
}

/* shuffle a whole number down by delta lanes among the lanes of `mask` */
template <int N> __device__ __forceinline__ mp_t<N> shfl_down(const mp_t<N> &v, int delta, unsigned mask = 0xffffffffu) {
    mp_t<N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = __shfl_down_sync(mask, v.d[i], delta);
    r.sign = __shfl_down_sync(mask, v.sign, delta);
    r.exp = __shfl_down_sync(mask, v.exp, delta);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        r.ev[k].frac = __shfl_down_sync(mask, v.ev[k].frac, delta);
        r.ev[k].exp = __shfl_down_sync(mask, v.ev[k].exp, delta);
    }
    return r;
}

/* The tree of src/mpreduct.cuh:59-67 over the `len` entries s[0 .. len-1] of one
 * group of threads (lt = the thread's index in the group): for i = nextPow2(len)/2,
 * ..., 2, 1, entry lt < i with lt + i < len becomes s[lt] + s[lt + i].  Levels
 * i >= 32 go through shared memory with a barrier each (every thread of the block
 * calls this); the levels below 32 involve only the group's first 32 entries and
 * run in the registers of the group's first warp, the partner's sum taken by a
 * shuffle: the same pairs, added in the same order, without five barriers and
 * shared-memory round trips.  The group must start at a multiple of 32 threads.
 * The sum ends in s[0], written by the thread with lt = 0. */
template <int N> __device__ __forceinline__ void tree_sum(mp_t<N> *s, int lt, int len, bool valid) {
    unsigned i = len > 1 ? 1u << (31 - __clz(len - 1)) : 0u;
    for (; i >= 32; i >>= 1) {
        if (valid && (unsigned)lt < i && (unsigned)lt + i < (unsigned)len) {
            mp_t<N> a = s[lt], b = s[lt + i], r;
            mp_add<N>(r, a, b);
            s[lt] = r;
        }
        __syncthreads();
    }
    if (valid && lt < 32 && lt < len) {
        const unsigned mask = len >= 32 ? 0xffffffffu : (1u << len) - 1;
        mp_t<N> v = s[lt];
        for (; i >= 1; i >>= 1) {
            const mp_t<N> o = shfl_down<N>(v, (int)i, mask);
            if ((unsigned)lt < i && (unsigned)lt + i < (unsigned)len) {
                mp_t<N> r;
                mp_add<N>(r, v, o);
                v = r;
            }
        }
        if (lt == 0) s[0] = v;
    }
    __syncthreads();
}

/* BLAS element index for a stride (negative strides start from the far end) */
__device__ __forceinline__ long long blas_index(long long i, int n, int inc) {
    return inc > 0 ? i * inc : ((long long)-n + i + 1) * inc;
}

} // namespace dev
} // namespace mpres

/* Per-translation-unit constant tables and their upload hook. */
#define MPRES_DEFINE_TABLES(TU)                                                                        \
    namespace mpres {                                                                                  \
    namespace {                                                                                        \
    __constant__ Tables<8> g_tab8;                                                                     \
    __constant__ Tables<16> g_tab16;                                                                   \
    __constant__ Tables<32> g_tab32;                                                                   \
    }                                                                                                  \
    namespace dev {                                                                                    \
    template <> __device__ __forceinline__ const Tables<8> &T<8>() { return g_tab8; }                  \
    template <> __device__ __forceinline__ const Tables<16> &T<16>() { return g_tab16; }               \
    template <> __device__ __forceinline__ const Tables<32> &T<32>() { return g_tab32; }               \
    }                                                                                                  \
    cudaError_t upload_tables_##TU(int n, const void *tab) {                                           \
        if (n == 8) return cudaMemcpyToSymbol(g_tab8, tab, sizeof(Tables<8>));                         \
        if (n == 16) return cudaMemcpyToSymbol(g_tab16, tab, sizeof(Tables<16>));                      \
        if (n == 32) return cudaMemcpyToSymbol(g_tab32, tab, sizeof(Tables<32>));                      \
        return cudaErrorInvalidValue;                                                                  \
    }                                                                                                  \
    }

#endif
