/*
 * Host computation of the constant tables of a moduli set.
 *
 * The reference computes them with GMP/MPFR in rns_const_init()
 * (src/rns.cuh:324-442) and mp_const_init() (src/arith/arith_utils.cuh:44-90).
 * Every value here is exact integer arithmetic or the same double expression,
 * so no multiple-precision library is needed:
 *  - residues of M and M_i modulo m_j or 2^j come from 64-bit modular products;
 *  - RNS_EVAL_UNIT = 1/M rounded down and up, where M is first rounded down to
 *    53 bits (the reference keeps M in a 53-bit MPFR variable), obtained from a
 *    128-bit integer division of 2^105 by the top 53 bits of M;
 *  - MP_PRECISION, MP_H and MP_J follow from floor(log2 M) because the top 53
 *    bits of M are not a power of two for any predefined set (checked).
 */
#include "tables.h"

#include <cmath>
#include <cstring>

#include "moduli_sets.h"

namespace mpres {

namespace {

int64_t inverse_mod(int64_t a, int64_t m) {
    a %= m;
    if (a < 0) a += m;
    int64_t r0 = m, r1 = a, t0 = 0, t1 = 1;
    while (r1 != 0) {
        int64_t q = r0 / r1, tmp;
        tmp = r0 - q * r1; r0 = r1; r1 = tmp;
        tmp = t0 - q * t1; t0 = t1; t1 = tmp;
    }
    if (t0 < 0) t0 += m;
    return t0;
}

/* Dekker-style emulated rounding of the reference's host code
 * (src/dinterval.cuh:130-150): c -/+ (PHI1*|c| + ETA), evaluated unfused. */
double emulated_rd(double c) {
    volatile double phi1 = std::ldexp(1.0, -53) * (1 + 2 * std::ldexp(1.0, -53));
    volatile double t = phi1 * std::fabs(c);
    volatile double e = t + std::ldexp(1.0, -1074);
    return c - e;
}
double emulated_ru(double c) {
    volatile double phi1 = std::ldexp(1.0, -53) * (1 + 2 * std::ldexp(1.0, -53));
    volatile double t = phi1 * std::fabs(c);
    volatile double e = t + std::ldexp(1.0, -1074);
    return c + e;
}

/* product of the moduli as little-endian 32-bit words */
int product_words(const int *moduli, int n, uint32_t *w) {
    int len = 1;
    w[0] = 1;
    for (int i = 0; i < n; i++) {
        uint64_t carry = 0;
        for (int j = 0; j < len; j++) {
            uint64_t v = (uint64_t)w[j] * (uint32_t)moduli[i] + carry;
            w[j] = (uint32_t)v;
            carry = v >> 32;
        }
        if (carry) w[len++] = (uint32_t)carry;
    }
    return len;
}

/* v = M * 2^shift with M the 53-bit significand of v as an integer (v > 0);
 * false unless the shift lands in [0, 10] */
bool mantissa_at(double v, int shift, uint64_t &M) {
    int e;
    const double f = std::frexp(v, &e); /* v = f * 2^e, f in [0.5, 1) */
    const uint64_t m = (uint64_t)std::ldexp(f, 53);
    const int s = e - 53 - shift;       /* v = m * 2^(e-53) = (m << s) * 2^shift */
    if (s < 0 || s > 10) return false;
    M = m << s;
    return true;
}

/* floor(2^116 / Z) for the 53-bit significand Z of a positive normal double,
 * saturated at 2^64 - 1 (Z = 2^52); the device's integer er_md divides by Z
 * with it */
static uint64_t significand_inverse(double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof(u));
    const uint64_t z = (u & ((1ull << 52) - 1)) | (1ull << 52);
    const unsigned __int128 q = (((unsigned __int128)1) << 116) / z;
    return q >> 64 ? ~0ull : (uint64_t)q;
}

/* the integer forms the fixed-point evaluation uses (every recip is R * 2^-83
 * with a 53-bit R; eval_acc as the 128-bit ceiling of eval_acc * 2^83); false
 * if a constant is outside that range */
bool compute_fixed_forms(HostTables &t) {
    for (int i = 0; i < t.n; i++) {
        int e;
        std::frexp(t.recip_rd[i], &e);
        if (e != -30 || !mantissa_at(t.recip_rd[i], -83, t.recip_rd_m[i])) return false;
        std::frexp(t.recip_ru[i], &e);
        if (e != -30 || !mantissa_at(t.recip_ru[i], -83, t.recip_ru_m[i])) return false;
        if (t.recip_rd_m[i] >= (1ull << 53) || t.recip_ru_m[i] >= (1ull << 53)) return false;
    }
    int e;
    const uint64_t m = (uint64_t)std::ldexp(std::frexp(t.eval_acc, &e), 53); /* eval_acc = m * 2^(e-53) */
    const int s = e - 53 + 83;
    if (!(t.eval_acc > 0) || s > 64 || s < -63) return false;
    const unsigned __int128 acc =
        s >= 0 ? (unsigned __int128)m << s : ((unsigned __int128)m + ((1ull << -s) - 1)) >> -s;
    t.eval_acc_fx[0] = (uint64_t)acc;
    t.eval_acc_fx[1] = (uint64_t)(acc >> 64);
    if (!(t.unit_upp.frac > 0) || !(t.unit_low.frac > 0)) return false;
    t.unit_upp_recip = 1.0 / t.unit_upp.frac;
    t.unit_low_recip = 1.0 / t.unit_low.frac;
    t.unit_upp_inv = significand_inverse(t.unit_upp.frac);
    t.unit_low_inv = significand_inverse(t.unit_low.frac);
    return true;
}

} // namespace

bool compute_host_tables(int n, HostTables &t) {
    static const int m8[] = MPRES_SET8_MODULI, m16[] = MPRES_SET16_MODULI, m32[] = MPRES_SET32_MODULI;
    const int *mod;
    if (n == 8) { mod = m8; t.log2m = MPRES_SET8_LOG2; }
    else if (n == 16) { mod = m16; t.log2m = MPRES_SET16_LOG2; }
    else if (n == 32) { mod = m32; t.log2m = MPRES_SET32_LOG2; }
    else return false;
    t.n = n;
    for (int i = 0; i < n; i++) {
        t.moduli[i] = mod[i];
        /* the Barrett reduction and the scaling step assume 2^30 < m_i < 2^32 / 3 */
        if (mod[i] <= (1 << 30) || (int64_t)mod[i] * 3 >= ((int64_t)1 << 32)) return false;
        t.mu[i] = (uint32_t)((((unsigned __int128)1) << 62) / (uint32_t)mod[i]);
    }
    for (int i = 0; i < n; i++) {
        int64_t mi = 1;
        for (int j = 0; j < n; j++)
            if (j != i) mi = mi * mod[j] % mod[i];
        t.part_inv[i] = (int)inverse_mod(mi, mod[i]);
    }
    delete[] t.pow2;
    t.pow2 = new int[(size_t)(t.log2m + 1) * n];
    for (int j = 0; j < n; j++) {
        int64_t v = 1;
        for (int r = 0; r <= t.log2m; r++) {
            t.pow2[(size_t)r * n + j] = (int)v;
            v = v * 2 % mod[j];
        }
    }
    uint32_t m_low = 1;
    for (int i = 0; i < n; i++) m_low *= (uint32_t)mod[i];
    for (int r = 0; r < kScaleBits; r++) {
        uint32_t mask = (1u << (r + 1)) - 1;
        t.m_pow2_res[r] = (int)(m_low & mask);
        for (int j = 0; j < n; j++) {
            uint32_t p = 1;
            for (int k = 0; k < n; k++)
                if (k != j) p *= (uint32_t)mod[k];
            t.part_pow2_res[r][j] = (int)(p & mask);
            t.pow2_inv[r][j] = (int)inverse_mod(((int64_t)1 << (r + 1)) % mod[j], mod[j]);
        }
    }
    for (int i = 0; i < n; i++) {
        volatile double q = 1.0 / mod[i];
        t.recip_rd[i] = emulated_rd(q);
        t.recip_ru[i] = emulated_ru(q);
    }
    std::memset(t.mrc_inv, 0, sizeof(t.mrc_inv));
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) t.mrc_inv[i][j] = (int)inverse_mod(mod[i], mod[j]);
    /* src/rns.cuh:385-387 */
    volatile double acc = 4 * std::pow(2.0, 1 - 53);
    acc = acc * n;
    acc = acc * std::log2((double)n);
    acc = acc * (1 + MPRES_EVAL_RELATIVE_ERROR / 2);
    acc = acc / MPRES_EVAL_RELATIVE_ERROR;
    t.eval_acc = acc;
    t.ref_factor = (int)std::floor(std::log2(1 / (2 * t.eval_acc)));

    uint32_t w[40];
    int len = product_words(mod, n, w);
    int bitlen = (len - 1) * 32 + (32 - __builtin_clz(w[len - 1]));
    uint64_t top = 0;
    for (int b = bitlen - 1; b >= bitlen - 53; b--) top = (top << 1) | ((w[b / 32] >> (b % 32)) & 1u);
    if (top == ((uint64_t)1 << 52)) return false; /* M53 a power of two: formulas below would not hold */
    const int e53 = bitlen - 53; /* M53 = top * 2^e53 */
    unsigned __int128 num = ((unsigned __int128)1) << 105;
    uint64_t q = (uint64_t)(num / top);
    bool inexact = (num % top) != 0;
    int ex;
    t.unit_low.frac = std::frexp((double)q, &ex);
    t.unit_low.exp = (long long)ex - 105 - e53;
    t.unit_upp.frac = std::frexp((double)(q + (inexact ? 1 : 0)), &ex);
    t.unit_upp.exp = (long long)ex - 105 - e53;
    /* 1 - 1/M53 rounded up is 1 (0.5 * 2^1), rounded down 1 - 2^-53 */
    t.inv_unit_upp.frac = 0.5;
    t.inv_unit_upp.exp = 1;
    t.inv_unit_low.frac = 1.0 - std::ldexp(1.0, -53);
    t.inv_unit_low.exp = 0;
    const int E = bitlen - 1; /* floor(log2 M) */
    t.mp_precision = E / 2 - 1;
    t.mp_h = (E % 2 == 0) ? -(E / 2) - 1 : -((E + 1) / 2);
    t.mp_j = -1;
    return compute_fixed_forms(t);
}

} // namespace mpres
