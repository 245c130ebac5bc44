/*
 * CPU oracle for the RNS multiple-precision hot path of MPRES-BLAS.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py load it.
 *
 * It restates, function by function, the reference's DEVICE arithmetic
 * (namespace cuda in the src/ headers) and its HOST conversion mp_set_d, plus the
 * summation order of the kernels behind mp_dot, mp_gemv, mp_gemm and
 * mp_spmv_csr/csrv/ell.  Each function cites the reference file:line it follows.
 *
 * Directed rounding (the __dadd_rd/__dmul_ru/__ddiv_rd... intrinsics of the
 * device code) is computed here in round-to-nearest with error-free
 * transformations (TwoSum, an FMA product remainder, an FMA division remainder)
 * followed by a one-ulp step; this gives the correctly rounded IEEE result in
 * the requested direction, including the sign of exact zeros.  The host
 * conversion keeps the reference's emulated rounding (src/dinterval.cuh), which
 * is a different, deliberately non-IEEE formula.
 *
 * Build with -ffp-contract=off: the reference evaluates x*y+z unfused on the
 * host (src/dinterval.cuh:43-49, EMPLOY_STD_FMA false).
 */
#include "mpres_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../mpres-blas_gb300/csrc/moduli_sets.h"
#include "cuda_log2_table.h"

typedef ora_er_t er_t;

typedef struct {
    int digits[ORA_MAXN];
    int sign;
    int exp;
    er_t eval[2];
} mpf_t;

/* ------------------------------------------------------------------------- */
/* bit helpers                                                               */
/* ------------------------------------------------------------------------- */

static inline uint64_t bits_of(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static inline double dbl_of(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
#define SIGN_BIT ((uint64_t)1 << 63)
#define ZERO_EXP_MASK ((((uint64_t)1 << 52) - 1) | SIGN_BIT)
#define BIAS_EXP_MASK ((uint64_t)1023 << 52)

static inline double next_up(double x) { return nextafter(x, INFINITY); }
static inline double next_down(double x) { return nextafter(x, -INFINITY); }

/* ------------------------------------------------------------------------- */
/* directed rounding in round-to-nearest arithmetic                          */
/* ------------------------------------------------------------------------- */

/* exact error of s = RN(a + b) (Knuth's TwoSum) */
static inline double two_sum_err(double a, double b, double s) {
    double bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

static double add_rd(double a, double b) {
    double s = a + b;
    if (s == 0) return (signbit(a) && signbit(b)) || (signbit(a) != signbit(b)) ? -0.0 : 0.0;
    return two_sum_err(a, b, s) < 0 ? next_down(s) : s;
}
static double add_ru(double a, double b) {
    double s = a + b;
    if (s == 0) return s; /* IEEE: +0 unless both operands are -0, same as nearest */
    return two_sum_err(a, b, s) > 0 ? next_up(s) : s;
}
static double sub_rd(double a, double b) { return add_rd(a, -b); }
static double sub_ru(double a, double b) { return add_ru(a, -b); }
static double mul_rd(double a, double b) {
    double p = a * b;
    if (p == 0 || !isfinite(p)) return p;
    return fma(a, b, -p) < 0 ? next_down(p) : p;
}
static double mul_ru(double a, double b) {
    double p = a * b;
    if (p == 0 || !isfinite(p)) return p;
    return fma(a, b, -p) > 0 ? next_up(p) : p;
}
/* The remainder a - q*b of the nearest quotient q is exact (no underflow here). */
static double div_rd(double a, double b) {
    double q = a / b;
    if (q == 0 || !isfinite(q)) return q;
    double r = fma(-q, b, a);
    int q_too_big = (b > 0) ? (r < 0) : (r > 0);
    return q_too_big ? next_down(q) : q;
}
static double div_ru(double a, double b) {
    double q = a / b;
    if (q == 0 || !isfinite(q)) return q;
    double r = fma(-q, b, a);
    int q_too_small = (b > 0) ? (r > 0) : (r < 0);
    return q_too_small ? next_up(q) : q;
}

/* Host emulated rounding, src/dinterval.cuh:55-154 with EMPLOY_STD_FMA false:
 * c = a op b; c -/+ (PHI1*|c| + ETA), PHI1 = 2^-53*(1 + 2*2^-53), ETA = 2^-1074. */
static double host_phi1(void) { return ldexp(1.0, -53) * (1 + 2 * ldexp(1.0, -53)); }
static double host_eta(void) { return ldexp(1.0, -1074); }
static double host_rd(double c) { return c - (host_phi1() * fabs(c) + host_eta()); }
static double host_ru(double c) { return c + (host_phi1() * fabs(c) + host_eta()); }

/* ------------------------------------------------------------------------- */
/* residue arithmetic, src/modular.cuh (64-bit % exactly as written)         */
/* ------------------------------------------------------------------------- */

static inline int mod_mul(int x, int y, int m) { return (int)(((int64_t)x * (int64_t)y) % (int64_t)m); }
static inline int mod_psub(int x, int y, int m) { return (int)(((int64_t)x - (int64_t)y + (int64_t)m) % (int64_t)m); }
static inline int mod_sub(int x, int y, int m) { return (int)(((int64_t)x - (int64_t)y) % (int64_t)m); }

/* host mod_mul with a double quotient (src/modular.cuh:88-93) */
static inline int host_mod_mul_d(int x, int y, int m, double d) {
    int64_t r = (int64_t)x * (int64_t)y;
    double quotient = (double)r * d;
    int i = (int)quotient;
    return (int)(r - (int64_t)i * (int64_t)m);
}

/* double -> int conversion of the GPU (cvt.rzi.s32.f64): truncation, saturating */
static inline int gpu_d2i(double q) {
    if (q != q) return 0;
    if (q >= 2147483647.0) return 2147483647;
    if (q <= -2147483648.0) return (int)(-2147483647 - 1);
    return (int)q;
}

/* device mod_axby with a double quotient (src/modular.cuh:163-168) */
static inline int dev_mod_axby_d(int a, int x, int b, int y, int m, double d) {
    int64_t r = (int64_t)a * (int64_t)x + (int64_t)b * (int64_t)y;
    double quotient = (double)r * d;
    int i = gpu_d2i(quotient);
    return (int)(uint32_t)(uint64_t)(r - (int64_t)i * (int64_t)m);
}

/* ------------------------------------------------------------------------- */
/* constants, src/rns.cuh:324-442 and src/arith/arith_utils.cuh:44-90        */
/* ------------------------------------------------------------------------- */

static int64_t mod_inverse(int64_t x, int64_t m) {
    /* extended Euclid on non-negative values */
    int64_t a = x % m, b = m, u = 1, v = 0;
    if (a < 0) a += m;
    while (b) {
        int64_t q = a / b, t;
        t = a - q * b; a = b; b = t;
        t = u - q * v; u = v; v = t;
    }
    u %= m;
    if (u < 0) u += m;
    return u;
}

static ora_ctx_t g_ctx[3];
static int g_ready[3];

static int set_index(int n) { return n == 8 ? 0 : n == 16 ? 1 : n == 32 ? 2 : -1; }

/* 1/M53 rounded to 53 bits in the given direction, where M53 is the moduli
 * product rounded down to 53 bits (the reference holds M in a default-precision,
 * i.e. 53-bit, MPFR variable: src/rns.cuh:334-335), returned as MPFR's
 * mpfr_get_d_2exp does: frac in [0.5, 1). */
static er_t inv_m53(const int *moduli, int n, int up) {
    /* M as little-endian 32-bit limbs */
    uint32_t limb[ORA_MAXN + 2];
    int nl = 1;
    memset(limb, 0, sizeof(limb));
    limb[0] = 1;
    for (int i = 0; i < n; i++) {
        uint64_t carry = 0;
        for (int j = 0; j < nl; j++) {
            uint64_t t = (uint64_t)limb[j] * (uint32_t)moduli[i] + carry;
            limb[j] = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) limb[nl++] = (uint32_t)carry;
    }
    int top = nl - 1;
    int lz = __builtin_clz(limb[top]);
    int bitlen = top * 32 + (32 - lz);
    /* top 53 bits */
    uint64_t m53 = 0;
    for (int b = bitlen - 1; b >= bitlen - 53; b--) m53 = (m53 << 1) | ((limb[b / 32] >> (b % 32)) & 1u);
    int e53 = bitlen - 53; /* M53 = m53 * 2^e53 */
    unsigned __int128 num = (unsigned __int128)1 << 105;
    uint64_t q = (uint64_t)(num / m53);
    uint64_t rem = (uint64_t)(num - (unsigned __int128)q * m53);
    if (up && rem) q += 1;
    er_t r;
    int ex;
    r.frac = frexp((double)q, &ex); /* q <= 2^53 is exact */
    r.exp = (int64_t)ex - 105 - e53;
    return r;
}

static void build_ctx(ora_ctx_t *c, int n, int log2m, const int *moduli) {
    c->n = n;
    c->log2m = log2m;
    for (int i = 0; i < n; i++) c->moduli[i] = moduli[i];
    for (int i = 0; i < n; i++) {
        int64_t mi = 1;
        for (int j = 0; j < n; j++)
            if (j != i) mi = (mi * moduli[j]) % moduli[i];
        c->part_inv[i] = (int)mod_inverse(mi, moduli[i]);
    }
    c->pow2 = (int *)malloc(sizeof(int) * (size_t)(log2m + 1) * n);
    for (int j = 0; j < n; j++) {
        int v = 1;
        for (int i = 0; i <= log2m; i++) {
            c->pow2[i * n + j] = v;
            v = mod_mul(v, 2, moduli[j]);
        }
    }
    uint32_t mlow = 1;
    for (int i = 0; i < n; i++) mlow *= (uint32_t)moduli[i];
    for (int i = 0; i < ORA_T; i++) {
        uint32_t mask = (i + 1 == 32) ? 0xffffffffu : ((1u << (i + 1)) - 1);
        c->m_pow2_res[i] = (int)(mlow & mask);
        for (int j = 0; j < n; j++) {
            uint32_t p = 1;
            for (int k = 0; k < n; k++)
                if (k != j) p *= (uint32_t)moduli[k];
            c->part_pow2_res[i][j] = (int)(p & mask);
            int64_t pw = ((int64_t)1 << (i + 1)) % moduli[j];
            c->pow2_inv[i][j] = (int)mod_inverse(pw, moduli[j]);
        }
    }
    for (int i = 0; i < n; i++) {
        double q = 1.0 / moduli[i];
        c->recip_rd[i] = host_rd(q);
        c->recip_ru[i] = host_ru(q);
    }
    memset(c->mrc_inv, 0, sizeof(c->mrc_inv));
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) c->mrc_inv[i][j] = (int)mod_inverse(moduli[i], moduli[j]);
    c->eval_acc = 4 * pow(2.0, 1 - 53) * n * log2((double)n) * (1 + MPRES_EVAL_RELATIVE_ERROR / 2) /
                  MPRES_EVAL_RELATIVE_ERROR;
    c->ref_factor = (int)floor(log2(1 / (2 * c->eval_acc)));
    c->unit_upp = inv_m53(moduli, n, 1);
    c->unit_low = inv_m53(moduli, n, 0);
    /* 1 - 1/M53 rounded up is 1.0 and rounded down is 1 - 2^-53 for every set */
    c->inv_unit_upp.frac = 0.5;
    c->inv_unit_upp.exp = 1;
    c->inv_unit_low.frac = 1.0 - ldexp(1.0, -53);
    c->inv_unit_low.exp = 0;
    /* MP_PRECISION, MP_H, MP_J (src/arith/arith_utils.cuh:46-64) from E = floor(log2 M) */
    {
        /* E = floor(log2 M53) = bitlen(M) - 1 */
        uint32_t limb[ORA_MAXN + 2];
        int nl = 1;
        memset(limb, 0, sizeof(limb));
        limb[0] = 1;
        for (int i = 0; i < n; i++) {
            uint64_t carry = 0;
            for (int j = 0; j < nl; j++) {
                uint64_t t = (uint64_t)limb[j] * (uint32_t)moduli[i] + carry;
                limb[j] = (uint32_t)t;
                carry = t >> 32;
            }
            if (carry) limb[nl++] = (uint32_t)carry;
        }
        int E = (nl - 1) * 32 + (31 - __builtin_clz(limb[nl - 1]));
        /* M53 is not a power of two for any predefined set (checked by the tests) */
        c->mp_precision = E / 2 - 1;
        c->mp_h = (E % 2 == 0) ? -(E / 2) - 1 : -((E + 1) / 2);
        c->mp_j = -1;
    }
}

const ora_ctx_t *ora_init(int n) {
    int s = set_index(n);
    if (s < 0) return NULL;
    if (!g_ready[s]) {
#pragma omp critical(ora_init)
        {
            if (!g_ready[s]) {
                static const int m8[] = MPRES_SET8_MODULI, m16[] = MPRES_SET16_MODULI, m32[] = MPRES_SET32_MODULI;
                if (n == 8) build_ctx(&g_ctx[s], 8, MPRES_SET8_LOG2, m8);
                if (n == 16) build_ctx(&g_ctx[s], 16, MPRES_SET16_LOG2, m16);
                if (n == 32) build_ctx(&g_ctx[s], 32, MPRES_SET32_LOG2, m32);
                g_ready[s] = 1;
            }
        }
    }
    return &g_ctx[s];
}

int ora_mp_size(int n) { return 4 * n + 40; }

int ora_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ora_tables(int n, int *part_inv, int *pow2, int *m_pow2_res, int *part_pow2_res, int *pow2_inv,
                double *recip_rd, double *recip_ru, int *mrc_inv, double *eval_acc, int *ref_factor,
                ora_er_t *units, int *mp_consts) {
    const ora_ctx_t *c = ora_init(n);
    memcpy(part_inv, c->part_inv, sizeof(int) * n);
    memcpy(pow2, c->pow2, sizeof(int) * n * (c->log2m + 1));
    memcpy(m_pow2_res, c->m_pow2_res, sizeof(int) * ORA_T);
    for (int i = 0; i < ORA_T; i++)
        for (int j = 0; j < n; j++) {
            part_pow2_res[i * n + j] = c->part_pow2_res[i][j];
            pow2_inv[i * n + j] = c->pow2_inv[i][j];
        }
    memcpy(recip_rd, c->recip_rd, sizeof(double) * n);
    memcpy(recip_ru, c->recip_ru, sizeof(double) * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) mrc_inv[i * n + j] = c->mrc_inv[i][j];
    *eval_acc = c->eval_acc;
    *ref_factor = c->ref_factor;
    units[0] = c->unit_low;
    units[1] = c->unit_upp;
    units[2] = c->inv_unit_low;
    units[3] = c->inv_unit_upp;
    mp_consts[0] = c->mp_precision;
    mp_consts[1] = c->mp_h;
    mp_consts[2] = c->mp_j;
}

/* ------------------------------------------------------------------------- */
/* AoS load/store in the reference's mp_float_t layout                       */
/* ------------------------------------------------------------------------- */

static void load_mp(int n, const void *base, long i, mpf_t *o) {
    const char *p = (const char *)base + (size_t)i * ora_mp_size(n);
    memcpy(o->digits, p, 4 * n);
    memcpy(&o->sign, p + 4 * n, 4);
    memcpy(&o->exp, p + 4 * n + 4, 4);
    memcpy(o->eval, p + 4 * n + 8, 32);
}
static void store_mp(int n, void *base, long i, const mpf_t *o) {
    char *p = (char *)base + (size_t)i * ora_mp_size(n);
    memcpy(p, o->digits, 4 * n);
    memcpy(p + 4 * n, &o->sign, 4);
    memcpy(p + 4 * n + 4, &o->exp, 4);
    memcpy(p + 4 * n + 8, o->eval, 32);
}
static void mp_zero(mpf_t *z) { memset(z, 0, sizeof(*z)); } /* MP_ZERO, arith_utils.cuh:66-75 */

/* ------------------------------------------------------------------------- */
/* extended-range arithmetic, device half of src/extrange.cuh                */
/* ------------------------------------------------------------------------- */

/* src/extrange.cuh:412-421 */
static inline void er_adjust(er_t *x) {
    uint64_t u = bits_of(x->frac);
    int nz = (x->frac != 0);
    x->exp = (int64_t)(((uint64_t)x->exp + ((u & ~SIGN_BIT) >> 52) - 1023u) * (uint64_t)nz);
    u = (u & ZERO_EXP_MASK) | BIAS_EXP_MASK;
    x->frac = dbl_of(u) * nz;
}

/* src/extrange.cuh:451-490 (er_add_rd / er_add_ru); scalbn in nearest mode */
static er_t er_add_dir(er_t x, er_t y, int up) {
    x.exp *= (x.frac != 0);
    y.exp *= (y.frac != 0);
    int64_t dexp = (x.exp - y.exp) * (x.frac != 0) * (y.frac != 0);
    er_t r;
    if (dexp > 0) {
        r.exp = x.exp;
        double t = scalbn(y.frac, (int)-dexp);
        r.frac = up ? add_ru(x.frac, t) : add_rd(x.frac, t);
    } else if (dexp < 0) {
        r.exp = y.exp;
        double t = scalbn(x.frac, (int)dexp);
        r.frac = up ? add_ru(y.frac, t) : add_rd(y.frac, t);
    } else {
        r.exp = (x.exp == 0) ? y.exp : x.exp;
        r.frac = up ? add_ru(x.frac, y.frac) : add_rd(x.frac, y.frac);
    }
    er_adjust(&r);
    return r;
}

/* src/extrange.cuh:627-644 */
static er_t er_md_rd(er_t x, er_t y, er_t z) {
    er_t r;
    r.exp = x.exp + y.exp - z.exp;
    r.frac = div_rd(mul_rd(x.frac, y.frac), z.frac);
    er_adjust(&r);
    return r;
}
static er_t er_md_ru(er_t x, er_t y, er_t z) {
    er_t r;
    r.exp = x.exp + y.exp - z.exp;
    r.frac = div_ru(mul_ru(x.frac, y.frac), z.frac);
    er_adjust(&r);
    return r;
}

/* src/extrange.cuh:93-107 (er_set_d) */
static void er_set_d(er_t *r, double x) {
    uint64_t u = bits_of(x);
    if (x != 0) {
        r->exp = (int64_t)((u & ~SIGN_BIT) >> 52) - 1023;
        r->frac = dbl_of((u & ZERO_EXP_MASK) | BIAS_EXP_MASK);
    } else {
        r->exp = 0;
        r->frac = 0;
    }
}

/* ------------------------------------------------------------------------- */
/* pairwise sums, src/pairwise.cuh: balanced tree over a power-of-two span,   */
/* missing leaves read as 0 (device :855-929, host :401-479)                  */
/* ------------------------------------------------------------------------- */

typedef double (*add2_fn)(double, double);

static double psum_node(const double *x, int len, int span, add2_fn add) {
    if (span == 2) return add(x[0], len > 1 ? x[1] : 0.0);
    int h = span / 2;
    double s1 = psum_node(x, len, h, add);
    double s2 = (len > h) ? psum_node(x + h, len - h, h, add) : 0.0;
    return add(s1, s2);
}
static double psum(const double *x, int len, add2_fn add) {
    if (len >= 4) {
        int span = 8;
        while (span <= len) span *= 2; /* 4..7 -> 8, 8..15 -> 16, ... */
        return psum_node(x, len, span, add);
    }
    if (len == 3) return add(add(x[0], x[1]), x[2]);
    if (len == 2) return add(x[0], x[1]);
    if (len == 1) return x[0];
    return 0;
}
static double host_add_rd(double a, double b) { return host_rd(a + b); }
static double host_add_ru(double a, double b) { return host_ru(a + b); }

/* ------------------------------------------------------------------------- */
/* inter-modular RNS algorithms, device half of src/rns.cuh                  */
/* ------------------------------------------------------------------------- */

/* src/rns.cuh:587-603 (cuda::mrd) */
static int mrd(const ora_ctx_t *c, const int *x) {
    int mixed[ORA_MAXN];
    const int n = c->n;
    for (int i = 0; i < n; i++) {
        mixed[i] = x[i];
        for (int j = 0; j < i; j++) {
            if (mixed[i] < mixed[j]) mixed[i] = mod_psub(mixed[i], mixed[j], c->moduli[i]);
            else mixed[i] = mixed[i] - mixed[j];
            mixed[i] = mod_mul(mixed[i], c->mrc_inv[j][i], c->moduli[i]);
        }
    }
    return mixed[n - 1];
}
/* src/rns.cuh:570-584 (cuda::mrc) and :608-630 (mrs_cmp, mrc_compare_rns) */
static void mrc(const ora_ctx_t *c, int *mr, const int *x) {
    const int n = c->n;
    for (int i = 0; i < n; i++) {
        mr[i] = x[i];
        for (int j = 0; j < i; j++) {
            if (mr[i] < mr[j]) mr[i] = mod_psub(mr[i], mr[j], c->moduli[i]);
            else mr[i] = mr[i] - mr[j];
            mr[i] = mod_mul(mr[i], c->mrc_inv[j][i], c->moduli[i]);
        }
    }
}
static int mrc_compare(const ora_ctx_t *c, const int *x, const int *y) {
    int mx[ORA_MAXN], my[ORA_MAXN];
    mrc(c, mx, x);
    mrc(c, my, y);
    for (int i = c->n - 1; i >= 0; i--) {
        if (mx[i] > my[i]) return 1;
        if (my[i] > mx[i]) return -1;
    }
    return 0;
}

static void rns_mul(const ora_ctx_t *c, int *r, const int *x, const int *y) {
    for (int i = 0; i < c->n; i++) r[i] = mod_mul(x[i], y[i], c->moduli[i]);
}

/* ceil(log2(x)) as the reference's DEVICE code obtains it (CUDA's log2,
 * src/rns.cuh:848, :913): the exact ceiling, corrected within a few ulps of a
 * power of two by the deviations of CUDA's log2 measured on the GPU
 * (cuda_log2_table.h, made by gen_cuda_log2_table.py). */
static double exact_ceil_log2(double x) {
    int e;
    double m = frexp(x, &e); /* x = m * 2^e, m in [0.5, 1) */
    return (m == 0.5) ? e - 1 : e;
}
static int log2_row_lo[2100], log2_row_hi[2100]; /* rows of each binade in the table */
static int log2_index_ready;
static void log2_index(void) {
    for (int i = 0; i < 2100; i++) log2_row_lo[i] = log2_row_hi[i] = 0;
    for (int r = 0; r < ORA_CUDA_LOG2_RUNS; r++) {
        int b = ORA_CUDA_LOG2_TABLE[r][0] + 1074;
        if (log2_row_hi[b] == 0) log2_row_lo[b] = r;
        log2_row_hi[b] = r + 1;
    }
    log2_index_ready = 1;
}
static int log2_delta(int e, int64_t steps) {
    if (e < -1074 || e > 1023) return 0;
    int b = e + 1074;
    for (int r = log2_row_lo[b]; r < log2_row_hi[b]; r++)
        if (steps >= ORA_CUDA_LOG2_TABLE[r][1] && steps <= ORA_CUDA_LOG2_TABLE[r][2]) return ORA_CUDA_LOG2_TABLE[r][3];
    return 0;
}
static double dev_ceil_log2(double x) {
    if (!log2_index_ready) {
#pragma omp critical(ora_log2)
        if (!log2_index_ready) log2_index();
    }
    int e;
    frexp(x, &e);
    e -= 1; /* 2^e <= x < 2^(e+1) */
    int64_t bx = (int64_t)bits_of(x);
    int64_t below = bx - (int64_t)bits_of(ldexp(1.0, e));       /* steps above 2^e, >= 0 */
    int64_t above = bx - (int64_t)bits_of(ldexp(1.0, e + 1));   /* steps below 2^(e+1), < 0 */
    int d = log2_delta(e, below);
    if (!d) d = log2_delta(e + 1, above);
    return exact_ceil_log2(x) + d;
}

/* the refinement loop shared by rns_eval_compute[_fast] (src/rns.cuh:843-867, :908-932) */
static void eval_refine(const ora_ctx_t *c, int *s, double sumu, er_t *low, er_t *upp) {
    const int n = c->n;
    double fracl[ORA_MAXN], fracu[ORA_MAXN];
    int K = 0;
    while (sumu < c->eval_acc) {
        int k;
        if (sumu == 0) {
            /* log2(0) = -inf: the reference's row index saturates past RNS_POW2; the
             * library clamps it to the last row, and so does the oracle */
            k = c->log2m;
        } else {
            double a = -(dev_ceil_log2(sumu) + 1);
            k = (int)(a > c->ref_factor ? a : c->ref_factor);
            if (k > c->log2m) k = c->log2m;
        }
        rns_mul(c, s, s, &c->pow2[k * n]);
        for (int i = 0; i < n; i++) fracu[i] = mul_ru(s[i], c->recip_ru[i]);
        sumu = psum(fracu, n, add_ru);
        sumu = sub_ru(sumu, (unsigned int)sumu);
        K += k;
    }
    for (int i = 0; i < n; i++) fracl[i] = mul_rd(s[i], c->recip_rd[i]);
    double suml = psum(fracl, n, add_rd);
    suml = sub_rd(suml, (unsigned int)suml);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    low->exp -= K;
    upp->exp -= K;
}

/* src/rns.cuh:878-933 (cuda::rns_eval_compute_fast) */
static void eval_fast(const ora_ctx_t *c, er_t *low, er_t *upp, const int *x) {
    const int n = c->n;
    int s[ORA_MAXN];
    double fracl[ORA_MAXN], fracu[ORA_MAXN];
    rns_mul(c, s, x, c->part_inv);
    for (int i = 0; i < n; i++) {
        fracl[i] = mul_rd(s[i], c->recip_rd[i]);
        fracu[i] = mul_ru(s[i], c->recip_ru[i]);
    }
    double suml = psum(fracl, n, add_rd);
    double sumu = psum(fracu, n, add_ru);
    if (suml == 0 && sumu == 0) {
        low->frac = 0; low->exp = 0;
        upp->frac = 0; upp->exp = 0;
        return;
    }
    suml = sub_rd(suml, (unsigned int)suml);
    sumu = sub_ru(sumu, (unsigned int)sumu);
    if (sumu >= c->eval_acc) {
        er_set_d(low, suml);
        er_set_d(upp, sumu);
        return;
    }
    eval_refine(c, s, sumu, low, upp);
}

/* src/rns.cuh:797-868 (cuda::rns_eval_compute) */
static void eval_full(const ora_ctx_t *c, er_t *low, er_t *upp, const int *x) {
    const int n = c->n;
    int s[ORA_MAXN];
    double fracl[ORA_MAXN], fracu[ORA_MAXN];
    rns_mul(c, s, x, c->part_inv);
    for (int i = 0; i < n; i++) {
        fracl[i] = mul_rd(s[i], c->recip_rd[i]);
        fracu[i] = mul_ru(s[i], c->recip_ru[i]);
    }
    double suml = psum(fracl, n, add_rd);
    double sumu = psum(fracu, n, add_ru);
    if (suml == 0 && sumu == 0) {
        low->frac = 0; low->exp = 0;
        upp->frac = 0; upp->exp = 0;
        return;
    }
    unsigned int whl = (unsigned int)suml, whu = (unsigned int)sumu;
    suml = sub_rd(suml, whl);
    sumu = sub_ru(sumu, whu);
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    int mr = -1;
    if (whl != whu) mr = mrd(c, x);
    if (mr > 0) {
        *upp = c->inv_unit_upp;
        return;
    }
    if (mr == 0) *low = c->unit_low;
    if (sumu >= c->eval_acc) return;
    eval_refine(c, s, sumu, low, upp);
}

/* src/rns.cuh:1061-1079 (cuda::rns_rank_compute) */
static int rank_full(const ora_ctx_t *c, const int *x, const int *s) {
    const int n = c->n;
    double fracl[ORA_MAXN], fracu[ORA_MAXN];
    for (int i = 0; i < n; i++) {
        fracl[i] = mul_rd(s[i], c->recip_rd[i]);
        fracu[i] = mul_ru(s[i], c->recip_ru[i]);
    }
    double suml = psum(fracl, n, add_rd);
    double sumu = psum(fracu, n, add_ru);
    unsigned int whl = (unsigned int)suml, whu = (unsigned int)sumu;
    if (whl == whu) return (int)whl;
    return (mrd(c, x) == 0) ? (int)whu : (int)whl;
}
/* src/rns.cuh:1088-1096 (cuda::rns_rank_compute_fast) */
static int rank_fast(const ora_ctx_t *c, const int *s) {
    double fracu[ORA_MAXN];
    for (int i = 0; i < c->n; i++) fracu[i] = mul_ru(s[i], c->recip_ru[i]);
    return (int)psum(fracu, c->n, add_ru);
}
/* src/rns.cuh:1101-1124 (cuda::make_scaling_step) */
static void scaling_step(const ora_ctx_t *c, int *y, int k, unsigned j, int pow2j, const int *x, const int *cc) {
    const int n = c->n;
    int64_t residue = 0;
    for (int i = 0; i < n; i++) residue += (int64_t)mod_mul(c->part_pow2_res[j - 1][i], cc[i], pow2j);
    int64_t temp = (int64_t)k * (int64_t)c->m_pow2_res[j - 1];
    residue = (residue - temp) % pow2j;
    if (residue < 0) residue += pow2j;
    for (int i = 0; i < n; i++) {
        int multiple = (int)(residue % c->moduli[i]);
        multiple = mod_psub(x[i], multiple, c->moduli[i]);
        y[i] = mod_mul(multiple, c->pow2_inv[j - 1][i], c->moduli[i]);
    }
}
/* src/rns.cuh:1132-1158 (cuda::rns_scale2pow); result may alias x */
static void scale2pow(const ora_ctx_t *c, int *result, const int *xin, unsigned D) {
    const int n = c->n;
    int x[ORA_MAXN], cc[ORA_MAXN];
    memcpy(x, xin, sizeof(int) * n);
    for (int i = 0; i < n; i++) result[i] = x[i];
    int t = D / ORA_T;
    int k;
    if (t > 0) {
        rns_mul(c, cc, x, c->part_inv);
        k = rank_full(c, x, cc);
        scaling_step(c, result, k, ORA_T, 1 << ORA_T, x, cc);
        t -= 1;
    }
    while (t > 0) {
        rns_mul(c, cc, result, c->part_inv);
        k = rank_fast(c, cc);
        scaling_step(c, result, k, ORA_T, 1 << ORA_T, result, cc);
        t -= 1;
    }
    unsigned d = D % ORA_T;
    if (d > 0) {
        rns_mul(c, cc, result, c->part_inv);
        k = (d < D) ? rank_full(c, result, cc) : rank_fast(c, cc);
        scaling_step(c, result, k, d, 1 << d, result, cc);
    }
}

/* ------------------------------------------------------------------------- */
/* multiple-precision arithmetic, device half of src/arith/                  */
/* ------------------------------------------------------------------------- */

/* Rounding of a result (src/arith/arith_utils.cuh:181-190; the same test and
 * steps as mp_vector_round_kernel, src/mpvector.cuh:669-688, and
 * mp_matrix_round_kernel, src/mpmatrix.cuh:410-428). */
static void mp_round_if_needed(const ora_ctx_t *c, mpf_t *x) {
    int bits = (int)((x->eval[1].exp - c->mp_h + 1) * (x->eval[1].frac != 0));
    if (bits > 0) {
        x->exp += bits;
        scale2pow(c, x->digits, x->digits, (unsigned)bits);
        eval_fast(c, &x->eval[0], &x->eval[1], x->digits);
    }
}

static inline int pow2_row(const ora_ctx_t *c, int idx) {
    /* the reference indexes RNS_POW2 past its last row when the operand that
     * index scales is zero; the product with zero digits is 0 whatever the row */
    return idx > c->log2m ? c->log2m : idx;
}

/* src/arith/arith_utils.cuh:197-206 (cuda::sign_estimate) */
static int sign_estimate(const ora_ctx_t *c, const int *dx, const int *dy, int sx, int sy, int gamma, int theta,
                         int nzx, int nzy) {
    int lx[ORA_MAXN] = {0}, ly[ORA_MAXN] = {0};
    const int *pg = &c->pow2[pow2_row(c, gamma) * c->n], *pt = &c->pow2[pow2_row(c, theta) * c->n];
    for (int i = 0; i < c->n; i++) {
        lx[i] = nzx * mod_mul(dx[i], pg[i], c->moduli[i]);
        ly[i] = nzy * mod_mul(dy[i], pt[i], c->moduli[i]);
    }
    int cmp = mrc_compare(c, lx, ly);
    return (cmp < 0 ? sy : sx) * (cmp != 0);
}

/* src/arith/add.cuh:126-188 (cuda::mp_add_common) followed by the rounding of
 * the mp_add overloads (:190-271) */
static void mp_add(const ora_ctx_t *c, mpf_t *r, const mpf_t *xin, const mpf_t *yin) {
    const int n = c->n;
    mpf_t x = *xin, y = *yin;
    int ex = x.exp, ey = y.exp, sx = x.sign, sy = y.sign;
    er_t *evalx = x.eval, *evaly = y.eval;
    int dexp = ex - ey;
    int gamma = dexp * (dexp > 0);
    int theta = -dexp * (dexp < 0);
    const int nzx = ((evaly[1].frac == 0) || (theta + evaly[1].exp) < c->mp_j);
    const int nzy = ((evalx[1].frac == 0) || (gamma + evalx[1].exp) < c->mp_j);
    gamma = gamma * nzy;
    theta = theta * nzx;
    ex = (ex - gamma) * nzx;
    ey = (ey - theta) * nzy;
    sx *= nzx;
    sy *= nzy;
    int factor_x = (1 - 2 * sx) * nzx;
    int factor_y = (1 - 2 * sy) * nzy;
    evalx[0].exp += gamma;
    evalx[1].exp += gamma;
    evaly[0].exp += theta;
    evaly[1].exp += theta;
    evalx[0].frac *= factor_x;
    evalx[1].frac *= factor_x;
    evaly[0].frac *= factor_y;
    evaly[1].frac *= factor_y;
    er_t lo = er_add_dir(evalx[sx], evaly[sy], 0);
    er_t up = er_add_dir(evalx[1 - sx], evaly[1 - sy], 1);
    er_t ev[2] = {lo, up};
    unsigned char sign = ev[0].frac < 0;
    if (sign != (ev[1].frac < 0)) {
        sign = (unsigned char)sign_estimate(c, x.digits, y.digits, sx, sy, gamma, theta, nzx, nzy);
        ev[sign].frac = c->unit_low.frac * (1 - 2 * sign);
        ev[sign].exp = c->unit_low.exp;
    }
    mpf_t out;
    out.sign = sign;
    out.exp = (ex == 0) ? ey : ex;
    /* src/modular.cuh:306-314 (cuda::rns_axby_cd) */
    const int *pg = &c->pow2[pow2_row(c, gamma) * n], *pt = &c->pow2[pow2_row(c, theta) * n];
    for (int i = 0; i < n; i++) {
        int64_t res = (int64_t)pg[i] * (int64_t)x.digits[i] * (int64_t)factor_x +
                      (int64_t)pt[i] * (int64_t)y.digits[i] * (int64_t)factor_y;
        res = res % (int64_t)c->moduli[i];
        out.digits[i] = (int)res + (res < 0) * c->moduli[i];
    }
    if (sign == 1) {
        for (int i = 0; i < n; i++) out.digits[i] = (out.digits[i] != 0) * (c->moduli[i] - out.digits[i]);
        er_t tmp = ev[0];
        ev[0].frac = -ev[1].frac;
        ev[0].exp = ev[1].exp;
        ev[1].frac = -1 * tmp.frac;
        ev[1].exp = tmp.exp;
    }
    out.eval[0] = ev[0];
    out.eval[1] = ev[1];
    if (out.eval[1].frac != 0 && out.eval[1].exp >= c->mp_h) {
        int bits = (int)(out.eval[1].exp - c->mp_h + 1);
        if (bits > 0) {
            out.exp += bits;
            scale2pow(c, out.digits, out.digits, (unsigned)bits);
            eval_fast(c, &out.eval[0], &out.eval[1], out.digits);
        }
    }
    *r = out;
}

/* src/arith/addabs.cuh:81-127 (cuda::mp_add_abs_common + rounding): |x| + |y| */
static void mp_add_abs(const ora_ctx_t *c, mpf_t *r, const mpf_t *xin, const mpf_t *yin) {
    const int n = c->n;
    mpf_t x = *xin, y = *yin;
    int ex = x.exp, ey = y.exp;
    er_t *evalx = x.eval, *evaly = y.eval;
    int dexp = ex - ey;
    int gamma = dexp * (dexp > 0);
    int theta = -dexp * (dexp < 0);
    const int nzx = ((evaly[1].frac == 0) || (theta + evaly[1].exp) < c->mp_j);
    const int nzy = ((evalx[1].frac == 0) || (gamma + evalx[1].exp) < c->mp_j);
    gamma = gamma * nzy;
    theta = theta * nzx;
    ex = (ex - gamma) * nzx;
    ey = (ey - theta) * nzy;
    mpf_t out;
    out.exp = (ex == 0) ? ey : ex;
    out.sign = 0;
    evalx[0].exp += gamma;
    evalx[1].exp += gamma;
    evaly[0].exp += theta;
    evaly[1].exp += theta;
    evalx[0].frac *= nzx;
    evalx[1].frac *= nzx;
    evaly[0].frac *= nzy;
    evaly[1].frac *= nzy;
    out.eval[0] = er_add_dir(evalx[0], evaly[0], 0);
    out.eval[1] = er_add_dir(evalx[1], evaly[1], 1);
    const int *pg = &c->pow2[pow2_row(c, gamma) * n], *pt = &c->pow2[pow2_row(c, theta) * n];
    for (int i = 0; i < n; i++) {
        int64_t res = (int64_t)pg[i] * (int64_t)x.digits[i] * (int64_t)nzx + (int64_t)pt[i] * (int64_t)y.digits[i] * (int64_t)nzy;
        res = res % (int64_t)c->moduli[i];
        out.digits[i] = (int)res + (res < 0) * c->moduli[i];
    }
    mp_round_if_needed(c, &out);
    *r = out;
}

/* src/arith/mul.cuh:53-113 (cuda::mp_mul_common + rounding); the split kernels
 * mp_vector_mul_esi/digits_kernel + mp_vector_round_kernel compute the same. */
static void mp_mul(const ora_ctx_t *c, mpf_t *r, const mpf_t *x, const mpf_t *y) {
    mpf_t out;
    out.exp = x->exp + y->exp;
    out.sign = x->sign ^ y->sign;
    out.eval[0] = er_md_rd(x->eval[0], y->eval[0], c->unit_upp);
    out.eval[1] = er_md_ru(x->eval[1], y->eval[1], c->unit_low);
    rns_mul(c, out.digits, x->digits, y->digits);
    mp_round_if_needed(c, &out);
    *r = out;
}

/* src/arith/muld.cuh:59-74 (cuda::mp_mul_d) */
static void mp_mul_d(const ora_ctx_t *c, mpf_t *r, const mpf_t *x, double y) {
    uint64_t u = bits_of(y);
    int64_t significand = (int64_t)(((u & (((uint64_t)1 << 52) - 1)) | ((uint64_t)1 << 52)) * (uint64_t)(y != 0));
    int dexp = (int)(((u >> 52) & 2047) - (uint64_t)(1023 + 52) * (y != 0));
    mpf_t out;
    out.exp = x->exp + dexp;
    out.sign = x->sign ^ (int)(u >> 63);
    out.eval[0].exp = x->eval[0].exp;
    out.eval[1].exp = x->eval[1].exp;
    out.eval[0].frac = mul_rd(x->eval[0].frac, (double)significand);
    out.eval[1].frac = mul_ru(x->eval[1].frac, (double)significand);
    er_adjust(&out.eval[0]);
    er_adjust(&out.eval[1]);
    for (int i = 0; i < c->n; i++) out.digits[i] = mod_mul(x->digits[i], (int)(significand % c->moduli[i]), c->moduli[i]);
    mp_round_if_needed(c, &out);
    *r = out;
}

/* ------------------------------------------------------------------------- */
/* host conversion, src/arith/assign.cuh:54-81 with the host evaluation       */
/* src/rns.cuh:645-716 (emulated rounding of src/dinterval.cuh)               */
/* ------------------------------------------------------------------------- */

static int host_mrd(const ora_ctx_t *c, const int *x) {
    /* src/rns.cuh:514-531: same digit recurrence with the long-typed subtraction */
    int mixed[ORA_MAXN];
    for (int i = 0; i < c->n; i++) {
        mixed[i] = x[i];
        for (int j = 0; j < i; j++) {
            if (mixed[i] < mixed[j]) mixed[i] = (int)((int64_t)c->moduli[i] - (int64_t)mixed[j] + (int64_t)mixed[i]);
            else mixed[i] = mixed[i] - mixed[j];
            mixed[i] = mod_mul(mixed[i], c->mrc_inv[j][i], c->moduli[i]);
        }
    }
    return mixed[c->n - 1];
}

static void host_eval(const ora_ctx_t *c, er_t *low, er_t *upp, const int *x) {
    const int n = c->n;
    int s[ORA_MAXN];
    double fracl[ORA_MAXN], fracu[ORA_MAXN];
    int zero = 1;
    for (int i = 0; i < n; i++) zero &= (x[i] == 0);
    if (zero) {
        low->frac = 0; low->exp = 0;
        upp->frac = 0; upp->exp = 0;
        return;
    }
    for (int i = 0; i < n; i++) s[i] = host_mod_mul_d(x[i], c->part_inv[i], c->moduli[i], 1.0 / c->moduli[i]);
    for (int i = 0; i < n; i++) {
        fracl[i] = host_rd(s[i] * c->recip_rd[i]);
        fracu[i] = host_ru(s[i] * c->recip_ru[i]);
    }
    double suml = psum(fracl, n, host_add_rd);
    double sumu = psum(fracu, n, host_add_ru);
    unsigned int whl = (unsigned int)suml, whu = (unsigned int)sumu;
    suml = suml - whl;
    sumu = sumu - whu;
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    int mr = -1;
    if (whl != whu) mr = host_mrd(c, x);
    if (mr > 0) {
        *upp = c->inv_unit_upp;
        return;
    }
    if (mr == 0) *low = c->unit_low;
    if (sumu >= c->eval_acc) return;
    int K = 0;
    while (sumu < c->eval_acc) {
        double a = -(ceil(log2(sumu)) + 1);
        int k = (int)(a > c->ref_factor ? a : c->ref_factor);
        for (int i = 0; i < n; i++) s[i] = host_mod_mul_d(s[i], c->pow2[k * n + i], c->moduli[i], 1.0 / c->moduli[i]);
        for (int i = 0; i < n; i++) fracu[i] = host_ru((double)s[i] / (double)c->moduli[i]);
        sumu = psum(fracu, n, host_add_ru);
        sumu -= (unsigned int)sumu;
        K += k;
    }
    for (int i = 0; i < n; i++) fracl[i] = host_rd((double)s[i] / (double)c->moduli[i]);
    suml = psum(fracl, n, host_add_rd);
    suml -= (unsigned int)suml;
    er_set_d(low, suml);
    er_set_d(upp, sumu);
    low->exp -= K;
    upp->exp -= K;
}

static void set_d(const ora_ctx_t *c, mpf_t *r, double x) {
    uint64_t u = bits_of(x);
    int sign = (int)(u >> 63);
    int exp = (int)((u >> 52) & 2047);
    int64_t significand;
    if (exp == 0) significand = (int64_t)(u & (((uint64_t)1 << 52) - 1));
    else significand = (int64_t)((u & (((uint64_t)1 << 52) - 1)) | ((uint64_t)1 << 52));
    exp = exp - 1023 - 52;
    if (significand != 0) {
        while ((significand & 1) == 0) {
            significand >>= 1;
            exp++;
        }
    } else {
        exp = 0;
    }
    mpf_t out;
    memset(&out, 0, sizeof(out));
    out.sign = sign;
    out.exp = exp;
    for (int i = 0; i < c->n; i++) out.digits[i] = (int)(significand % (int64_t)c->moduli[i]);
    host_eval(c, &out.eval[0], &out.eval[1], out.digits);
    /* a 53-bit significand never reaches the rounding threshold 2^-MP_H of any set */
    *r = out;
}

/* ------------------------------------------------------------------------- */
/* exported element-wise entry points                                        */
/* ------------------------------------------------------------------------- */

void ora_set_d(int n, const double *x, long count, void *out) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) {
        mpf_t r;
        set_d(c, &r, x[i]);
        store_mp(n, out, i, &r);
    }
}

void ora_add(int n, const void *x, const void *y, void *r, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) {
        mpf_t a, b, o;
        load_mp(n, x, i, &a);
        load_mp(n, y, i, &b);
        mp_add(c, &o, &a, &b);
        store_mp(n, r, i, &o);
    }
}

void ora_mul(int n, const void *x, const void *y, void *r, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) {
        mpf_t a, b, o;
        load_mp(n, x, i, &a);
        load_mp(n, y, i, &b);
        mp_mul(c, &o, &a, &b);
        store_mp(n, r, i, &o);
    }
}

void ora_mul_d(int n, const void *x, const double *y, void *r, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) {
        mpf_t a, o;
        load_mp(n, x, i, &a);
        mp_mul_d(c, &o, &a, y[i]);
        store_mp(n, r, i, &o);
    }
}

void ora_eval_fast(int n, const int *digits, ora_er_t *low, ora_er_t *upp, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) eval_fast(c, &low[i], &upp[i], digits + (size_t)i * n);
}

void ora_eval(int n, const int *digits, ora_er_t *low, ora_er_t *upp, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) eval_full(c, &low[i], &upp[i], digits + (size_t)i * n);
}

void ora_scale2pow(int n, const int *digits, const unsigned *D, int *out, long count) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; i++) scale2pow(c, out + (size_t)i * n, digits + (size_t)i * n, D[i]);
}

/* ------------------------------------------------------------------------- */
/* BLAS in kernel order                                                      */
/* ------------------------------------------------------------------------- */

static unsigned next_pow2(unsigned v) {
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    return v + 1;
}

static long bl_index(long i, int len, int inc) { return inc > 0 ? i * inc : (-(long)len + i + 1) * inc; }

/* the shared-memory tree of src/mpreduct.cuh:59-67 and src/blas/gemv.cuh:60-68 */
static void block_tree(const ora_ctx_t *c, mpf_t *s, int bsize) {
    for (unsigned i = next_pow2((unsigned)bsize) >> 1; i >= 1; i >>= 1)
        for (unsigned t = 0; t < i; t++)
            if (t + i < (unsigned)bsize) mp_add(c, &s[t], &s[t], &s[t + i]);
}

/* cuda::mp_dot<g1,b1,g2,g3,b3> (src/blas/dot.cuh:85-108): products by
 * mp_vector_mul_{esi,digits}_kernel + mp_vector_round_kernel (src/mpvector.cuh),
 * then mp_array_reduce_sum_kernel1 over g3 blocks of b3 threads and
 * mp_array_reduce_sum_kernel2 over one block (src/mpreduct.cuh:38-115). */
void ora_dot(int n, int len, const void *x, int incx, const void *y, int incy, void *r, int g3, int b3) {
    const ora_ctx_t *c = ora_init(n);
    if (len <= 0) return;
    const long K = (long)g3 * b3;
    mpf_t *part = (mpf_t *)malloc(sizeof(mpf_t) * K);
#pragma omp parallel for schedule(dynamic, 16)
    for (long p = 0; p < K; p++) {
        mpf_t acc, a, b, prod;
        mp_zero(&acc);
        for (long i = p; i < len; i += K) {
            load_mp(n, x, bl_index(i, len, incx), &a);
            load_mp(n, y, bl_index(i, len, incy), &b);
            mp_mul(c, &prod, &a, &b);
            mp_add(c, &acc, &acc, &prod);
        }
        part[p] = acc;
    }
    mpf_t *blk = (mpf_t *)malloc(sizeof(mpf_t) * g3);
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < g3; b++) {
        block_tree(c, &part[(long)b * b3], b3);
        blk[b] = part[(long)b * b3];
    }
    mpf_t *s = (mpf_t *)malloc(sizeof(mpf_t) * b3);
    for (int t = 0; t < b3; t++) {
        mp_zero(&s[t]);
        for (int i = t; i < g3; i += b3) mp_add(c, &s[t], &s[t], &blk[i]);
    }
    block_tree(c, s, b3);
    store_mp(n, r, 0, &s[0]);
    free(s);
    free(blk);
    free(part);
}

void ora_add_abs(int n, const void *x, const void *y, void *r, long count) {
    const ora_ctx_t *c = ora_init(n);
    for (long i = 0; i < count; i++) {
        mpf_t a, b, out;
        load_mp(n, x, i, &a);
        load_mp(n, y, i, &b);
        mp_add_abs(c, &out, &a, &b);
        store_mp(n, r, i, &out);
    }
}

static void block_tree_abs(const ora_ctx_t *c, mpf_t *s, int bsize) {
    for (unsigned i = next_pow2((unsigned)bsize) >> 1; i >= 1; i >>= 1)
        for (unsigned t = 0; t < i; t++)
            if (t + i < (unsigned)bsize) mp_add_abs(c, &s[t], &s[t], &s[t + i]);
}

/* cuda::mp_dot<blocks, threads> (src/blas/v2/dot_v2.cuh) and the sum of squares
 * of cuda::mp_norm2<blocks, threads> (src/blas/v2/norm2_v2.cuh:39-123, with
 * mp_add_abs): the v1 two-pass order over AoS vectors with unit strides.
 * sumsq: r[0] = sum |x_i x_i|, y unused. */
void ora_reduce_v2(int n, int sumsq, int len, const void *x, const void *y, void *r, int blocks, int threads) {
    const ora_ctx_t *c = ora_init(n);
    const long K = (long)blocks * threads;
    mpf_t *part = (mpf_t *)malloc(sizeof(mpf_t) * K);
#pragma omp parallel for schedule(dynamic, 16)
    for (long p = 0; p < K; p++) {
        mpf_t acc, a, b, prod;
        mp_zero(&acc);
        for (long i = p; i < len; i += K) {
            load_mp(n, x, i, &a);
            if (sumsq) {
                mp_mul(c, &prod, &a, &a);
                mp_add_abs(c, &acc, &acc, &prod);
            } else {
                load_mp(n, y, i, &b);
                mp_mul(c, &prod, &a, &b);
                mp_add(c, &acc, &acc, &prod);
            }
        }
        part[p] = acc;
    }
    mpf_t *blk = (mpf_t *)malloc(sizeof(mpf_t) * blocks);
    for (int b = 0; b < blocks; b++) {
        if (sumsq) block_tree_abs(c, &part[(long)b * threads], threads);
        else block_tree(c, &part[(long)b * threads], threads);
        blk[b] = part[(long)b * threads];
    }
    mpf_t *s = (mpf_t *)malloc(sizeof(mpf_t) * threads);
    for (int t = 0; t < threads; t++) {
        mp_zero(&s[t]);
        for (int i = t; i < blocks; i += threads) {
            if (sumsq) mp_add_abs(c, &s[t], &s[t], &blk[i]);
            else mp_add(c, &s[t], &s[t], &blk[i]);
        }
    }
    if (sumsq) block_tree_abs(c, s, threads);
    else block_tree(c, s, threads);
    store_mp(n, r, 0, &s[0]);
    free(s);
    free(blk);
    free(part);
}

/* cuda::mp_gemv<g1,b1,g2,b3> (src/blas/gemv.cuh:151-269): buffer1 = alpha*x,
 * y = beta*y, buffer2 = A*diag(buffer1) (or diag(buffer1)*A), then per row
 * (column) a strided serial sum over b3 threads, the shared tree, and
 * y = y + sum (matrix_row_sum_kernel / matrix_col_sum_kernel, :44-128). */
void ora_gemv(int n, int trans, int m, int cols, const void *alpha, const void *A, int lda, const void *x,
              int incx, const void *beta, void *y, int incy, int b3) {
    const ora_ctx_t *c = ora_init(n);
    if (m <= 0 || cols <= 0) return;
    if (incx == 0 || incy == 0 || lda < (m > 1 ? m : 1)) return;
    const int nt = (trans == 111);
    const int lx = nt ? cols : m, ly = nt ? m : cols;
    mpf_t al, be;
    load_mp(n, alpha, 0, &al);
    load_mp(n, beta, 0, &be);
    mpf_t *b1 = (mpf_t *)malloc(sizeof(mpf_t) * lx);
#pragma omp parallel for schedule(static)
    for (long j = 0; j < lx; j++) {
        mpf_t v;
        load_mp(n, x, bl_index(j, lx, incx), &v);
        mp_mul(c, &b1[j], &v, &al);
    }
    mpf_t *yy = (mpf_t *)malloc(sizeof(mpf_t) * ly);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ly; i++) {
        mpf_t v;
        load_mp(n, y, bl_index(i, ly, incy), &v);
        mp_mul(c, &yy[i], &v, &be);
    }
    const int outer = nt ? m : cols, inner = nt ? cols : m;
#pragma omp parallel for schedule(dynamic, 1)
    for (int o = 0; o < outer; o++) {
        mpf_t *s = (mpf_t *)malloc(sizeof(mpf_t) * b3);
        for (int t = 0; t < b3; t++) {
            mp_zero(&s[t]);
            for (int i = t; i < inner; i += b3) {
                /* element (row, col) of buffer2 = A(row, col) * buffer1(col or row) */
                int row = nt ? o : i, col = nt ? i : o;
                mpf_t a, prod;
                load_mp(n, A, (long)col * lda + row, &a);
                mp_mul(c, &prod, &a, &b1[nt ? col : row]);
                mp_add(c, &s[t], &s[t], &prod);
            }
        }
        block_tree(c, s, b3);
        mp_add(c, &yy[o], &yy[o], &s[0]);
        free(s);
    }
    for (long i = 0; i < ly; i++) store_mp(n, y, bl_index(i, ly, incy), &yy[i]);
    free(yy);
    free(b1);
}

/* cuda::mp_gemm NN (src/blas/gemm.cuh:70-168): buffer = A*B by a serial k chain
 * per element (matrix_multiply_notrans_kernel, :39-60), buffer = alpha*buffer,
 * C = beta*C, then C = C + buffer by the split esi/digits kernels
 * (src/mpmatrix.cuh:47-166) and the final rounding. */
void ora_gemm(int n, int m, int cols, int k, const void *alpha, const void *A, int lda, const void *B, int ldb,
              const void *beta, void *C, int ldc) {
    const ora_ctx_t *c = ora_init(n);
    if (m <= 0 || cols <= 0 || k <= 0) return;
    if (lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1)) return;
    mpf_t al, be;
    load_mp(n, alpha, 0, &al);
    load_mp(n, beta, 0, &be);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int col = 0; col < cols; col++) {
        for (int row = 0; row < m; row++) {
            mpf_t sum, mul, a, b, cc;
            mp_zero(&sum);
            for (int i = 0; i < k; i++) {
                load_mp(n, A, (long)lda * i + row, &a);
                load_mp(n, B, (long)col * ldb + i, &b);
                mp_mul(c, &mul, &a, &b);
                mp_add(c, &sum, &sum, &mul);
            }
            mpf_t buf;
            mp_mul(c, &buf, &sum, &al); /* mp_mat2scal_mul_* + mp_matrix_round_kernel */
            load_mp(n, C, (long)col * ldc + row, &cc);
            mp_mul(c, &cc, &cc, &be);
            /* mp_matrix_add_esi_kernel (src/mpmatrix.cuh:47-126) */
            er_t evalA[2] = {cc.eval[0], cc.eval[1]}, evalB[2] = {buf.eval[0], buf.eval[1]};
            int expA = cc.exp, expB = buf.exp, signA = cc.sign, signB = buf.sign;
            int dexp = expA - expB;
            int gamma = dexp * (dexp > 0);
            int theta = -dexp * (dexp < 0);
            int nzA = ((evalB[1].frac == 0) || (theta + evalB[1].exp) < c->mp_j);
            int nzB = ((evalA[1].frac == 0) || (gamma + evalA[1].exp) < c->mp_j);
            gamma = gamma * nzB;
            theta = theta * nzA;
            expA = (expA - gamma) * nzA;
            expB = (expB - theta) * nzB;
            signA *= nzA;
            signB *= nzB;
            int factorA = (1 - 2 * signA) * nzA;
            int factorB = (1 - 2 * signB) * nzB;
            evalA[0].exp += gamma; evalA[1].exp += gamma;
            evalB[0].exp += theta; evalB[1].exp += theta;
            evalA[0].frac *= factorA; evalA[1].frac *= factorA;
            evalB[0].frac *= factorB; evalB[1].frac *= factorB;
            mpf_t res;
            res.eval[0] = er_add_dir(evalA[signA], evalB[signB], 0);
            res.eval[1] = er_add_dir(evalA[1 - signA], evalB[1 - signB], 1);
            res.exp = (expA == 0) ? expB : expA;
            int minus = res.eval[0].frac < 0 && res.eval[1].frac < 0;
            res.sign = minus;
            if (minus) {
                er_t tmp = res.eval[0];
                res.eval[0].frac = -res.eval[1].frac;
                res.eval[0].exp = res.eval[1].exp;
                res.eval[1].frac = -tmp.frac;
                res.eval[1].exp = tmp.exp;
            }
            /* mp_matrix_add_digits_kernel (src/mpmatrix.cuh:143-166) */
            const int *pg = &c->pow2[pow2_row(c, gamma) * n], *pt = &c->pow2[pow2_row(c, theta) * n];
            for (int i = 0; i < n; i++) {
                int lm = c->moduli[i];
                int residue = dev_mod_axby_d(factorA * cc.digits[i], pg[i], factorB * buf.digits[i], pt[i], lm,
                                             1.0 / lm);
                if (res.sign == 1) residue = mod_sub(lm, residue, lm);
                res.digits[i] = residue < 0 ? residue + lm : residue;
            }
            mp_round_if_needed(c, &res);
            store_mp(n, C, (long)col * ldc + row, &res);
        }
    }
}

/* cuda::mp_spmv_csr<threads> (src/sparse/spmv/spmv_csr.cuh:49-63) */
void ora_spmv_csr(int n, int m, const int *irp, const int *ja, const double *as, const void *x, void *y) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int row = 0; row < m; row++) {
        mpf_t sum, prod, xv;
        mp_zero(&sum);
        for (int i = irp[row]; i < irp[row + 1]; i++) {
            load_mp(n, x, ja[i], &xv);
            mp_mul_d(c, &prod, &xv, as[i]);
            mp_add(c, &sum, &sum, &prod);
        }
        store_mp(n, y, row, &sum);
    }
}

/* cuda::mp_spmv_csrv<threads, tpr> (src/sparse/spmv/spmv_csrv.cuh:49-86):
 * lane-strided partial sums, then the lane tree 16, 8, 4, 2, 1 */
void ora_spmv_csrv(int n, int m, int tpr, const int *irp, const int *ja, const double *as, const void *x, void *y) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int row = 0; row < m; row++) {
        mpf_t sums[32], prod, xv;
        for (int lane = 0; lane < tpr; lane++) {
            mp_zero(&sums[lane]);
            for (int i = irp[row] + lane; i < irp[row + 1]; i += tpr) {
                load_mp(n, x, ja[i], &xv);
                mp_mul_d(c, &prod, &xv, as[i]);
                mp_add(c, &sums[lane], &sums[lane], &prod);
            }
        }
        for (int s = 16; s >= 1; s >>= 1)
            if (tpr >= 2 * s)
                for (int lane = 0; lane < s; lane++) mp_add(c, &sums[lane], &sums[lane], &sums[lane + s]);
        store_mp(n, y, row, &sums[0]);
    }
}

/* cuda::mp_spmv_ell<threads> (src/sparse/spmv/spmv_ell.cuh:50-67): column-major
 * slots, explicit zeros skipped */
void ora_spmv_ell(int n, int m, int maxnzr, const int *ja, const double *as, const void *x, void *y) {
    const ora_ctx_t *c = ora_init(n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int row = 0; row < m; row++) {
        mpf_t sum, prod, xv;
        mp_zero(&sum);
        for (int col = 0; col < maxnzr; col++) {
            int j = ja[(long)col * m + row];
            double val = as[(long)col * m + row];
            if (val != 0) {
                load_mp(n, x, j, &xv);
                mp_mul_d(c, &prod, &xv, val);
                mp_add(c, &sum, &sum, &prod);
            }
        }
        store_mp(n, y, row, &sum);
    }
}
