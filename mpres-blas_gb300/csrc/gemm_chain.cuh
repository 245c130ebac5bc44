/*
 * The lazy-residue k chain of mp_gemm as device functions, shared by the plain
 * kernels (gemm.cu) and the GEMM tiles of the persistent batch kernel
 * (batch.cu): W(A), W(B) encoding, the scalar half of a step, the out-of-line
 * full step, the per-output chain and the epilogue (C + alpha*A*B as the
 * reference's split kernels, src/mpmatrix.cuh:47-166).  Each including
 * translation unit has its own tables (MPRES_DEFINE_TABLES) and evaluation
 * form (MPRES_EVAL_FIXED_POINT); the results are the same bits either way.
 */
#ifndef MPRES_GEMM_CHAIN_CUH
#define MPRES_GEMM_CHAIN_CUH

#include "mp_device.cuh"

namespace mpres {
namespace {
using namespace dev;

/* an SoA mp_array_t's fields (src/types.cuh:85-92) */
struct MatSoA {
    const int *digits;
    const int *sign;
    const int *exp;
    const er_t *eval;
    const int *len;
};
inline MatSoA mat_soa(const mp_array_t &a) {
    return MatSoA{a.digits, a.sign, a.exp, reinterpret_cast<const er_t *>(a.eval), a.len};
}
using SoA = MatSoA;

/* C + buffer as mp_matrix_add_esi_kernel + mp_matrix_add_digits_kernel
 * (src/mpmatrix.cuh:47-166) + mp_matrix_round_kernel (:410-428). */
template <int N> __device__ __forceinline__ void split_add(mp_t<N> &res, const mp_t<N> &A, const mp_t<N> &B) {
    const Tables<N> &t = T<N>();
    int expA = A.exp, expB = B.exp, signA = A.sign, signB = B.sign;
    const int dexp = expA - expB;
    int gamma = dexp > 0 ? dexp : 0;
    int theta = dexp < 0 ? -dexp : 0;
    const int nzA = (!dnz(B.ev[1].frac) || (theta + B.ev[1].exp) < t.mp_j);
    const int nzB = (!dnz(A.ev[1].frac) || (gamma + A.ev[1].exp) < t.mp_j);
    gamma *= nzB;
    theta *= nzA;
    expA = (expA - gamma) * nzA;
    expB = (expB - theta) * nzB;
    signA *= nzA;
    signB *= nzB;
    const int fA = (1 - 2 * signA) * nzA;
    const int fB = (1 - 2 * signB) * nzB;
    er_t eA[2], eB[2];
    eA[0].exp = A.ev[0].exp + gamma; eA[1].exp = A.ev[1].exp + gamma;
    eB[0].exp = B.ev[0].exp + theta; eB[1].exp = B.ev[1].exp + theta;
    eA[0].frac = dscale_sign(A.ev[0].frac, fA); eA[1].frac = dscale_sign(A.ev[1].frac, fA);
    eB[0].frac = dscale_sign(B.ev[0].frac, fB); eB[1].frac = dscale_sign(B.ev[1].frac, fB);
    er_t lo = er_add<false>(signA ? eA[1] : eA[0], signB ? eB[1] : eB[0]);
    er_t up = er_add<true>(signA ? eA[0] : eA[1], signB ? eB[0] : eB[1]);
    res.exp = (expA == 0) ? expB : expA;
    const int minus = dneg(lo.frac) && dneg(up.frac);
    res.sign = minus;
    if (minus) {
        res.ev[0].frac = dflip(up.frac); res.ev[0].exp = up.exp;
        res.ev[1].frac = dflip(lo.frac); res.ev[1].exp = lo.exp;
    } else {
        res.ev[0] = lo;
        res.ev[1] = up;
    }
    const int *pg = t.pow2 + (size_t)pow2_row_index<N>(gamma) * N;
    const int *pt = t.pow2 + (size_t)pow2_row_index<N>(theta) * N;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const int lm = t.moduli[i];
        /* cuda::mod_axby with the double quotient (src/modular.cuh:163-168) */
        const long long r = (long long)(fA * A.d[i]) * (long long)__ldg(pg + i) +
                            (long long)(fB * B.d[i]) * (long long)__ldg(pt + i);
        const double quotient = (double)r * (1.0 / lm);
        const int q = (int)quotient;
        int residue = (int)(r - (long long)q * (long long)lm);
        if (minus) residue = (int)(((long long)lm - (long long)residue) % (long long)lm);
        res.d[i] = residue < 0 ? residue + lm : residue;
    }
    round_if_needed<N>(res);
}

/* 2^e mod m for any integer e (2^-1 = (m+1)/2 for the odd m), square and multiply */
__device__ __forceinline__ uint32_t pow2mod(long long e, uint32_t m, uint32_t mu) {
    uint32_t base = e >= 0 ? 2u : (m + 1u) / 2u;
    unsigned long long k = e >= 0 ? (unsigned long long)e : 0ull - (unsigned long long)e;
    uint32_t r = 1u;
    while (k) {
        if (k & 1u) r = mulmod(r, base, m, mu);
        base = mulmod(base, base, m, mu);
        k >>= 1;
    }
    return r;
}

/* v mod m for any 64-bit v: two folds by c32 = 2^32 mod m (v < 2^61 after
 * them), then the Barrett step of mulmod */
__device__ __forceinline__ uint32_t reduce64(uint64_t v, uint32_t m, uint32_t mu, uint32_t c32) {
    v = (v >> 32) * c32 + (v & 0xffffffffull);
    v = (v >> 32) * c32 + (v & 0xffffffffull);
    uint32_t q = __umulhi((uint32_t)(v >> 30), mu);
    uint32_t r = (uint32_t)v - q * m;
    r = min(r, r - m);
    r = min(r, r - m);
    return r;
}

/* W = (-1)^s * d * 2^e mod m_i of one element, for every modulus.  2^e is the
 * RNS_POW2 row e for 0 <= e <= log2m, the row e + log2m times 2^-log2m for
 * -log2m <= e < 0 (the usual case: a converted double's exponent), else by
 * square and multiply; the same residue every way. */
template <int N> __device__ __forceinline__ uint32_t encode_residue(int d, int s, long long e, int i) {
    const Tables<N> &t = T<N>();
    const uint32_t m = (uint32_t)t.moduli[i], mu = t.mu[i];
    const uint32_t v = s ? (d ? m - (uint32_t)d : 0u) : (uint32_t)d;
    uint32_t f;
    if (e >= 0 && e <= t.log2m)
        f = (uint32_t)__ldg(t.pow2 + (size_t)e * N + i);
    else if (e < 0 && e >= -t.log2m)
        f = mulmod((uint32_t)__ldg(t.pow2 + (size_t)(e + t.log2m) * N + i), t.pow2_neg_top[i], m, mu);
    else
        f = pow2mod(e, m, mu);
    return mulmod(v, f, m, mu);
}

/* W(A) and W(B): element e (column-major, e = c * rows + r) of a rows x cols
 * matrix with leading dimension ld, stored for the k chain -- A_LAYOUT:
 * int4 [c][N/4][rows] (the lanes of a warp, on consecutive rows, read 512
 * contiguous bytes); otherwise int4 [c][r][N/4] (a warp on one column of B
 * reads one 128-byte row). */
template <int N, bool A_LAYOUT>
__device__ __forceinline__ void prescale_element(const int *digits, const int *sign, const int *exp, int ld,
                                                 int rows, long long e, int4 *out) {
    constexpr int Q = N / 4;
    const int r = (int)(e % rows), c = (int)(e / rows);
    const long long src = (long long)ld * c + r;
    const int s = __ldg(sign + src), x = __ldg(exp + src);
    const int4 *dp = reinterpret_cast<const int4 *>(digits + (size_t)src * N);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int4 d = __ldg(dp + q);
        int4 w;
        w.x = (int)encode_residue<N>(d.x, s, x, 4 * q);
        w.y = (int)encode_residue<N>(d.y, s, x, 4 * q + 1);
        w.z = (int)encode_residue<N>(d.z, s, x, 4 * q + 2);
        w.w = (int)encode_residue<N>(d.w, s, x, 4 * q + 3);
        const size_t o = A_LAYOUT ? ((size_t)c * Q + q) * rows + r : ((size_t)c * rows + r) * Q + q;
        out[o] = w;
    }
}

/* sign, exponent and interval of a number, without residues */
struct Scal {
    int sign, exp;
    er_t ev[2];
};

/* the residues D = (-1)^s * W * 2^-e mod m_i of a number from its accumulators */
template <int N> __device__ __noinline__ void residues_from_acc(int *d, const uint64_t *w, int s, int e) {
    const Tables<N> &t = T<N>();
    for (int i = 0; i < N; i++) {
        const uint32_t m = (uint32_t)t.moduli[i], mu = t.mu[i];
        const uint32_t v = mulmod(reduce64(w[i], m, mu, t.pow2_32[i]), pow2mod(-(long long)e, m, mu), m, mu);
        d[i] = (int)(s ? (v ? m - v : 0u) : v);
    }
}

/* One step of the chain the general way: the full mp_mul and mp_add on the
 * residues recovered from the accumulators w, then the result re-encoded. */
template <int N>
__device__ __noinline__ void full_step(uint64_t *w, Scal *sum, SoA A, long long ia, int lenA, SoA B, long long ib,
                                       int lenB) {
    mp_t<N> x, a, b, p, r;
    x.sign = sum->sign;
    x.exp = sum->exp;
    x.ev[0] = sum->ev[0];
    x.ev[1] = sum->ev[1];
    residues_from_acc<N>(x.d, w, x.sign, x.exp);
    load_soa<N>(a, A.digits, A.sign, A.exp, A.eval, lenA, ia);
    load_soa<N>(b, B.digits, B.sign, B.exp, B.eval, lenB, ib);
    mp_mul<N>(p, a, b);
    mp_add<N>(r, x, p);
    for (int i = 0; i < N; i++) w[i] = encode_residue<N>(r.d[i], r.sign, r.exp, i);
    sum->sign = r.sign;
    sum->exp = r.exp;
    sum->ev[0] = r.ev[0];
    sum->ev[1] = r.ev[1];
}

/* ------------- the scalar half of a step with 32-bit exponents --------------
 *
 * The same values as er_md / er_add / add_scalars / needs_round with the
 * exponents held in 32-bit integers: identical values as long as nothing
 * overflows, which the callers guarantee by taking this form only when every
 * exponent entering the step is within +-2^27 (the operands' exponents within
 * +-2^26): then no intermediate exceeds 2^30 in magnitude.  Half the integer
 * instructions and registers of the 64-bit forms in the hot loop. */
struct er32 {
    double frac;
    int exp;
};
struct Scal32 {
    int sign, exp;
    er32 ev[2];
};
constexpr int kExp32 = 1 << 27;
__device__ __forceinline__ bool fits32(long long e, int lim) { return e >= -lim && e <= lim; }

__device__ __forceinline__ void er_adjust32(er32 &x) {
    const uint64_t u = dbits(x.frac);
    const bool nz = (u << 1) != 0;
    const int e = x.exp + (int)((u >> 52) & 2047) - 1023;
    x.exp = nz ? e : 0;
    x.frac = nz ? bdbl((u & kZeroExpMask) | kBiasExpMask) : bdbl(u & kSign);
}

template <bool UP> __device__ __forceinline__ er32 er_add32(const er32 &x, const er32 &y) {
    const bool xnz = dnz(x.frac), ynz = dnz(y.frac);
    const int xe = xnz ? x.exp : 0, ye = ynz ? y.exp : 0;
    const int dexp = (xnz && ynz) ? xe - ye : 0;
    const bool swap = dexp < 0;
    const double big = swap ? y.frac : x.frac, small = swap ? x.frac : y.frac;
    er32 r;
    r.exp = dexp != 0 ? (swap ? ye : xe) : (xe == 0 ? ye : xe);
    r.frac = dadd<UP>(big, scale2(small, swap ? dexp : -dexp));
    er_adjust32(r);
    return r;
}

/* er_md (mp_device.cuh) in the 32-bit exponent form, with the significands'
 * product from one directed FP64 multiplication (what __dmul_rd / __dmul_ru
 * compute, correctly rounded, so the same 53 bits and exponent as er_md's
 * integer product) and the division by the unit on the integer pipes as there.  The GEMM chains are bound by their integer pipe: one FP64 instruction
 * in place of the 106-bit product, its normalisation and rounding (the split
 * form's scalar chain, 1024^3: 19.1 -> 16.0 ms). */
template <bool UP>
__device__ __forceinline__ er32 er_md32_dp(const er32 &x, const er32 &y, const er_t &z, double zr, uint64_t zinv) {
    constexpr uint64_t kMant = (1ull << 52) - 1, kHidden = 1ull << 52;
    const uint64_t bx = dbits(x.frac), by = dbits(y.frac);
    const uint32_t ex = (uint32_t)(bx >> 52) & 2047u, ey = (uint32_t)(by >> 52) & 2047u;
    const uint64_t sgn = (bx ^ by) & kSign;
    er32 r;
    if (ex == 1023u && ey == 1023u) {
        const bool up = UP != (sgn != 0);
        /* x*y in [1, 4): the significand p and e = 52 + (exponent of the product) */
        const uint64_t bp = dbits(dmul<UP>(x.frac, y.frac));
        const uint64_t p = (bp & kMant) | kHidden;
        const int e = (int)((bp >> 52) & 2047u) - 1023 + 52;
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
        int E = e - 52 - ez - (k52 ? 52 : 53);
        if (q >> 53) {
            q >>= 1;
            E++;
        }
        r.exp = x.exp + y.exp - (int)z.exp + E + 52;
        r.frac = bdbl(sgn | kBiasExpMask | (q & kMant));
        return r;
    }
    if (((bx << 1) == 0 && ey != 2047u) || ((by << 1) == 0 && ex != 2047u)) {
        r.exp = 0;
        r.frac = bdbl(sgn);
        return r;
    }
    r.exp = x.exp + y.exp - (int)z.exp;
    r.frac = div_by_const<UP>(dmul<UP>(x.frac, y.frac), z.frac, zr);
    er_adjust32(r);
    return r;
}

template <int N> __device__ __forceinline__ bool needs_round32(const er32 &u) {
    const Tables<N> &t = T<N>();
    return dnz(u.frac) && u.exp >= t.mp_h; /* then u.exp - mp_h + 1 > 0 as well */
}

template <int N>
__device__ __forceinline__ bool add_scalars32(Scal32 &r, int &nzx_out, int &nzy_out, const Scal32 &x, const Scal32 &y) {
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
    er32 ax[2], ay[2];
    ax[0].exp = x.ev[0].exp + gamma; ax[1].exp = x.ev[1].exp + gamma;
    ay[0].exp = y.ev[0].exp + theta; ay[1].exp = y.ev[1].exp + theta;
    ax[0].frac = dscale_sign(x.ev[0].frac, fx); ax[1].frac = dscale_sign(x.ev[1].frac, fx);
    ay[0].frac = dscale_sign(y.ev[0].frac, fy); ay[1].frac = dscale_sign(y.ev[1].frac, fy);
    er32 ev[2];
    ev[0] = er_add32<false>(sx ? ax[1] : ax[0], sy ? ay[1] : ay[0]);
    ev[1] = er_add32<true>(sx ? ax[0] : ax[1], sy ? ay[0] : ay[1]);
    const int sign = dneg(ev[0].frac);
    const bool decided = sign == (int)dneg(ev[1].frac);
    r.sign = sign;
    r.exp = (ex == 0) ? ey : ex;
    if (sign) {
        r.ev[0].frac = dflip(ev[1].frac); r.ev[0].exp = ev[1].exp;
        r.ev[1].frac = dflip(ev[0].frac); r.ev[1].exp = ev[0].exp;
    } else {
        r.ev[0] = ev[0];
        r.ev[1] = ev[1];
    }
    nzx_out = nzx;
    nzy_out = nzy;
    return decided;
}

/* the 64-bit sum as a Scal32 when every exponent fits the 32-bit form */
__device__ __forceinline__ bool narrow32(const Scal &x, Scal32 &y) {
    y.sign = x.sign;
    y.exp = x.exp;
    y.ev[0].frac = x.ev[0].frac;
    y.ev[0].exp = (int)x.ev[0].exp;
    y.ev[1].frac = x.ev[1].frac;
    y.ev[1].exp = (int)x.ev[1].exp;
    return fits32(x.exp, kExp32) && fits32(x.ev[0].exp, kExp32) && fits32(x.ev[1].exp, kExp32);
}
__device__ __forceinline__ void widen32(const Scal32 &x, Scal &y) {
    y.sign = x.sign;
    y.exp = x.exp;
    y.ev[0].frac = x.ev[0].frac;
    y.ev[0].exp = x.ev[0].exp;
    y.ev[1].frac = x.ev[1].frac;
    y.ev[1].exp = x.ev[1].exp;
}


/* Products added between two folds of the accumulators: after a fold an
 * accumulator is below 2^32 * m < 2^62.3, each product below m^2 < 2^60.6
 * (every predefined modulus is below 2^30.3), so six more stay below 2^64. */
constexpr int kFoldEvery = 6;

/* One output C(row, col) of C = alpha*A*B + beta*C with the lazy-residue k
 * chain (per-thread loads of W(A), W(B) and of the A and B scalars), then the
 * epilogue: alpha*sum, beta*C and the split addition.  W(A) is int4
 * [k][N/4][m]; W(B) is int4 [n][k][N/4], or with B_KQN int4 [k][N/4][n] (n
 * given), the layout of the split chain's modular product. */
template <int N, bool B_KQN = false>
__device__ __forceinline__ void gemm_lazy_output(int m, int k, const MatSoA &alpha, const MatSoA &A, int lda,
                                                 const MatSoA &B, int ldb, const MatSoA &beta, int *cd, int *cs,
                                                 int *ce, er_t *cv, const int *clen, int ldc, const int4 *WA,
                                                 const int4 *WB, int row, int col, int n = 0) {
    constexpr int Q = N / 4;
    const Tables<N> &t = T<N>();
    const int lenA = __ldg(A.len), lenB = __ldg(B.len);
    const longlong2 *aev = reinterpret_cast<const longlong2 *>(A.eval);
    const longlong2 *bev = reinterpret_cast<const longlong2 *>(B.eval);
    const int4 *wa = WA + row;
    const int4 *wb = B_KQN ? WB + col : WB + (size_t)col * k * Q;
    const size_t wb_k = B_KQN ? (size_t)Q * n : (size_t)Q, wb_q = B_KQN ? (size_t)n : 1;
    uint64_t acc[N];
#pragma unroll
    for (int i = 0; i < N; i++) acc[i] = 0;
    Scal sum;
    sum.sign = 0;
    sum.exp = 0;
    sum.ev[0].frac = 0.0; sum.ev[0].exp = 0;
    sum.ev[1].frac = 0.0; sum.ev[1].exp = 0;
    /* The k chain, in runs of kFoldEvery steps with one fold of the
     * accumulators after each (a fold on a step counter inside the loop cost
     * the tiled kernel 3.5%).  The inner loop runs the steps that stay lazy and
     * leaves at the first that does not; that step runs out of line, then the
     * loop resumes.  Keeping the call outside the inner loop keeps the loop free
     * of the register saves around it (measured 4% of the time at 1024^3). */
    for (int i0 = 0; i0 < k; i0 += kFoldEvery) {
        const int i1 = min(i0 + kFoldEvery, k);
        int i = i0;
        for (;;) {
            /* the steps that stay lazy, with the sum's scalars in the 32-bit form
             * while every exponent is within its range */
            Scal32 s32;
            if (narrow32(sum, s32)) {
                for (; i < i1; i++) {
                    const long long ia = (long long)lda * i + row, ib = (long long)col * ldb + i;
                    int4 u[Q], v[Q];
#pragma unroll
                    for (int q = 0; q < Q; q++) {
                        u[q] = __ldg(wa + ((size_t)i * Q + q) * m);
                        v[q] = __ldg(wb + (size_t)i * wb_k + q * wb_q);
                    }
                    const int sa = __ldg(A.sign + ia), ea = __ldg(A.exp + ia);
                    const int sb = __ldg(B.sign + ib), eb = __ldg(B.exp + ib);
                    const longlong2 a0 = __ldg(aev + ia), a1 = __ldg(aev + lenA + ia);
                    const longlong2 b0 = __ldg(bev + ib), b1 = __ldg(bev + lenB + ib);
                    if (!(fits32(ea, kExp32 / 2) && fits32(eb, kExp32 / 2) && fits32(a0.y, kExp32) &&
                          fits32(a1.y, kExp32) && fits32(b0.y, kExp32) && fits32(b1.y, kExp32) &&
                          fits32(s32.exp, kExp32) && fits32(s32.ev[0].exp, kExp32) && fits32(s32.ev[1].exp, kExp32)))
                        break;
                    const er32 ae0{__longlong_as_double(a0.x), (int)a0.y}, ae1{__longlong_as_double(a1.x), (int)a1.y};
                    const er32 be0{__longlong_as_double(b0.x), (int)b0.y}, be1{__longlong_as_double(b1.x), (int)b1.y};
                    /* mp_mul without residues */
                    Scal32 p;
                    p.sign = sa ^ sb;
                    p.exp = ea + eb;
                    p.ev[0] = er_md32_dp<false>(ae0, be0, t.unit_upp, t.unit_upp_recip, t.unit_upp_inv);
                    p.ev[1] = er_md32_dp<true>(ae1, be1, t.unit_low, t.unit_low_recip, t.unit_low_inv);
                    Scal32 r;
                    int nzx, nzy;
                    const bool decided = add_scalars32<N>(r, nzx, nzy, s32, p);
                    if (!decided || needs_round32<N>(p.ev[1]) || needs_round32<N>(r.ev[1])) break;
                    if (!nzx) {
#pragma unroll
                        for (int j = 0; j < N; j++) acc[j] = 0;
                    }
                    if (nzy) {
#pragma unroll
                        for (int q = 0; q < Q; q++) {
                            acc[4 * q] += (uint64_t)(uint32_t)u[q].x * (uint32_t)v[q].x;
                            acc[4 * q + 1] += (uint64_t)(uint32_t)u[q].y * (uint32_t)v[q].y;
                            acc[4 * q + 2] += (uint64_t)(uint32_t)u[q].z * (uint32_t)v[q].z;
                            acc[4 * q + 3] += (uint64_t)(uint32_t)u[q].w * (uint32_t)v[q].w;
                        }
                    }
                    s32 = r;
                }
                widen32(s32, sum);
            }
            if (i >= i1) break;
            {
                uint64_t w[N]; /* copies: see round_if_needed */
                Scal sc = sum;
#pragma unroll
                for (int j = 0; j < N; j++) w[j] = acc[j];
                full_step<N>(w, &sc, A, (long long)lda * i + row, lenA, B, (long long)col * ldb + i, lenB);
#pragma unroll
                for (int j = 0; j < N; j++) acc[j] = w[j];
                sum = sc;
            }
            i++;
        }
#pragma unroll
        for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
    }
    mp_t<N> s;
    {
        uint64_t w[N];
        int d[N];
#pragma unroll
        for (int j = 0; j < N; j++) w[j] = acc[j];
        residues_from_acc<N>(d, w, sum.sign, sum.exp);
#pragma unroll
        for (int j = 0; j < N; j++) s.d[j] = d[j];
    }
    s.sign = sum.sign;
    s.exp = sum.exp;
    s.ev[0] = sum.ev[0];
    s.ev[1] = sum.ev[1];
    const int lenC = __ldg(clen);
    const long long ic = (long long)col * ldc + row;
    mp_t<N> al, be, buf, c0, cb, res;
    load_soa<N>(al, alpha.digits, alpha.sign, alpha.exp, alpha.eval, __ldg(alpha.len), 0);
    load_soa<N>(be, beta.digits, beta.sign, beta.exp, beta.eval, __ldg(beta.len), 0);
    mp_mul<N>(buf, s, al);
    load_soa<N>(c0, cd, cs, ce, cv, lenC, ic);
    mp_mul<N>(cb, c0, be);
    split_add<N>(res, cb, buf);
    store_soa<N>(res, cd, cs, ce, cv, lenC, ic);
}

} // namespace
} // namespace mpres

#endif
