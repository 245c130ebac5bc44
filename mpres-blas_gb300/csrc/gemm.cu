/*
 * mp_gemm (no-transpose): C = alpha*A*B + beta*C, column-major SoA matrices.
 *
 * Reference: cuda::mp_gemm<b1x,b1y,g2x,g2y,b3> (src/blas/gemm.cuh:70-168):
 *   1. matrix_multiply_notrans_kernel (:39-60): buffer(r,c) = a strictly
 *      sequential chain over i of mp_mul(A(r,i), B(i,c)) then mp_add;
 *   2. buffer = alpha*buffer and C = beta*C (mp_mat2scal_mul_* and
 *      mp_matrix_round_kernel, src/mpmatrix.cuh:190-253, :410-428);
 *   3. C = C + buffer by the split kernels mp_matrix_add_esi_kernel and
 *      mp_matrix_add_digits_kernel (src/mpmatrix.cuh:47-166) -- which take the
 *      sign from the interval alone and reduce residues through a double
 *      quotient -- and a final rounding.
 * All three stages are fused here into one kernel per output tile with the same
 * arithmetic, so the buffer matrix never leaves registers.  The k chain keeps
 * the reference's order (no split-k), so results are bit-identical.
 *
 * Residues of the k chain, carried lazily.  The moduli are odd, so 2 is
 * invertible modulo each of them and every number X = (-1)^s * D * 2^e has the
 * residue vector W = (-1)^s * D * 2^e mod m_i, for negative e too.  mp_add
 * aligns its operands by multiplying the one with the larger exponent by
 * 2^(difference) and adds them with their signs; in terms of W that is
 * W(x + y) = nzx * W(x) + nzy * W(y), where nzx, nzy are mp_add's flags that
 * drop an operand too small to matter -- whatever the exponents, and whatever
 * sign the sum is given.  mp_mul gives W(a * b) = W(a) * W(b).  So as long as
 * no rounding intervenes (a rounding rescales the residues by a power of two
 * with a remainder), the chain's residues are the plain modular dot product
 * sum_i W(A(r,i)) * W(B(i,c)), while its sign, exponent and interval come from
 * the scalar half of mp_mul and mp_add, computed step by step exactly as
 * before.  gemm_prescale forms W(A) and W(B) once per call; the k chain adds
 * their 62-bit products into 64-bit accumulators and folds them every few
 * steps (2^32 mod m_i).  A step that rounds the product or the sum, whose
 * sum's sign the bounds leave open (sign_estimate needs the residues), or
 * whose exponents are large enough for the integer exponent arithmetic to wrap
 * runs the full mp_mul + mp_add on residues recovered from the accumulators,
 * D = (-1)^s * W * 2^-e, and re-encodes the result.  Results are the same
 * bits as the step-by-step chain; the residue work per step drops from two
 * modular products and the sign handling per modulus to one multiply-add.
 */
/* every SM holds many product chains here and the FP64 pipe is narrow: the
 * interval evaluation (out-of-line steps, epilogue, step-by-step chain) runs in
 * fixed point on the integer pipes (mp_device.cuh) */
#define MPRES_EVAL_FIXED_POINT 1
#include <cstdlib>

#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(gemm)

namespace mpres {
namespace {
using namespace dev;

struct SoA {
    const int *digits;
    const int *sign;
    const int *exp;
    const er_t *eval;
    const int *len;
};
SoA soa(const mp_array_t &a) { return SoA{a.digits, a.sign, a.exp, reinterpret_cast<const er_t *>(a.eval), a.len}; }

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

/* The step-by-step chain, for calls without room for the W(A), W(B) scratch.
 * Three 128-thread blocks per SM (at most 168 registers a thread): measured
 * faster than two (255 registers) despite the spills, 94.8 against 108.0 ms at
 * 1024^3; four (128 registers) spill too much. */
template <int N, int BX, int BY>
__global__ void __launch_bounds__(BX *BY, 3) gemm_nn(int m, int n, int k, SoA alpha, SoA A, int lda, SoA B, int ldb,
                                                  SoA beta, int *cd, int *cs, int *ce, er_t *cv, const int *clen,
                                                  int ldc) {
    __shared__ __align__(16) int pow2s[pow2_cache_words<N>()];
    const uint32_t cache = pow2_cache_setup<N>(pow2s);
    const int row = blockIdx.x * BX + threadIdx.x;
    const int col = blockIdx.y * BY + threadIdx.y;
    if (row >= m || col >= n) return;
    const int lenA = __ldg(A.len), lenB = __ldg(B.len);
    mp_t<N> sum;
    set_zero<N>(sum);
    for (int i = 0; i < k; i++) {
        mp_t<N> a, b, p, s;
        load_soa<N>(a, A.digits, A.sign, A.exp, A.eval, lenA, (long long)lda * i + row);
        load_soa<N>(b, B.digits, B.sign, B.exp, B.eval, lenB, (long long)col * ldb + i);
        mp_mul<N>(p, a, b);
        mp_add<N>(s, sum, p, cache);
        sum = s;
    }
    const int lenC = __ldg(clen);
    const long long ic = (long long)col * ldc + row;
    mp_t<N> al, be, buf, c0, cb, res;
    load_soa<N>(al, alpha.digits, alpha.sign, alpha.exp, alpha.eval, __ldg(alpha.len), 0);
    load_soa<N>(be, beta.digits, beta.sign, beta.exp, beta.eval, __ldg(beta.len), 0);
    mp_mul<N>(buf, sum, al);
    load_soa<N>(c0, cd, cs, ce, cv, lenC, ic);
    mp_mul<N>(cb, c0, be);
    split_add<N>(res, cb, buf);
    store_soa<N>(res, cd, cs, ce, cv, lenC, ic);
}


/* ----------------------- the lazy-residue k chain ------------------------ */

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

/* W = (-1)^s * d * 2^e mod m_i of one element, for every modulus */
template <int N> __device__ __forceinline__ uint32_t encode_residue(int d, int s, long long e, int i) {
    const Tables<N> &t = T<N>();
    const uint32_t m = (uint32_t)t.moduli[i];
    const uint32_t v = s ? (d ? m - (uint32_t)d : 0u) : (uint32_t)d;
    return mulmod(v, pow2mod(e, m, t.mu[i]), m, t.mu[i]);
}

/* W(A) and W(B): A(r, c) of a rows x cols column-major matrix with leading
 * dimension ld, stored for the k chain -- A_LAYOUT: int4 [c][N/4][rows] (the
 * lanes of a warp, on consecutive rows, read 512 contiguous bytes); otherwise
 * int4 [c][r][N/4] (a warp on one column of B reads one 128-byte row). */
template <int N, bool A_LAYOUT>
__global__ void __launch_bounds__(256) gemm_prescale(const int *digits, const int *sign, const int *exp, int ld,
                                                     int rows, int cols, int4 *out) {
    constexpr int Q = N / 4;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)rows * cols) return;
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

/* the test of round_if_needed */
template <int N> __device__ __forceinline__ bool needs_round(const er_t &u) {
    const Tables<N> &t = T<N>();
    return dnz(u.frac) && u.exp >= t.mp_h && (int)(u.exp - t.mp_h + 1) > 0;
}

/* The scalar half of mp_add (mp_device.cuh), the same expressions: the sum's
 * sign, exponent and interval, and the flags that keep or drop each operand.
 * Returns false when the signs of the bounds disagree: the sign then comes from
 * sign_estimate, which needs the residues. */
template <int N>
__device__ __forceinline__ bool add_scalars(Scal &r, int &nzx_out, int &nzy_out, const Scal &x, const Scal &y) {
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

__device__ __forceinline__ bool small_exp(int e, int lim) { return e >= -lim && e <= lim; }

/* Products added between two folds of the accumulators: after a fold an
 * accumulator is below 2^32 * m < 2^62.3, each product below m^2 < 2^60.6
 * (every predefined modulus is below 2^30.3), so six more stay below 2^64. */
constexpr int kFoldEvery = 6;

template <int N, int BX, int BY>
__global__ void __launch_bounds__(BX *BY, 3) gemm_nn_lazy(int m, int n, int k, SoA alpha, SoA A, int lda, SoA B,
                                                       int ldb, SoA beta, int *cd, int *cs, int *ce, er_t *cv,
                                                       const int *clen, int ldc, const int4 *WA, const int4 *WB) {
    constexpr int Q = N / 4;
    const Tables<N> &t = T<N>();
    const int row = blockIdx.x * BX + threadIdx.x;
    const int col = blockIdx.y * BY + threadIdx.y;
    if (row >= m || col >= n) return;
    const int lenA = __ldg(A.len), lenB = __ldg(B.len);
    const longlong2 *aev = reinterpret_cast<const longlong2 *>(A.eval);
    const longlong2 *bev = reinterpret_cast<const longlong2 *>(B.eval);
    const int4 *wa = WA + row;
    const int4 *wb = WB + (size_t)col * k * Q;
    uint64_t acc[N];
#pragma unroll
    for (int i = 0; i < N; i++) acc[i] = 0;
    Scal sum;
    sum.sign = 0;
    sum.exp = 0;
    sum.ev[0].frac = 0.0; sum.ev[0].exp = 0;
    sum.ev[1].frac = 0.0; sum.ev[1].exp = 0;
    int since_fold = 0;
    /* The k chain.  The inner loop runs the steps that stay lazy and leaves at
     * the first that does not; that step runs out of line, then the loop
     * resumes.  Keeping the call outside the inner loop keeps the loop free of
     * the register saves around it (measured 4% of the time at 1024^3). */
    int i = 0;
    for (;;) {
        for (; i < k; i++) {
            const long long ia = (long long)lda * i + row, ib = (long long)col * ldb + i;
            int4 u[Q], v[Q];
#pragma unroll
            for (int q = 0; q < Q; q++) {
                u[q] = __ldg(wa + ((size_t)i * Q + q) * m);
                v[q] = __ldg(wb + (size_t)i * Q + q);
            }
            const int sa = __ldg(A.sign + ia), ea = __ldg(A.exp + ia);
            const int sb = __ldg(B.sign + ib), eb = __ldg(B.exp + ib);
            const longlong2 a0 = __ldg(aev + ia), a1 = __ldg(aev + lenA + ia);
            const longlong2 b0 = __ldg(bev + ib), b1 = __ldg(bev + lenB + ib);
            const er_t ae0{__longlong_as_double(a0.x), a0.y}, ae1{__longlong_as_double(a1.x), a1.y};
            const er_t be0{__longlong_as_double(b0.x), b0.y}, be1{__longlong_as_double(b1.x), b1.y};
            /* mp_mul without residues */
            Scal p;
            p.sign = sa ^ sb;
            p.exp = ea + eb;
            p.ev[0] = er_md<false>(ae0, be0, t.unit_upp, t.unit_upp_recip, t.unit_upp_inv);
            p.ev[1] = er_md<true>(ae1, be1, t.unit_low, t.unit_low_recip, t.unit_low_inv);
            Scal r;
            int nzx, nzy;
            const bool decided = add_scalars<N>(r, nzx, nzy, sum, p);
            const bool lazy = decided && !needs_round<N>(p.ev[1]) && !needs_round<N>(r.ev[1]) &&
                              small_exp(ea, 1 << 28) && small_exp(eb, 1 << 28) && small_exp(sum.exp, 1 << 29);
            if (!lazy) break;
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
            sum = r;
            if (++since_fold == kFoldEvery) {
                since_fold = 0;
#pragma unroll
                for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
            }
        }
        if (i >= k) break;
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
        if (++since_fold == kFoldEvery) {
            since_fold = 0;
#pragma unroll
            for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
        }
        i++;
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

/* ------------------- the k chain with shared-memory k tiles ------------------
 *
 * The same lazy-residue chain as gemm_nn_lazy, with its operands staged: for
 * every KT consecutive k steps the block copies, with cp.async into a second
 * buffer while it works on the first,
 *   W(A) of its 32 rows (KT x N/4 x 32 int4), W(B) of its 4 columns
 *   (KT x 4 x N/4 int4), and the sign, exponent and interval of those A and B
 *   elements;
 * each thread then reads its residues one quad at a time (its row's quad and
 * the column's quad, a broadcast) right where they are accumulated.  W(A) is
 * read from L2 once per block instead of once per warp, and only one quad of
 * residues is live at a time: at most 128 registers, so four blocks fit on an
 * SM.  Blocks walk C in groups of kGroupRows row blocks, so the blocks resident
 * at once share their rows of W(A) and columns of W(B) in L2. */
constexpr int kKT = 4;          /* k steps per staged tile */
constexpr int kGroupRows = 8;   /* row blocks per group of the block order */

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, bool ok) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src, bool ok) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void lds128(uint32_t addr, uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d) {
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(a), "=r"(b), "=r"(c), "=r"(d) : "r"(addr));
}

/* one buffer of a k tile */
template <int N, int BX, int BY> struct GemmTile {
    int4 wa[kKT][N / 4][BX];
    int4 wb[kKT][BY][N / 4];
    longlong2 aev[kKT][2][BX]; /* lower, upper bound of A(row, k) */
    longlong2 bev[kKT][2][BY];
    int as[kKT][BX], ae[kKT][BX];
    int bs[kKT][BY], be[kKT][BY];
};

template <int N, int BX, int BY>
__device__ __forceinline__ void stage_tile(GemmTile<N, BX, BY> &tl, int k0, int m, int n, int k, int r0, int c0,
                                           SoA A, int lda, int lenA, SoA B, int ldb, int lenB, const int4 *WA,
                                           const int4 *WB) {
    constexpr int Q = N / 4, T = BX * BY;
    const int t = threadIdx.y * BX + threadIdx.x;
    const int4 *wa0 = WA, *wb0 = WB;
    for (int e = t; e < kKT * Q * BX; e += T) {
        const int r = e % BX, q = (e / BX) % Q, kk = e / (BX * Q);
        const bool ok = (k0 + kk < k) && (r0 + r < m);
        const int4 *src = ok ? WA + ((size_t)(k0 + kk) * Q + q) * m + r0 + r : wa0;
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.wa[kk][q][r]), src, ok);
    }
    for (int e = t; e < kKT * BY * Q; e += T) {
        const int q = e % Q, kk = (e / Q) % kKT, cy = e / (Q * kKT);
        const bool ok = (k0 + kk < k) && (c0 + cy < n);
        const int4 *src = ok ? WB + ((size_t)(c0 + cy) * k + k0 + kk) * Q + q : wb0;
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.wb[kk][cy][q]), src, ok);
    }
    const longlong2 *aev = reinterpret_cast<const longlong2 *>(A.eval);
    const longlong2 *bev = reinterpret_cast<const longlong2 *>(B.eval);
    for (int e = t; e < kKT * BX; e += T) {
        const int r = e % BX, kk = e / BX;
        const bool ok = (k0 + kk < k) && (r0 + r < m);
        const long long i = ok ? (long long)lda * (k0 + kk) + r0 + r : 0;
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.as[kk][r]), A.sign + i, ok);
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.ae[kk][r]), A.exp + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.aev[kk][0][r]), aev + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.aev[kk][1][r]), aev + lenA + i, ok);
    }
    for (int e = t; e < kKT * BY; e += T) {
        const int kk = e % kKT, cy = e / kKT;
        const bool ok = (k0 + kk < k) && (c0 + cy < n);
        const long long i = ok ? (long long)ldb * (c0 + cy) + k0 + kk : 0;
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.bs[kk][cy]), B.sign + i, ok);
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.be[kk][cy]), B.exp + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.bev[kk][0][cy]), bev + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.bev[kk][1][cy]), bev + lenB + i, ok);
    }
}

template <int N, int BX, int BY, int MINB>
__global__ void __launch_bounds__(BX *BY, MINB) gemm_nn_tiled(int m, int n, int k, SoA alpha, SoA A, int lda, SoA B,
                                                          int ldb, SoA beta, int *cd, int *cs, int *ce, er_t *cv,
                                                          const int *clen, int ldc, const int4 *WA, const int4 *WB) {
    constexpr int Q = N / 4;
    extern __shared__ __align__(16) unsigned char gemm_smem[];
    GemmTile<N, BX, BY> *tiles = reinterpret_cast<GemmTile<N, BX, BY> *>(gemm_smem);
    const Tables<N> &t = T<N>();
    /* block order: groups of kGroupRows row blocks, column blocks inside a group */
    const int gx = (m + BX - 1) / BX, gy = (n + BY - 1) / BY;
    const int per_group = kGroupRows * gy;
    const int grp = blockIdx.x / per_group, in = blockIdx.x % per_group;
    const int rows_in_group = min(kGroupRows, gx - grp * kGroupRows);
    const int bx = grp * kGroupRows + in % rows_in_group, by = in / rows_in_group;
    const int r0 = bx * BX, c0 = by * BY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int row = r0 + tx, col = c0 + ty;
    const bool live = row < m && col < n;
    const int lenA = __ldg(A.len), lenB = __ldg(B.len);
    uint64_t acc[N];
#pragma unroll
    for (int i = 0; i < N; i++) acc[i] = 0;
    Scal sum;
    sum.sign = 0;
    sum.exp = 0;
    sum.ev[0].frac = 0.0; sum.ev[0].exp = 0;
    sum.ev[1].frac = 0.0; sum.ev[1].exp = 0;
    int since_fold = 0;
    const int ntiles = (k + kKT - 1) / kKT;
    stage_tile<N, BX, BY>(tiles[0], 0, m, n, k, r0, c0, A, lda, lenA, B, ldb, lenB, WA, WB);
    cp_async_commit();
    for (int tile = 0; tile < ntiles; tile++) {
        const int buf = tile & 1;
        if (tile + 1 < ntiles)
            stage_tile<N, BX, BY>(tiles[buf ^ 1], (tile + 1) * kKT, m, n, k, r0, c0, A, lda, lenA, B, ldb, lenB, WA,
                                  WB);
        cp_async_commit();
        cp_async_wait_one();
        __syncthreads();
        const GemmTile<N, BX, BY> &tl = tiles[buf];
        const int k0 = tile * kKT;
        const int kend = min(kKT, k - k0);
        if (live) {
            const uint32_t wa_s = (uint32_t)__cvta_generic_to_shared(&tl.wa[0][0][tx]);
            const uint32_t wb_s = (uint32_t)__cvta_generic_to_shared(&tl.wb[0][ty][0]);
            /* the steps that stay lazy run in the inner loop, which leaves at the
             * first that does not; that step runs out of line (as in gemm_nn_lazy) */
            int kk = 0;
            for (;;) {
                for (; kk < kend; kk++) {
                    const longlong2 a0 = tl.aev[kk][0][tx], a1 = tl.aev[kk][1][tx];
                    const longlong2 b0 = tl.bev[kk][0][ty], b1 = tl.bev[kk][1][ty];
                    const int sa = tl.as[kk][tx], ea = tl.ae[kk][tx], sb = tl.bs[kk][ty], eb = tl.be[kk][ty];
                    const er_t ae0{__longlong_as_double(a0.x), a0.y}, ae1{__longlong_as_double(a1.x), a1.y};
                    const er_t be0{__longlong_as_double(b0.x), b0.y}, be1{__longlong_as_double(b1.x), b1.y};
                    /* mp_mul without residues */
                    Scal p;
                    p.sign = sa ^ sb;
                    p.exp = ea + eb;
                    p.ev[0] = er_md<false>(ae0, be0, t.unit_upp, t.unit_upp_recip, t.unit_upp_inv);
                    p.ev[1] = er_md<true>(ae1, be1, t.unit_low, t.unit_low_recip, t.unit_low_inv);
                    Scal r;
                    int nzx, nzy;
                    const bool decided = add_scalars<N>(r, nzx, nzy, sum, p);
                    const bool lazy = decided && !needs_round<N>(p.ev[1]) && !needs_round<N>(r.ev[1]) &&
                                      small_exp(ea, 1 << 28) && small_exp(eb, 1 << 28) && small_exp(sum.exp, 1 << 29);
                    if (!lazy) break;
                    if (!nzx) {
#pragma unroll
                        for (int j = 0; j < N; j++) acc[j] = 0;
                    }
                    if (nzy) {
                        const uint32_t ua = wa_s + (uint32_t)(kk * Q * BX * 16);
                        const uint32_t ub = wb_s + (uint32_t)(kk * BY * Q * 16);
#pragma unroll
                        for (int q = 0; q < Q; q++) {
                            uint32_t u0, u1, u2, u3, v0, v1, v2, v3;
                            lds128(ua + (uint32_t)(q * BX * 16), u0, u1, u2, u3);
                            lds128(ub + (uint32_t)(q * 16), v0, v1, v2, v3);
                            acc[4 * q] += (uint64_t)u0 * v0;
                            acc[4 * q + 1] += (uint64_t)u1 * v1;
                            acc[4 * q + 2] += (uint64_t)u2 * v2;
                            acc[4 * q + 3] += (uint64_t)u3 * v3;
                        }
                    }
                    sum = r;
                    if (++since_fold == kFoldEvery) {
                        since_fold = 0;
#pragma unroll
                        for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
                    }
                }
                if (kk >= kend) break;
                {
                    uint64_t w[N]; /* copies: see round_if_needed */
                    Scal sc = sum;
#pragma unroll
                    for (int j = 0; j < N; j++) w[j] = acc[j];
                    full_step<N>(w, &sc, A, (long long)lda * (k0 + kk) + row, lenA, B,
                                 (long long)col * ldb + k0 + kk, lenB);
#pragma unroll
                    for (int j = 0; j < N; j++) acc[j] = w[j];
                    sum = sc;
                }
                if (++since_fold == kFoldEvery) {
                    since_fold = 0;
#pragma unroll
                    for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
                }
                kk++;
            }
        }
        __syncthreads(); /* the buffer is restaged by the next iteration */
    }
    cp_async_wait_all();
    if (!live) return;
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
    mp_t<N> al, be, buf, c0v, cb, res;
    load_soa<N>(al, alpha.digits, alpha.sign, alpha.exp, alpha.eval, __ldg(alpha.len), 0);
    load_soa<N>(be, beta.digits, beta.sign, beta.exp, beta.eval, __ldg(beta.len), 0);
    mp_mul<N>(buf, s, al);
    load_soa<N>(c0v, cd, cs, ce, cv, lenC, ic);
    mp_mul<N>(cb, c0v, be);
    split_add<N>(res, cb, buf);
    store_soa<N>(res, cd, cs, ce, cv, lenC, ic);
}

template <int N>
cudaError_t run(int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda, const mp_array_t &B,
                int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc, Workspace ws, cudaStream_t s) {
    constexpr int BX = 32, BY = 4;
    dim3 block(BX, BY), grid((m + BX - 1) / BX, (n + BY - 1) / BY);
    er_t *cv = reinterpret_cast<er_t *>(C.eval);
    if (ws.ptr != nullptr && ws.bytes >= gemm_workspace_bytes(N, m, n, k)) {
        int4 *wa = static_cast<int4 *>(ws.ptr);
        int4 *wb = wa + (size_t)m * k * (N / 4);
        const long long na = (long long)m * k, nb = (long long)k * n;
        gemm_prescale<N, true><<<(unsigned)((na + 255) / 256), 256, 0, s>>>(A.digits, A.sign, A.exp, lda, m, k, wa);
        gemm_prescale<N, false><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(B.digits, B.sign, B.exp, ldb, k, n, wb);
        const char *v1 = std::getenv("MPRES_GEMM_V1");
        if (v1 && v1[0] == '1') {
            gemm_nn_lazy<N, BX, BY><<<grid, block, 0, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb, soa(beta),
                                                           C.digits, C.sign, C.exp, cv, C.len, ldc, wa, wb);
        } else {
            constexpr size_t smem = 2 * sizeof(GemmTile<N, BX, BY>);
            const char *mb = std::getenv("MPRES_GEMM_MINB");
            const bool three = mb && mb[0] == '3';
            static PerDevice<cudaError_t> attrs(cuda_ok);
            cudaError_t e = attrs.get(current_device(), cudaErrorInvalidDevice, [] {
                cudaError_t r = cudaFuncSetAttribute(gemm_nn_tiled<N, BX, BY, 4>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (r != cudaSuccess) return r;
                return cudaFuncSetAttribute(gemm_nn_tiled<N, BX, BY, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem);
            });
            if (e != cudaSuccess) return e;
            const unsigned blocks = grid.x * grid.y;
            if (three)
                gemm_nn_tiled<N, BX, BY, 3><<<blocks, block, smem, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb,
                                                                        soa(beta), C.digits, C.sign, C.exp, cv, C.len,
                                                                        ldc, wa, wb);
            else
                gemm_nn_tiled<N, BX, BY, 4><<<blocks, block, smem, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb,
                                                                        soa(beta), C.digits, C.sign, C.exp, cv, C.len,
                                                                        ldc, wa, wb);
        }
    } else {
        gemm_nn<N, BX, BY><<<grid, block, 0, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb, soa(beta), C.digits,
                                                  C.sign, C.exp, cv, C.len, ldc);
    }
    return cudaGetLastError();
}

} // namespace

size_t gemm_workspace_bytes(int nmod, int m, int n, int k) {
    return ((size_t)m * k + (size_t)k * n) * (size_t)nmod * 4;
}

cudaError_t launch_gemm(int nmod, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                        const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc,
                        Workspace ws, cudaStream_t s) {
    switch (nmod) {
    case 8: return run<8>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, s);
    case 16: return run<16>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, s);
    case 32: return run<32>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
