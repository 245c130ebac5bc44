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
#include "kernels.h"
#include "mp_device.cuh"
#include "gemm_chain.cuh"

MPRES_DEFINE_TABLES(gemm)

namespace mpres {
namespace {
using namespace dev;

SoA soa(const mp_array_t &a) { return mat_soa(a); }


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

/* W(A) and W(B) of a whole matrix (prescale_element, gemm_chain.cuh) */
template <int N, bool A_LAYOUT>
__global__ void __launch_bounds__(256) gemm_prescale(const int *digits, const int *sign, const int *exp, int ld,
                                                     int rows, int cols, int4 *out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)rows * cols) return;
    prescale_element<N, A_LAYOUT>(digits, sign, exp, ld, rows, e, out);
}


/* ------------------- the k chain with shared-memory k tiles ------------------
 *
 * The lazy-residue chain of gemm_lazy_output (gemm_chain.cuh, which the batch
 * kernel runs per thread), with its operands staged: for
 * every KT consecutive k steps the block copies, with cp.async into a second
 * buffer while it works on the first,
 *   W(A) of its 32 rows (KT x N/4 x 32 int4), W(B) of its 4 columns
 *   (KT x 4 x N/4 int4), and the sign, exponent and interval of those A and B
 *   elements;
 * each thread then reads its residues one quad at a time (its row's quad and
 * the column's quad, a broadcast) right where they are accumulated.  W(A) is
 * read from L2 once per block instead of once per warp, and only one quad of
 * residues is live at a time.  Three blocks an SM (168 registers; mp_gemm
 * 1024^3 with 32 moduli: 37.8 ms, against 38.3 at four blocks and 128
 * registers, 44.3 at two; eight k steps a tile 51.3, two 38.5).  Blocks walk C
 * in groups of kGroupRows row blocks, so the blocks resident at once share
 * their rows of W(A) and columns of W(B) in L2 (16 rows a group: 38.5 ms). */
constexpr int kKT = 4;          /* k steps per staged tile */
static_assert(kKT <= kFoldEvery, "the accumulators are folded once per tile");
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

template <int N, int BX, int BY>
__global__ void __launch_bounds__(BX *BY, 3) gemm_nn_tiled(int m, int n, int k, SoA alpha, SoA A, int lda, SoA B,
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
             * first that does not; that step runs out of line (as in gemm_lazy_output).
             * The inner loop carries the sum's scalars in the 32-bit form. */
            int kk = 0;
            for (;;) {
                Scal32 s32;
                if (narrow32(sum, s32)) {
                    for (; kk < kend; kk++) {
                        const longlong2 a0 = tl.aev[kk][0][tx], a1 = tl.aev[kk][1][tx];
                        const longlong2 b0 = tl.bev[kk][0][ty], b1 = tl.bev[kk][1][ty];
                        const int sa = tl.as[kk][tx], ea = tl.ae[kk][tx], sb = tl.bs[kk][ty], eb = tl.be[kk][ty];
                        /* the 32-bit form holds: exponents small enough that no sum of them overflows */
                        if (!(fits32(ea, kExp32 / 2) && fits32(eb, kExp32 / 2) && fits32(a0.y, kExp32) &&
                              fits32(a1.y, kExp32) && fits32(b0.y, kExp32) && fits32(b1.y, kExp32) &&
                              fits32(s32.exp, kExp32) && fits32(s32.ev[0].exp, kExp32) &&
                              fits32(s32.ev[1].exp, kExp32)))
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
                        s32 = r;
                    }
                    widen32(s32, sum);
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
                kk++;
            }
            /* one fold per tile: at most kKT products since the last one (a full
             * step leaves reduced residues), fewer than kFoldEvery; folding on a
             * step count instead cost 1.3 ms of 37.8 at 1024^3 */
#pragma unroll
            for (int j = 0; j < N; j++) acc[j] = (acc[j] >> 32) * t.pow2_32[j] + (acc[j] & 0xffffffffull);
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

/* ------------------ the split k chain: scalars, then residues -----------------
 *
 * The lazy chain of an output is a modular dot product of W(A) and W(B) for its
 * residues, weighted by the flags of the scalar half, beside a scalar chain
 * that never looks at the residues as long as every step stays lazy.  When in
 * addition no step drops an operand (nzx = nzy = 1 after the first step), the
 * residues are the unweighted sum_i W(A(r,i)) * W(B(i,c)) mod m_j: one modular
 * matrix product per modulus.  The split form runs the two halves as separate
 * kernels, each with the registers and schedule its own work wants:
 *   gemm_scalar_chain   the scalar chain of every output (sign, exponent,
 *                       interval), no residues: no 64-bit accumulators live in
 *                       the loop, so more warps share an SM;
 *   gemm_limbs, gemm_mma_product  W(A) x W(B) per modulus on the tensor
 *                       cores: each residue as four 8-bit limbs in bf16, the
 *                       limb products summed exactly in fp32 and weighted by
 *                       2^(8s) mod m_j in 64-bit integers;
 *   gemm_split_epilogue the residues of each sum recovered as
 *                       (-1)^s * W * 2^-e, then alpha*sum, beta*C and the split
 *                       addition as in the other kernels;
 *   gemm_redo           outputs whose chain left that form (a step that
 *                       rounds, an undecided sign, a dropped operand,
 *                       exponents outside the 32-bit range) run the
 *                       per-output lazy chain from the start instead.
 * Every value is the one the single chain computes, so results are the same
 * bits.  The scratch: W(A), W(B), their limb planes (twice the size of W), the
 * product (the size of C's residues) and 48 bytes an output. */
constexpr int kKT1 = 8;   /* k steps per staged tile of the scalar chain */
constexpr int kRedo = 2;  /* sign marker: the output runs the per-output chain */

template <int BX, int BY> struct ScalTile {
    longlong2 aev[kKT1][2][BX];
    longlong2 bev[kKT1][2][BY];
    int as[kKT1][BX], ae[kKT1][BX];
    int bs[kKT1][BY], be[kKT1][BY];
};

template <int BX, int BY>
__device__ __forceinline__ void stage_scalars(ScalTile<BX, BY> &tl, int k0, int m, int n, int k, int r0, int c0,
                                              SoA A, int lda, int lenA, SoA B, int ldb, int lenB) {
    constexpr int T = BX * BY;
    const int t = threadIdx.y * BX + threadIdx.x;
    const longlong2 *aev = reinterpret_cast<const longlong2 *>(A.eval);
    const longlong2 *bev = reinterpret_cast<const longlong2 *>(B.eval);
    for (int e = t; e < kKT1 * BX; e += T) {
        const int r = e % BX, kk = e / BX;
        const bool ok = (k0 + kk < k) && (r0 + r < m);
        const long long i = ok ? (long long)lda * (k0 + kk) + r0 + r : 0;
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.as[kk][r]), A.sign + i, ok);
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.ae[kk][r]), A.exp + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.aev[kk][0][r]), aev + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.aev[kk][1][r]), aev + lenA + i, ok);
    }
    for (int e = t; e < kKT1 * BY; e += T) {
        const int kk = e % kKT1, cy = e / kKT1;
        const bool ok = (k0 + kk < k) && (c0 + cy < n);
        const long long i = ok ? (long long)ldb * (c0 + cy) + k0 + kk : 0;
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.bs[kk][cy]), B.sign + i, ok);
        cp_async4((uint32_t)__cvta_generic_to_shared(&tl.be[kk][cy]), B.exp + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.bev[kk][0][cy]), bev + i, ok);
        cp_async16((uint32_t)__cvta_generic_to_shared(&tl.bev[kk][1][cy]), bev + lenB + i, ok);
    }
}

/* what the scalar chain leaves for each output e = col * m + row */
struct ChainOut {
    int *sign;   /* the sum's sign, or kRedo */
    int *exp;
    er_t *ev;    /* lower bounds of all outputs, then the upper bounds */
    int2 *redo;  /* (row, col) of the outputs marked kRedo, in no fixed order */
    int *nredo;
};

template <int N, int BX, int BY>
__global__ void __launch_bounds__(BX *BY, 8) gemm_scalar_chain(int m, int n, int k, SoA A, int lda, SoA B, int ldb,
                                                              ChainOut out) {
    extern __shared__ __align__(16) unsigned char chain_smem[];
    ScalTile<BX, BY> *tiles = reinterpret_cast<ScalTile<BX, BY> *>(chain_smem);
    const Tables<N> &t = T<N>();
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
    bool lazy = live;
    Scal32 s;
    s.sign = 0;
    s.exp = 0;
    s.ev[0].frac = 0.0; s.ev[0].exp = 0;
    s.ev[1].frac = 0.0; s.ev[1].exp = 0;
    const int ntiles = (k + kKT1 - 1) / kKT1;
    stage_scalars<BX, BY>(tiles[0], 0, m, n, k, r0, c0, A, lda, lenA, B, ldb, lenB);
    cp_async_commit();
    for (int tile = 0; tile < ntiles; tile++) {
        const int buf = tile & 1;
        if (tile + 1 < ntiles)
            stage_scalars<BX, BY>(tiles[buf ^ 1], (tile + 1) * kKT1, m, n, k, r0, c0, A, lda, lenA, B, ldb, lenB);
        cp_async_commit();
        cp_async_wait_one();
        __syncthreads();
        const ScalTile<BX, BY> &tl = tiles[buf];
        const int k0 = tile * kKT1;
        const int kend = min(kKT1, k - k0);
        /* The operands' exponents, checked once per tile by the whole block (the
         * staged slots past m, n or k hold zeros): if one is outside the 32-bit
         * form's range, every output of the block runs the per-output chain.
         * Inside the range the sum's exponent needs no check of its own: a sum
         * takes the exponent of one of its operands or their minimum, and the
         * products' exponents ea + eb are within +-2^27. */
        bool out_of_range = false;
        for (int e = threadIdx.y * BX + tx; e < kKT1 * BX; e += BX * BY)
            out_of_range |= !(fits32(tl.ae[e / BX][e % BX], kExp32 / 2) &&
                              fits32(tl.aev[e / BX][0][e % BX].y, kExp32) &&
                              fits32(tl.aev[e / BX][1][e % BX].y, kExp32));
        for (int e = threadIdx.y * BX + tx; e < kKT1 * BY; e += BX * BY)
            out_of_range |= !(fits32(tl.be[e / BY][e % BY], kExp32 / 2) &&
                              fits32(tl.bev[e / BY][0][e % BY].y, kExp32) &&
                              fits32(tl.bev[e / BY][1][e % BY].y, kExp32));
        if (__syncthreads_or(out_of_range)) lazy = false;
        if (lazy) {
            for (int kk = 0; kk < kend; kk++) {
                const longlong2 a0 = tl.aev[kk][0][tx], a1 = tl.aev[kk][1][tx];
                const longlong2 b0 = tl.bev[kk][0][ty], b1 = tl.bev[kk][1][ty];
                const int sa = tl.as[kk][tx], ea = tl.ae[kk][tx], sb = tl.bs[kk][ty], eb = tl.be[kk][ty];
                if (!(fits32(s.ev[0].exp, kExp32) && fits32(s.ev[1].exp, kExp32))) {
                    lazy = false;
                    break;
                }
                const er32 ae0{__longlong_as_double(a0.x), (int)a0.y}, ae1{__longlong_as_double(a1.x), (int)a1.y};
                const er32 be0{__longlong_as_double(b0.x), (int)b0.y}, be1{__longlong_as_double(b1.x), (int)b1.y};
                Scal32 p;
                p.sign = sa ^ sb;
                p.exp = ea + eb;
                p.ev[0] = er_md32_dp<false>(ae0, be0, t.unit_upp, t.unit_upp_recip, t.unit_upp_inv);
                p.ev[1] = er_md32_dp<true>(ae1, be1, t.unit_low, t.unit_low_recip, t.unit_low_inv);
                Scal32 r;
                int nzx, nzy;
                const bool decided = add_scalars32<N>(r, nzx, nzy, s, p);
                /* the first step adds to zero: dropping that zero changes no residue */
                if (!decided || needs_round32<N>(p.ev[1]) || needs_round32<N>(r.ev[1]) || !nzy ||
                    (!nzx && k0 + kk > 0)) {
                    lazy = false;
                    break;
                }
                s = r;
            }
        }
        __syncthreads(); /* the buffer is restaged by the next iteration */
    }
    cp_async_wait_all();
    /* every thread of the warp (BX = 32 lanes of one row block) arrives here */
    const unsigned redo = __ballot_sync(0xffffffffu, live && !lazy);
    if (live) {
        const size_t e = (size_t)col * m + row, mn = (size_t)m * n;
        if (lazy) {
            out.sign[e] = s.sign;
            out.exp[e] = s.exp;
            out.ev[e] = er_t{s.ev[0].frac, s.ev[0].exp};
            out.ev[mn + e] = er_t{s.ev[1].frac, s.ev[1].exp};
        } else {
            out.sign[e] = kRedo;
        }
    }
    if (redo) {
        const int lane = tx & 31;
        int base = 0;
        if (lane == __ffs(redo) - 1) base = atomicAdd(out.nredo, __popc(redo));
        base = __shfl_sync(0xffffffffu, base, __ffs(redo) - 1);
        if (live && !lazy) out.redo[base + __popc(redo & ((1u << lane) - 1u))] = make_int2(row, col);
    }
}

/* W(B) of a k x n matrix as int4 [k][N/4][n]: consecutive threads take
 * consecutive columns, so the stores of a warp are contiguous */
template <int N>
__global__ void __launch_bounds__(256) gemm_prescale_kq(const int *digits, const int *sign, const int *exp, int ld,
                                                        int k, int n, int4 *out) {
    constexpr int Q = N / 4;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)k * n) return;
    const int r = (int)(e / n), c = (int)(e % n);
    const long long src = (long long)ld * c + r;
    const int sg = __ldg(sign + src), x = __ldg(exp + src);
    const int4 *dp = reinterpret_cast<const int4 *>(digits + (size_t)src * N);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int4 d = __ldg(dp + q);
        int4 w;
        w.x = (int)encode_residue<N>(d.x, sg, x, 4 * q);
        w.y = (int)encode_residue<N>(d.y, sg, x, 4 * q + 1);
        w.z = (int)encode_residue<N>(d.z, sg, x, 4 * q + 2);
        w.w = (int)encode_residue<N>(d.w, sg, x, 4 * q + 3);
        out[((size_t)r * Q + q) * n + c] = w;
    }
}

/* ---------------- the modular product on the tensor cores -------------------
 *
 * S_j = W_j(A) x W_j(B) mod m_j for every modulus j.  A residue w < m_j < 2^30.3
 * is the sum of four limbs w = l0 + l1 2^8 + l2 2^16 + l3 2^24 (l0..l2 <= 255,
 * l3 <= 78), each exact in bf16, so S_j = sum_s 2^(8s) G_s with
 * G_s = sum_{a+b=s} L_a(A) x L_b(B), seven limb-sum groups of sixteen bf16 products.
 * The tensor cores sum a group over one stage of kKC = 32 k steps in fp32,
 * started at 2^23: every partial sum is an integer below 2^24 (the largest group,
 * s = 2, is at most 3 x 32 x 255^2 < 6.3e6 < 2^23), so the additions are exact and
 * the group's value is the significand of the result (integer sums that large
 * measured exact on this GPU with the same mma.sync form).  Each group's value
 * then enters a 64-bit accumulator times 2^(8s) mod m_j: below 2^23 * 2^30.3 per
 * term, seven terms a stage, folded (2^32 mod m_j) every kFoldStages stages.  Same
 * residues as the integer product, bit for bit. */
constexpr int kTB = 64;         /* outputs per block side */
constexpr int kKC = 32;         /* k steps per stage and per fp32 group sum */
constexpr int kFoldStages = 128; /* 896 terms below 2^53.3 on a folded value below 2^62.3 stay below 2^64 */

/* W (int4 [k][8][rows], 32 moduli) as limb planes bf16 [32][4][kp][rows_p], rows_p
 * and kp the padded sizes (multiples of kTB and kKC), zeros in the padding */
__global__ void __launch_bounds__(256) gemm_limbs(const int4 *W, int rows, int k, int rows_p, int kp, uint16_t *L) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; /* e = kk * rows_p + r */
    if (e >= (long long)rows_p * kp) return;
    const int r = (int)(e % rows_p), kk = (int)(e / rows_p);
    const bool in = r < rows && kk < k;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int4 w = in ? __ldg(W + ((size_t)kk * 8 + q) * rows + r) : make_int4(0, 0, 0, 0);
        const uint32_t v[4] = {(uint32_t)w.x, (uint32_t)w.y, (uint32_t)w.z, (uint32_t)w.w};
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
            for (int a = 0; a < 4; a++) /* an integer below 256 as bf16: the top half of its float */
                L[(((size_t)(4 * q + x) * 4 + a) * kp + kk) * rows_p + r] =
                    (uint16_t)(__float_as_uint((float)((v[x] >> (8 * a)) & 255u)) >> 16);
    }
}

__device__ __forceinline__ void ldsm4t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
                 "{%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void cp_async16_cg(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

/* A block: a kTB x kTB tile of S_j, j = blockIdx.y; four warps of 32 x 32 (2 x 4
 * tiles of 16 x 8).  Per stage the four limb planes of A and of B (kKC rows of
 * kTB bf16, 128 bytes, 16-byte chunks XOR-swizzled by row so that ldmatrix reads
 * are free of bank conflicts) come in by cp.async, double buffered (64 KB); a
 * warp keeps the stage's A fragments (all limbs, both k16 steps) in registers
 * and loads B fragments per limb pair.  Output: int4 [n][8][m], modulus j in
 * component j % 4 of quad j / 4 (the blocks of one tile, j = blockIdx.x, run
 * side by side, so the four writers of an int4 meet in L2). */
__global__ void __launch_bounds__(128, 2) gemm_mma_product(int m, int n, int mp, int np, int kp, const uint16_t *LA,
                                                           const uint16_t *LB, uint32_t *S) {
    extern __shared__ __align__(128) unsigned char prod_smem[];
    const Tables<32> &t = T<32>();
    const int j = blockIdx.x, gx = mp / kTB;
    const int r0 = (blockIdx.y % gx) * kTB, c0 = (blockIdx.y / gx) * kTB;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int wm = (w & 1) * 32, wn = (w >> 1) * 32;
    const uint32_t md = (uint32_t)t.moduli[j], mu = t.mu[j], c32 = t.pow2_32[j];
    uint32_t wt[7]; /* 2^(8s) mod m_j */
    wt[0] = 1u;
#pragma unroll
    for (int s = 1; s < 7; s++) wt[s] = mulmod(wt[s - 1], 256u, md, mu);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(prod_smem);
    auto stage = [&](int st, int k0) {
        /* 2 operands x 4 limbs x kKC rows x 8 chunks of 16 bytes */
        for (int e = tid; e < 2 * 4 * kKC * 8; e += 128) {
            const int op = e >> 10, a = (e >> 8) & 3, kk = (e >> 3) & 31, c = e & 7;
            const uint16_t *src = op == 0 ? LA + (((size_t)(j * 4 + a) * kp + k0 + kk) * mp + r0 + 8 * c)
                                          : LB + (((size_t)(j * 4 + a) * kp + k0 + kk) * np + c0 + 8 * c);
            cp_async16_cg(sbase + st * 32768 + op * 16384 + (a * kKC + kk) * 128 + ((c ^ (kk & 7)) << 4), src);
        }
    };
    static_assert(kKC == 32 && kTB == 64, "the staging index arithmetic assumes these sizes");
    uint64_t acc[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) acc[mt][nt][i] = 0;
    const int nst = kp / kKC;
    const int mi = lane >> 3, r8 = lane & 7;
    stage(0, 0);
    cp_async_commit();
    for (int st = 0; st < nst; st++) {
        if (st + 1 < nst) stage((st + 1) & 1, (st + 1) * kKC);
        cp_async_commit();
        cp_async_wait_one();
        __syncthreads();
        const uint32_t sA = sbase + (st & 1) * 32768, sB = sA + 16384;
        uint32_t af[2][4][2][4]; /* [k16 step][limb][m16 tile][register] */
#pragma unroll
        for (int ks = 0; ks < 2; ks++)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int mt = 0; mt < 2; mt++) {
                    const int kk = ks * 16 + (mi >> 1) * 8 + r8, mc = wm + 16 * mt + (mi & 1) * 8;
                    ldsm4t(sA + (a * kKC + kk) * 128 + (((mc >> 3) ^ (kk & 7)) << 4), af[ks][a][mt][0],
                           af[ks][a][mt][1], af[ks][a][mt][2], af[ks][a][mt][3]);
                }
#pragma unroll
        for (int s = 0; s < 7; s++) {
            float d[2][4][4];
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int i = 0; i < 4; i++) d[mt][nt][i] = 8388608.0f; /* 2^23 */
#pragma unroll
            for (int ks = 0; ks < 2; ks++)
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int b = s - a;
                    if (b < 0 || b > 3) continue;
                    uint32_t bf[4][2];
#pragma unroll
                    for (int np2 = 0; np2 < 2; np2++) {
                        const int kk = ks * 16 + (mi & 1) * 8 + r8, nc = wn + 16 * np2 + (mi >> 1) * 8;
                        ldsm4t(sB + (b * kKC + kk) * 128 + (((nc >> 3) ^ (kk & 7)) << 4), bf[2 * np2][0],
                               bf[2 * np2][1], bf[2 * np2 + 1][0], bf[2 * np2 + 1][1]);
                    }
#pragma unroll
                    for (int mt = 0; mt < 2; mt++)
#pragma unroll
                        for (int nt = 0; nt < 4; nt++) mma_bf16(d[mt][nt], af[ks][a][mt], bf[nt][0], bf[nt][1]);
                }
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        acc[mt][nt][i] += (uint64_t)(__float_as_uint(d[mt][nt][i]) & 0x7fffffu) * wt[s];
        }
        if ((st % kFoldStages) == kFoldStages - 1) {
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        acc[mt][nt][i] = (acc[mt][nt][i] >> 32) * c32 + (acc[mt][nt][i] & 0xffffffffull);
        }
        __syncthreads(); /* the buffer is restaged by the next iteration */
    }
    cp_async_wait_all();
    /* the m16n8 accumulator layout: register i of lane (g, tq) is row g + 8 (i / 2), column 2 tq + i % 2 */
    const int g = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = r0 + wm + 16 * mt + g + 8 * (i >> 1), c = c0 + wn + 8 * nt + 2 * tq + (i & 1);
                if (r < m && c < n) S[(((size_t)c * 8 + (j >> 2)) * m + r) * 4 + (j & 3)] = reduce64(acc[mt][nt][i], md, mu, c32);
            }
}

/* the outputs whose chain stayed in the split form: residues of the sum from
 * the modular product, then the epilogue of the other kernels */
template <int N>
__global__ void __launch_bounds__(128) gemm_split_epilogue(int m, int n, SoA alpha, SoA beta, int *cd, int *cs,
                                                           int *ce, er_t *cv, const int *clen, int ldc,
                                                           const uint32_t *S, ChainOut in) {
    const Tables<N> &t = T<N>();
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long mn = (long long)m * n;
    if (e >= mn) return;
    const int sg = in.sign[e];
    if (sg == kRedo) return;
    const int row = (int)(e % m), col = (int)(e / m);
    mp_t<N> s;
    s.sign = sg;
    s.exp = in.exp[e];
    s.ev[0] = in.ev[e];
    s.ev[1] = in.ev[mn + e];
    const uint4 *ws = reinterpret_cast<const uint4 *>(S) + (size_t)col * 8 * m + row; /* quad q at ws[q * m] */
    /* D = W * 2^-e: 2^-e from the RNS_POW2 row -e when 0 <= -e <= log2m (a sum's
     * exponent is its smallest product's, so usually), else by squaring */
    const long long ne = -(long long)s.exp;
    const bool row_ok = ne >= 0 && ne <= t.log2m;
    const int *p2 = t.pow2 + (size_t)(row_ok ? ne : 0) * N;
#pragma unroll
    for (int q = 0; q < N / 4; q++) {
        const uint4 v = __ldg(ws + (size_t)q * m);
        const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int x = 0; x < 4; x++) {
            const int i = 4 * q + x;
            const uint32_t md = (uint32_t)t.moduli[i], mu = t.mu[i];
            const uint32_t f = row_ok ? (uint32_t)__ldg(p2 + i) : pow2mod(ne, md, mu);
            const uint32_t d = mulmod(vv[x], f, md, mu);
            s.d[i] = (int)(sg ? (d ? md - d : 0u) : d);
        }
    }
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

/* the outputs marked kRedo: the per-output lazy chain and its epilogue */
template <int N>
__global__ void __launch_bounds__(128, 3) gemm_redo(int m, int n, int k, SoA alpha, SoA A, int lda, SoA B, int ldb,
                                                    SoA beta, int *cd, int *cs, int *ce, er_t *cv, const int *clen,
                                                    int ldc, const int4 *WA, const int4 *WB, ChainOut in) {
    const int count = *in.nredo;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int2 rc = in.redo[i];
        gemm_lazy_output<N, true>(m, k, alpha, A, lda, B, ldb, beta, cd, cs, ce, cv, clen, ldc, WA, WB, rc.x, rc.y,
                                  n);
    }
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

/* the split form's scratch, carved in this order */
struct SplitScratch {
    int4 *wa, *wb;
    uint16_t *la, *lb; /* limb planes of W(A), W(B) */
    uint32_t *prod;    /* the modular product, int4 [n][N/4][m] */
    ChainOut out;
};
long long round_up(long long v, long long to) { return (v + to - 1) / to * to; }
size_t split_scratch(int nmod, int m, int n, int k, void *base, SplitScratch *sp) {
    const size_t mn = (size_t)m * n;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align256(off + bytes);
        return at;
    };
    const size_t wa = take((size_t)m * k * nmod * 4);
    const size_t wb = take((size_t)k * n * nmod * 4);
    const size_t mp = round_up(m, kTB), np = round_up(n, kTB), kp = round_up(k, kKC);
    const size_t la = take((size_t)nmod * 4 * kp * mp * 2);
    const size_t lb = take((size_t)nmod * 4 * kp * np * 2);
    const size_t ws = take(mn * nmod * 4);
    const size_t sg = take(mn * 4);
    const size_t ex = take(mn * 4);
    const size_t ev = take(mn * 2 * sizeof(er_t));
    const size_t rd = take(mn * sizeof(int2));
    const size_t nr = take(sizeof(int));
    if (sp) {
        char *p = static_cast<char *>(base);
        sp->wa = reinterpret_cast<int4 *>(p + wa);
        sp->wb = reinterpret_cast<int4 *>(p + wb);
        sp->la = reinterpret_cast<uint16_t *>(p + la);
        sp->lb = reinterpret_cast<uint16_t *>(p + lb);
        sp->prod = reinterpret_cast<uint32_t *>(p + ws);
        sp->out = ChainOut{reinterpret_cast<int *>(p + sg), reinterpret_cast<int *>(p + ex),
                           reinterpret_cast<er_t *>(p + ev), reinterpret_cast<int2 *>(p + rd),
                           reinterpret_cast<int *>(p + nr)};
    }
    return off;
}

/* shapes whose launch grids and indices the split form's kernels cover (the
 * others take the tiled lazy chain) */
bool split_shape_ok(int m, int n, int k) {
    const long long gx = (m + 31) / 32, gy = (n + 3) / 4;
    const long long tiles = (round_up(m, kTB) / kTB) * (round_up(n, kTB) / kTB);
    const long long la = round_up(m, kTB) * round_up(k, kKC), lb = round_up(n, kTB) * round_up(k, kKC);
    return gx * gy <= (1ll << 28) && tiles <= 65535 && la / 256 < (1ll << 31) && lb / 256 < (1ll << 31) &&
           (long long)m * n < (1ll << 31);
}

/* marks: null, or kGemmSplitPhases + 1 events recorded on s before the first
 * launch and after each phase (the phases' times for the probe) */
template <int N>
cudaError_t run_split(int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                      const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc,
                      Workspace ws, cudaStream_t s, cudaEvent_t *marks = nullptr) {
    constexpr int BX = 32, BY = 4;
    SplitScratch sp;
    split_scratch(N, m, n, k, ws.ptr, &sp);
    const long long na = (long long)m * k, nb = (long long)k * n, mn = (long long)m * n;
    const long long gx = (m + BX - 1) / BX, gy = (n + BY - 1) / BY;
    const int mp = (int)round_up(m, kTB), np = (int)round_up(n, kTB), kp = (int)round_up(k, kKC);
    const long long tiles = (long long)(mp / kTB) * (np / kTB);
    const long long la = (long long)mp * kp, lb = (long long)np * kp;
    if (!split_shape_ok(m, n, k)) return cudaErrorInvalidConfiguration;
    constexpr size_t smem = 2 * sizeof(ScalTile<BX, BY>);
    constexpr int prod_smem = 2 * 2 * 4 * kKC * kTB * 2; /* two stages of A and B limb planes: 64 KB */
    static PerDevice<cudaError_t> attrs(cuda_ok);
    const int dev = current_device();
    cudaError_t e = attrs.get(dev, cudaErrorInvalidDevice, [] {
        cudaError_t r = cudaFuncSetAttribute(gemm_scalar_chain<N, BX, BY>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(gemm_mma_product, cudaFuncAttributeMaxDynamicSharedMemorySize, prod_smem);
        return r;
    });
    if (e != cudaSuccess) return e;
    static PerDevice<int> redo_grid([](const int &g) { return g > 0; });
    const int rgrid = redo_grid.get(dev, 0, [dev] {
        int sms = 0, per = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gemm_redo<N>, 128, 0) != cudaSuccess)
            return 0;
        return sms * (per > 0 ? per : 1);
    });
    if (rgrid <= 0) return cudaErrorInvalidDevice;
    if ((e = cudaMemsetAsync(sp.out.nredo, 0, sizeof(int), s)) != cudaSuccess) return e;
    auto mark = [&](int i) { if (marks) cudaEventRecord(marks[i], s); };
    mark(0);
    gemm_prescale<N, true><<<(unsigned)((na + 255) / 256), 256, 0, s>>>(A.digits, A.sign, A.exp, lda, m, k, sp.wa);
    mark(1);
    gemm_prescale_kq<N><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(B.digits, B.sign, B.exp, ldb, k, n, sp.wb);
    mark(2);
    gemm_limbs<<<(unsigned)((la + 255) / 256), 256, 0, s>>>(sp.wa, m, k, mp, kp, sp.la);
    gemm_limbs<<<(unsigned)((lb + 255) / 256), 256, 0, s>>>(sp.wb, n, k, np, kp, sp.lb);
    mark(3);
    gemm_scalar_chain<N, BX, BY><<<(unsigned)(gx * gy), dim3(BX, BY), smem, s>>>(m, n, k, soa(A), lda, soa(B), ldb,
                                                                              sp.out);
    mark(4);
    gemm_mma_product<<<dim3(N, (unsigned)tiles), 128, prod_smem, s>>>(m, n, mp, np, kp, sp.la, sp.lb, sp.prod);
    mark(5);
    er_t *cv = reinterpret_cast<er_t *>(C.eval);
    gemm_split_epilogue<N><<<(unsigned)((mn + 127) / 128), 128, 0, s>>>(m, n, soa(alpha), soa(beta), C.digits, C.sign,
                                                                         C.exp, cv, C.len, ldc, sp.prod, sp.out);
    mark(6);
    const long long want = (mn + 127) / 128;
    gemm_redo<N><<<(unsigned)(want < rgrid ? want : rgrid), 128, 0, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B),
                                                                         ldb, soa(beta), C.digits, C.sign, C.exp, cv,
                                                                         C.len, ldc, sp.wa, sp.wb, sp.out);
    mark(7);
    return cudaGetLastError();
}

template <int N>
cudaError_t run(int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda, const mp_array_t &B,
                int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc, Workspace ws, cudaStream_t s) {
    constexpr int BX = 32, BY = 4;
    dim3 block(BX, BY), grid((m + BX - 1) / BX, (n + BY - 1) / BY);
    er_t *cv = reinterpret_cast<er_t *>(C.eval);
    if constexpr (N == 32) {
        if (ws.ptr != nullptr && ws.bytes >= gemm_split_workspace_bytes(N, m, n, k) && split_shape_ok(m, n, k))
            return run_split<N>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, s);
    }
    if (ws.ptr != nullptr && ws.bytes >= gemm_workspace_bytes(N, m, n, k)) {
        int4 *wa = static_cast<int4 *>(ws.ptr);
        int4 *wb = wa + (size_t)m * k * (N / 4);
        const long long na = (long long)m * k, nb = (long long)k * n;
        gemm_prescale<N, true><<<(unsigned)((na + 255) / 256), 256, 0, s>>>(A.digits, A.sign, A.exp, lda, m, k, wa);
        gemm_prescale<N, false><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(B.digits, B.sign, B.exp, ldb, k, n, wb);
        /* one-dimensional grid in groups of row blocks; the block index
         * arithmetic stays within int */
        if ((long long)grid.x * grid.y > (1ll << 28)) return cudaErrorInvalidConfiguration;
        constexpr size_t smem = 2 * sizeof(GemmTile<N, BX, BY>);
        static PerDevice<cudaError_t> attrs(cuda_ok);
        cudaError_t e = attrs.get(current_device(), cudaErrorInvalidDevice, [] {
            return cudaFuncSetAttribute(gemm_nn_tiled<N, BX, BY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem);
        });
        if (e != cudaSuccess) return e;
        gemm_nn_tiled<N, BX, BY><<<grid.x * grid.y, block, smem, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb,
                                                                     soa(beta), C.digits, C.sign, C.exp, cv, C.len,
                                                                     ldc, wa, wb);
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

size_t gemm_split_workspace_bytes(int nmod, int m, int n, int k) {
    if (nmod != 32 || !split_shape_ok(m, n, k)) return 0;
    return split_scratch(nmod, m, n, k, nullptr, nullptr);
}

cudaError_t launch_gemm_split_marked(int nmod, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A,
                                     int lda, const mp_array_t &B, int ldb, const mp_array_t &beta,
                                     const mp_array_t &C, int ldc, Workspace ws, cudaStream_t s, cudaEvent_t *marks) {
    if (nmod != 32 || ws.ptr == nullptr || ws.bytes < gemm_split_workspace_bytes(nmod, m, n, k) ||
        !split_shape_ok(m, n, k))
        return cudaErrorNotSupported;
    return run_split<32>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, s, marks);
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
