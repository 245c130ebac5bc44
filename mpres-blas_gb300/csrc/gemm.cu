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
 */
/* every SM holds many product chains here and the FP64 pipe binds: the
 * interval evaluation runs in fixed point on the integer pipes (mp_device.cuh) */
#define MPRES_EVAL_FIXED_POINT 1
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
        res.ev[0].frac = -up.frac; res.ev[0].exp = up.exp;
        res.ev[1].frac = -lo.frac; res.ev[1].exp = lo.exp;
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

/* Three 128-thread blocks per SM (at most 168 registers a thread): measured
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

template <int N>
cudaError_t run(int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda, const mp_array_t &B,
                int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc, cudaStream_t s) {
    constexpr int BX = 32, BY = 4;
    dim3 block(BX, BY), grid((m + BX - 1) / BX, (n + BY - 1) / BY);
    gemm_nn<N, BX, BY><<<grid, block, 0, s>>>(m, n, k, soa(alpha), soa(A), lda, soa(B), ldb, soa(beta), C.digits,
                                              C.sign, C.exp, reinterpret_cast<er_t *>(C.eval), C.len, ldc);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_gemm(int nmod, int m, int n, int k, const mp_array_t &alpha, const mp_array_t &A, int lda,
                        const mp_array_t &B, int ldb, const mp_array_t &beta, const mp_array_t &C, int ldc,
                        cudaStream_t s) {
    switch (nmod) {
    case 8: return run<8>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
    case 16: return run<16>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
    case 32: return run<32>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
