/*
 * mp_gemv: y = alpha*op(A)*x + beta*y, A column-major SoA (src/types.cuh:85-92).
 *
 * Reference: cuda::mp_gemv<g1,b1,g2,b3> (src/blas/gemv.cuh:151-269) runs ten
 * kernels: buffer1 = alpha*x, y = beta*y, the whole m-by-n matrix of products
 * buffer2 = A*diag(buffer1) (or diag(buffer1)*A) written to HBM, and finally
 * matrix_row_sum_kernel / matrix_col_sum_kernel (:44-128): per output, blockDim3
 * threads sum the products of strided columns (rows) serially, a shared-memory
 * tree adds the partial sums, and y = y + sum.
 *
 * Here: pass 1 forms buffer1 = alpha*x in a small workspace; pass 2 computes each
 * product in registers where it is summed (the m-by-n intermediate never exists)
 * and fuses y = beta*y into the final addition.  One block serves several
 * outputs with blockDim3 chains each, laid out so that a warp reads contiguous
 * matrix elements.  The summation order equals the reference's for the same
 * blockDim3, so results are bit-identical.
 */
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(gemv)

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

__host__ __device__ inline unsigned next_pow2(unsigned v) {
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    return v + 1;
}

/* buffer1[j] = alpha * x[j] (mp_vec2scal_mul_* + mp_vector_round_kernel) */
template <int N>
__global__ void __launch_bounds__(256) scale_vector(int len, SoA x, int incx, SoA alpha, void *out) {
    const int lenx = __ldg(x.len), lena = __ldg(alpha.len);
    mp_t<N> a;
    load_soa<N>(a, alpha.digits, alpha.sign, alpha.exp, alpha.eval, lena, 0);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < len; j += gridDim.x * blockDim.x) {
        mp_t<N> v, r;
        load_soa<N>(v, x.digits, x.sign, x.exp, x.eval, lenx, blas_index(j, len, incx));
        mp_mul<N>(r, v, a);
        store_aos<N>(r, out, j);
    }
}

/* Per output o (a row of A, or a column when TRANS), chain c of B3 sums the
 * products of inner indices c, c + b3, c + 2*b3, ...; then the tree, then
 * y[o] = beta*y[o] + sum. */
template <int N, int MAXT, bool TRANS>
__global__ void __launch_bounds__(MAXT) gemv_sums(int m, int n, SoA A, int lda, const void *buf1, SoA beta,
                                                  int *yd, int *ys, int *ye, er_t *yv, const int *ylen, int incy,
                                                  int b3, int outs_per_block) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    const int R = outs_per_block;
    const int t = threadIdx.x;
    /* no-trans: consecutive threads take consecutive rows; trans: consecutive chains */
    const int r = TRANS ? t / b3 : t % R;
    const int c = TRANS ? t % b3 : t / R;
    const int outs = TRANS ? n : m, inner = TRANS ? m : n;
    const int o = blockIdx.x * R + r;
    const bool active = (r < R) && (c < b3) && (o < outs);
    const int lena = __ldg(A.len);
    mp_t<N> acc;
    set_zero<N>(acc);
    if (active) {
        for (int j = c; j < inner; j += b3) {
            const long long row = TRANS ? j : o, col = TRANS ? o : j;
            mp_t<N> a, xb, p, s;
            load_soa<N>(a, A.digits, A.sign, A.exp, A.eval, lena, col * lda + row);
            load_aos<N>(xb, buf1, TRANS ? row : col);
            mp_mul<N>(p, a, xb);
            mp_add<N>(s, acc, p);
            acc = s;
        }
    }
    const int slot = TRANS ? (r * b3 + c) : (c * R + r);
    if (r < R && c < b3) sdata[slot] = acc;
    __syncthreads();
    for (unsigned i = next_pow2((unsigned)b3) >> 1; i >= 1; i >>= 1) {
        if (active && (unsigned)c < i && (unsigned)c + i < (unsigned)b3) {
            const int other = TRANS ? (r * b3 + c + (int)i) : ((c + (int)i) * R + r);
            mp_t<N> x0 = sdata[slot], x1 = sdata[other], s;
            mp_add<N>(s, x0, x1);
            sdata[slot] = s;
        }
        __syncthreads();
    }
    if (active && c == 0) {
        const int leny = __ldg(ylen), lenb = __ldg(beta.len);
        const long long iy = blas_index(o, outs, incy);
        mp_t<N> yv0, bv, yb, res;
        load_soa<N>(yv0, yd, ys, ye, yv, leny, iy);
        load_soa<N>(bv, beta.digits, beta.sign, beta.exp, beta.eval, lenb, 0);
        mp_mul<N>(yb, yv0, bv);
        mp_t<N> sum = sdata[slot];
        mp_add<N>(res, yb, sum);
        store_soa<N>(res, yd, ys, ye, yv, leny, iy);
    }
}

template <int N, int MAXT, bool TRANS>
cudaError_t sums(int m, int n, const mp_array_t &A, int lda, const void *buf1, const mp_array_t &beta,
                 const mp_array_t &y, int incy, int b3, cudaStream_t s) {
    const int R = MAXT / b3 > 32 ? 32 : (MAXT / b3 < 1 ? 1 : MAXT / b3);
    const int threads = R * b3;
    const int outs = TRANS ? n : m;
    const int grid = (outs + R - 1) / R;
    const size_t smem = (size_t)threads * sizeof(mp_t<N>);
    /* the shared-memory limit, raised on each device that runs the kernel */
    static PerDevice<cudaError_t> attrs(cuda_ok);
    cudaError_t e = attrs.get(current_device(), cudaErrorInvalidDevice, [] {
        return cudaFuncSetAttribute(gemv_sums<N, MAXT, TRANS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    MAXT * sizeof(mp_t<N>));
    });
    if (e != cudaSuccess) return e;
    gemv_sums<N, MAXT, TRANS><<<grid, threads, smem, s>>>(m, n, soa(A), lda, buf1, soa(beta), y.digits, y.sign, y.exp,
                                                          reinterpret_cast<er_t *>(y.eval), y.len, incy, b3, R);
    return cudaGetLastError();
}

template <int N>
cudaError_t run(bool trans, int m, int n, const mp_array_t &alpha, const mp_array_t &A, int lda, const mp_array_t &x,
                int incx, const mp_array_t &beta, const mp_array_t &y, int incy, int b3, Workspace ws,
                cudaStream_t s) {
    const int lx = trans ? m : n;
    if (ws.bytes < (size_t)lx * (4 * N + 40)) return cudaErrorInvalidValue;
    int g = (lx + 255) / 256;
    scale_vector<N><<<g, 256, 0, s>>>(lx, soa(x), incx, soa(alpha), ws.ptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (b3 <= 256) {
        return trans ? sums<N, 256, true>(m, n, A, lda, ws.ptr, beta, y, incy, b3, s)
                     : sums<N, 256, false>(m, n, A, lda, ws.ptr, beta, y, incy, b3, s);
    }
    return trans ? sums<N, 1024, true>(m, n, A, lda, ws.ptr, beta, y, incy, b3, s)
                 : sums<N, 1024, false>(m, n, A, lda, ws.ptr, beta, y, incy, b3, s);
}

} // namespace

cudaError_t launch_gemv(int nmod, bool trans, int m, int n, const mp_array_t &alpha, const mp_array_t &A, int lda,
                        const mp_array_t &x, int incx, const mp_array_t &beta, const mp_array_t &y, int incy,
                        int b3, Workspace ws, cudaStream_t s) {
    switch (nmod) {
    case 8: return run<8>(trans, m, n, alpha, A, lda, x, incx, beta, y, incy, b3, ws, s);
    case 16: return run<16>(trans, m, n, alpha, A, lda, x, incx, beta, y, incy, b3, ws, s);
    case 32: return run<32>(trans, m, n, alpha, A, lda, x, incx, beta, y, incy, b3, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
