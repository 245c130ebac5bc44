/*
 * mp_dot: r = sum_i x_i * y_i over SoA multiple-precision vectors.
 *
 * Reference: cuda::mp_dot<g1,b1,g2,g3,b3> (src/blas/dot.cuh:85-108) runs three
 * element-wise kernels that write every product to `buffer` (src/mpvector.cuh:45,
 * :96, :669) and then the two-pass reduction of src/mpreduct.cuh:38-115, which
 * cudaMallocs its block buffer on every call (src/blas/dot.cuh:42-66).
 *
 * Here the products are formed in registers by the threads that sum them, so no
 * product vector goes through HBM, and the block sums go to a preallocated
 * workspace.  The summation order -- which partial sum each product joins, and
 * the shape of both trees -- is exactly the reference's for the same
 * (gridDim3, blockDim3), so the result is bit-identical:
 *   pass 1: gridDim3 blocks of blockDim3 threads; thread p accumulates products
 *           p, p + K, p + 2K, ... (K = gridDim3 * blockDim3) from zero, then the
 *           tree halving from nextPow2(blockDim3)/2 (shared memory down to
 *           stride 32, warp shuffles below: tree_sum);
 *   pass 2: one block of blockDim3 threads does the same over the gridDim3
 *           block sums and writes r[0].
 */
#include "../../include/mpres_gb300.h"
#include "kernels.h"
#include "mp_device.cuh"

MPRES_DEFINE_TABLES(dot)

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
SoA soa(const mp_array_t &a) {
    return SoA{a.digits, a.sign, a.exp, reinterpret_cast<const er_t *>(a.eval), a.len};
}

__host__ __device__ inline unsigned next_pow2(unsigned v) {
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    return v + 1;
}

template <int N, int MAXT>
__global__ void __launch_bounds__(MAXT) dot_pass1(int n, SoA x, int incx, SoA y, int incy, void *block_sums) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    const unsigned tid = threadIdx.x, bsize = blockDim.x;
    const long long K = (long long)gridDim.x * bsize;
    const int lenx = __ldg(x.len), leny = __ldg(y.len);
    mp_t<N> acc;
    set_zero<N>(acc);
    for (long long i = (long long)blockIdx.x * bsize + tid; i < n; i += K) {
        mp_t<N> a, b, p, s;
        load_soa<N>(a, x.digits, x.sign, x.exp, x.eval, lenx, blas_index(i, n, incx));
        load_soa<N>(b, y.digits, y.sign, y.exp, y.eval, leny, blas_index(i, n, incy));
        mp_mul<N>(p, a, b);
        mp_add<N>(s, acc, p);
        acc = s;
    }
    sdata[tid] = acc;
    __syncthreads();
    tree_sum<N>(sdata, (int)tid, (int)bsize, true);
    if (tid == 0) store_aos<N>(sdata[0], block_sums, blockIdx.x);
}

template <int N, int MAXT>
__global__ void __launch_bounds__(MAXT) dot_pass2(int g3, const void *block_sums, int *rd, int *rs, int *re,
                                                  er_t *rv, const int *rlen) {
    extern __shared__ __align__(16) unsigned char smem[];
    mp_t<N> *sdata = reinterpret_cast<mp_t<N> *>(smem);
    const unsigned tid = threadIdx.x, bsize = blockDim.x;
    mp_t<N> acc;
    set_zero<N>(acc);
    for (int i = tid; i < g3; i += bsize) {
        mp_t<N> b, s;
        load_aos<N>(b, block_sums, i);
        mp_add<N>(s, acc, b);
        acc = s;
    }
    sdata[tid] = acc;
    __syncthreads();
    tree_sum<N>(sdata, (int)tid, (int)bsize, true);
    if (tid == 0) store_soa<N>(sdata[0], rd, rs, re, rv, __ldg(rlen), 0);
}

template <int N, int MAXT>
cudaError_t run_shape(int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy, const mp_array_t &r,
                      int g3, int b3, Workspace ws, cudaStream_t s) {
    const size_t smem = (size_t)b3 * sizeof(mp_t<N>);
    /* the shared-memory limit of both passes, raised on each device that runs them */
    static PerDevice<cudaError_t> attrs(cuda_ok);
    cudaError_t e = attrs.get(current_device(), cudaErrorInvalidDevice, [] {
        cudaError_t r = cudaFuncSetAttribute(dot_pass1<N, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             MAXT * sizeof(mp_t<N>));
        if (r != cudaSuccess) return r;
        return cudaFuncSetAttribute(dot_pass2<N, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    MAXT * sizeof(mp_t<N>));
    });
    if (e != cudaSuccess) return e;
    dot_pass1<N, MAXT><<<g3, b3, smem, s>>>(n, soa(x), incx, soa(y), incy, ws.ptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dot_pass2<N, MAXT><<<1, b3, smem, s>>>(g3, ws.ptr, r.digits, r.sign, r.exp, reinterpret_cast<er_t *>(r.eval),
                                           r.len);
    return cudaGetLastError();
}

template <int N>
cudaError_t run(int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy, const mp_array_t &r, int g3,
                int b3, Workspace ws, cudaStream_t s) {
    if (ws.bytes < (size_t)g3 * (4 * N + 40)) return cudaErrorInvalidValue;
    /* blocks of up to 256 threads get up to 255 registers; larger ones 64 */
    if (b3 <= 256) return run_shape<N, 256>(n, x, incx, y, incy, r, g3, b3, ws, s);
    return run_shape<N, 1024>(n, x, incx, y, incy, r, g3, b3, ws, s);
}

/* Scratch of mpres_dot_noalloc: the gridDim3 block sums of one call.  A
 * file-scope device array, so that the entry point never allocates; every GPU
 * that loads the library holds it until the process exits.  Its host-side name
 * is a stand-in, not a device address: the address comes from
 * cudaGetSymbolAddress, once per device, with that device current. */
__device__ __align__(256) unsigned char g_dot_noalloc_scratch[MPRES_DOT_NOALLOC_MAX_BLOCKS * (4 * 32 + 40)];

bool nonnull(void *const &p) { return p != nullptr; }

} // namespace

cudaError_t dot_noalloc_scratch(Workspace &ws) {
    static PerDevice<void *> addrs(nonnull);
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    cudaError_t e = cudaSuccess;
    void *p = addrs.get(dev, nullptr, [&e] {
        void *a = nullptr;
        e = cudaGetSymbolAddress(&a, g_dot_noalloc_scratch);
        return e == cudaSuccess ? a : nullptr;
    });
    if (!p) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
    ws.ptr = p;
    ws.bytes = sizeof(g_dot_noalloc_scratch);
    return cudaSuccess;
}

cudaError_t launch_dot(int nmod, int n, const mp_array_t &x, int incx, const mp_array_t &y, int incy,
                       const mp_array_t &r, int g3, int b3, Workspace ws, cudaStream_t s) {
    switch (nmod) {
    case 8: return run<8>(n, x, incx, y, incy, r, g3, b3, ws, s);
    case 16: return run<16>(n, x, incx, y, incy, r, g3, b3, ws, s);
    case 32: return run<32>(n, x, incx, y, incy, r, g3, b3, ws, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace mpres
