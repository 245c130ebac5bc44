/*
 * The reference library's device code (MPRES-BLAS src/, compiled UNMODIFIED
 * from where it lies) as a cubin for the GB300, so that the reference's own
 * GPU kernels and device arithmetic can run on the same device as this
 * library.  TEST AND BENCHMARK INFRASTRUCTURE ONLY.
 *
 * Built by oracle/ref/build_ref.sh into oracle/_ref/ref_kernels_<N>.cubin
 * (device code only: the cubin is loaded with the CUDA driver API by
 * oracle/ref_gpu.py; its __constant__ tables are filled from
 * oracle/_ref/ref_consts_<N>.bin, the values the reference's rns_const_init /
 * mp_const_init computes, dumped from the CPU build by dump_consts.py).
 *
 * Besides the reference's own __global__ kernels (mp_vector_*, mp_array_reduce_*,
 * matrix_multiply_notrans_kernel, matrix_row_sum_kernel, mp_mat*, mp_spmv_csr<32>, mp_spmv_csrv<32, tpr>,
 * mp_spmv_ell<32>, ...), three
 * element-wise entry points apply the reference's device arithmetic to AoS
 * records: r[i] = x[i] + y[i] (cuda::mp_add, src/arith/add.cuh:190-202),
 * x[i] * y[i] (cuda::mp_mul, src/arith/mul.cuh:71-80) and x[i] * d[i]
 * (cuda::mp_mul_d, src/arith/muld.cuh:59-74).
 */
#include <cstdint>
#include <cstdio>

#include "arith/assign.cuh"
#include "arith/add.cuh"
#include "arith/mul.cuh"
#include "arith/muld.cuh"
#include "mpvector.cuh"
#include "mpmatrix.cuh"
#include "mpreduct.cuh"
#include "blas/mblas_enum.cuh"
#include "kernel_config.cuh"
#include "blas/dot.cuh"
#include "blas/gemm.cuh"
#include "blas/gemv.cuh"
#include "sparse/spmv/spmv_csr.cuh"
#include "sparse/spmv/spmv_csrv.cuh"
#include "sparse/spmv/spmv_ell.cuh"

/* the SpMV kernels at the reference benchmark's block size (templates): CSR,
 * CSR-vector for every threads-per-row value, ELLPACK */
template __global__ void cuda::mp_spmv_csr<32>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 1>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 2>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 4>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 8>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 16>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_csrv<32, 32>(const int, const csr_t, mp_float_ptr, mp_float_ptr);
template __global__ void cuda::mp_spmv_ell<32>(const int, const int, const ell_t, mp_float_ptr, mp_float_ptr);

extern "C" __global__ void ref_ew_add(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        cuda::mp_add(&r[i], x[i], y[i]);
}
extern "C" __global__ void ref_ew_mul(const mp_float_t *x, const mp_float_t *y, mp_float_t *r, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        cuda::mp_mul(&r[i], x[i], y[i]);
}
extern "C" __global__ void ref_ew_mul_d(const mp_float_t *x, const double *d, mp_float_t *r, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        cuda::mp_mul_d(&r[i], x[i], d[i]);
}
