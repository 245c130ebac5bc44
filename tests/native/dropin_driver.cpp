// A benchmark-style driver written against the drop-in header
// include/mpres_gb300.hpp, the way the reference's own drivers call its hot path
// (tests/blas/performance/test_{dot,gemv,gemm}_performance.cu,
// tests/sparse/spmv/csr/test_mpres_spmv_csr.cuh): rns_const_init /
// mp_const_init, mp_array_init + host2device, the templated call, device2host.
// Inputs and outputs are raw files of mp_float_t records (ints and doubles for
// the CSR arrays), so a test can write seeded inputs and check the outputs.
// Compile with -DRNS_MODULI_SIZE=8|16|32.
//
//   driver dot  n x y out
//   driver gemv m n alpha A x beta y out        (NO_TRANS, lda = m)
//   driver gemm m n k alpha A B beta C out      (NN, lda = m, ldb = k, ldc = m)
//   driver spmv m nnz irp ja as x out           (CSR, x and y AoS in device memory)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "mpres_gb300.hpp"

template <class T> static std::vector<T> load(const char *path, size_t count) {
    std::vector<T> v(count);
    FILE *f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(T), count, f) != count) {
        std::fprintf(stderr, "cannot read %zu items from %s\n", count, path);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}
template <class T> static void save(const char *path, const std::vector<T> &v) {
    FILE *f = std::fopen(path, "wb");
    if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
}
static mp_array_t device_array(std::vector<mp_float_t> &h) {
    mp_array_t a;
    cuda::mp_array_init(a, h.size());
    cuda::mp_array_host2device(a, h.data(), h.size());
    return a;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    rns_const_init();
    mp_const_init();
    const char *op = argv[1];
    if (!std::strcmp(op, "dot") && argc == 6) {
        const int n = std::atoi(argv[2]);
        auto hx = load<mp_float_t>(argv[3], n), hy = load<mp_float_t>(argv[4], n);
        std::vector<mp_float_t> hr(1);
        mp_array_t x = device_array(hx), y = device_array(hy), r, buf;
        cuda::mp_array_init(r, 1);
        cuda::mp_array_init(buf, n);
        cuda::mp_dot<512, 128, 8192, 256, 64>(n, x, 1, y, 1, r, buf);
        cuda::mp_array_device2host(hr.data(), r, 1);
        save(argv[5], hr);
        cuda::mp_array_clear(x); cuda::mp_array_clear(y); cuda::mp_array_clear(r); cuda::mp_array_clear(buf);
    } else if (!std::strcmp(op, "gemv") && argc == 10) {
        const int m = std::atoi(argv[2]), n = std::atoi(argv[3]);
        auto ha = load<mp_float_t>(argv[4], 1), hA = load<mp_float_t>(argv[5], (size_t)m * n);
        auto hx = load<mp_float_t>(argv[6], n), hb = load<mp_float_t>(argv[7], 1), hy = load<mp_float_t>(argv[8], m);
        mp_array_t al = device_array(ha), A = device_array(hA), x = device_array(hx), be = device_array(hb),
                   y = device_array(hy), b1, b2;
        cuda::mp_array_init(b1, n);
        cuda::mp_array_init(b2, (size_t)m * n);
        cuda::mp_gemv<256, 128, 256, 32>(mblas_no_trans, m, n, al, A, m, x, 1, be, y, 1, b1, b2);
        cuda::mp_array_device2host(hy.data(), y, m);
        save(argv[9], hy);
        for (mp_array_t *a : {&al, &A, &x, &be, &y, &b1, &b2}) cuda::mp_array_clear(*a);
    } else if (!std::strcmp(op, "gemm") && argc == 11) {
        const int m = std::atoi(argv[2]), n = std::atoi(argv[3]), k = std::atoi(argv[4]);
        auto ha = load<mp_float_t>(argv[5], 1), hA = load<mp_float_t>(argv[6], (size_t)m * k);
        auto hB = load<mp_float_t>(argv[7], (size_t)k * n), hb = load<mp_float_t>(argv[8], 1);
        auto hC = load<mp_float_t>(argv[9], (size_t)m * n);
        mp_array_t al = device_array(ha), A = device_array(hA), B = device_array(hB), be = device_array(hb),
                   C = device_array(hC), buf;
        cuda::mp_array_init(buf, (size_t)m * n);
        cuda::mp_gemm<32, 1, 128, 64, 16>(mblas_no_trans, mblas_no_trans, m, n, k, al, A, m, B, k, be, C, m, buf);
        cuda::mp_array_device2host(hC.data(), C, (size_t)m * n);
        save(argv[10], hC);
        for (mp_array_t *a : {&al, &A, &B, &be, &C, &buf}) cuda::mp_array_clear(*a);
    } else if (!std::strcmp(op, "spmv") && argc == 9) {
        const int m = std::atoi(argv[2]), nnz = std::atoi(argv[3]);
        auto irp = load<int>(argv[4], m + 1), ja = load<int>(argv[5], nnz);
        auto as = load<double>(argv[6], nnz);
        auto hx = load<mp_float_t>(argv[7], m);
        std::vector<mp_float_t> hy(m);
        csr_t host{as.data(), ja.data(), irp.data()}, dev;
        cuda::csr_init(dev, m, nnz);
        cuda::csr_host2device(dev, host, m, nnz);
        mp_float_t *dx = nullptr, *dy = nullptr;
        if (cudaMalloc(&dx, sizeof(mp_float_t) * m) != cudaSuccess ||
            cudaMalloc(&dy, sizeof(mp_float_t) * m) != cudaSuccess)
            return 3;
        cudaMemcpy(dx, hx.data(), sizeof(mp_float_t) * m, cudaMemcpyHostToDevice);
        cuda::mp_spmv_csr<32>(m, dev, dx, dy);
        cudaDeviceSynchronize();
        cudaMemcpy(hy.data(), dy, sizeof(mp_float_t) * m, cudaMemcpyDeviceToHost);
        save(argv[8], hy);
        cudaFree(dx);
        cudaFree(dy);
        cuda::csr_clear(dev);
    } else {
        std::fprintf(stderr, "bad arguments\n");
        return 2;
    }
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 4;
}
