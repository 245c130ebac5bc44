/*
 * C ABI of libmpres_gb300.so (declared in include/mpres_gb300.h): argument
 * checks with the reference's quick-return rules, constant set-up, containers,
 * per-stream workspaces and the kernel launchers.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/mpres_gb300.h"
#include "../../include/mpres_gb300_probe.h"
#include "kernels.h"
#include "tables.h"

namespace mpres {
void host_set_d(const HostTables &t, const double *x, size_t count, void *out);
bool host_mp_div(const HostTables &t, const void *x, const void *y, void *r);
bool host_mp_sqrt(const HostTables &t, const void *x, void *r);
bool host_mp_dsqrt(const HostTables &t, const void *x, double &out);
}

using namespace mpres;

namespace {

/* last error of this host thread; a fixed buffer, so reporting never allocates */
thread_local char g_err[512];

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
int ok() {
    g_err[0] = '\0';
    return MPRES_SUCCESS;
}
int cuda_fail(cudaError_t e, const char *what) {
    return fail(MPRES_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int set_slot(int nmod) { return nmod == 8 ? 0 : nmod == 16 ? 1 : nmod == 32 ? 2 : -1; }

struct SetState {
    bool host_ready = false;
    HostTables host;
    std::map<int, bool> device_ready; /* device ordinal -> uploaded */
    std::map<int, std::pair<int *, int *>> device_tables;
};

std::mutex g_mu;
SetState g_sets[3];
int *g_ceil_log2[64]; /* per device */
int *g_host_log2[64];  /* per device: host_ceil_log2_table() */
int g_host_log2_tab[2 * kHostLog2Entries];
int g_host_log2_state = 0; /* 0 not measured, 1 measured, -1 the host's log2 is not usable */

struct WsKey {
    int device;
    cudaStream_t stream;
    bool operator<(const WsKey &o) const { return device != o.device ? device < o.device : stream < o.stream; }
};
std::map<WsKey, Workspace> g_ws;
Workspace g_staging[64]; /* per device: records in transit for the array copies */
std::mutex g_copy_mu;

/* ceil(log2(2^e)) for e = -1074..1023 with CUDA's log2, the values the
 * reference's refinement loop takes at exact powers of two (fixed_eval.cuh) */
__global__ void ceil_log2_pow2_kernel(int *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 2098) out[i] = (int)ceil(log2(ldexp(1.0, i - 1074)));
}

template <int N>
void fill_tables(const HostTables &h, const int *dpow2, const int *dpow2_inv, const int *dceil, const int *dhost_log2,
                 Tables<N> &t) {
    std::memset(&t, 0, sizeof(t));
    for (int i = 0; i < N; i++) {
        t.moduli[i] = h.moduli[i];
        t.mu[i] = h.mu[i];
        t.part_inv[i] = h.part_inv[i];
        t.recip_rd[i] = h.recip_rd[i];
        t.recip_ru[i] = h.recip_ru[i];
        t.part_pow2_res30[i] = h.part_pow2_res[kScaleBits - 1][i];
        for (int j = 0; j < N; j++) t.mrc_inv[i][j] = h.mrc_inv[i][j];
    }
    t.m_pow2_res30 = h.m_pow2_res[kScaleBits - 1];
    t.eval_acc = h.eval_acc;
    t.ref_factor = h.ref_factor;
    t.mp_h = h.mp_h;
    t.mp_j = h.mp_j;
    t.mp_precision = h.mp_precision;
    t.log2m = h.log2m;
    t.unit_low = h.unit_low;
    t.unit_upp = h.unit_upp;
    t.inv_unit_low = h.inv_unit_low;
    t.inv_unit_upp = h.inv_unit_upp;
    t.pow2 = dpow2;
    t.pow2_inv = dpow2_inv;
    t.ceil_log2_pow2 = dceil;
    t.host_ceil_log2 = dhost_log2;
    for (int i = 0; i < N; i++) t.recip_rn[i] = 1.0 / (double)h.moduli[i];
    for (int i = 0; i < N; i++) t.pow2_32[i] = (uint32_t)((1ull << 32) % (unsigned long long)h.moduli[i]);
    for (int i = 0; i < N; i++)
        t.inv94[i] = (uint64_t)((((unsigned __int128)1) << 94) / (unsigned __int128)(unsigned)h.moduli[i]);
    for (int i = 0; i < N; i++) { /* (2^-1)^log2m, 2^-1 = (m + 1) / 2 for the odd m */
        const uint64_t md = (uint64_t)(unsigned)h.moduli[i];
        uint64_t base = (md + 1) / 2, r = 1;
        for (unsigned e = (unsigned)h.log2m; e; e >>= 1) {
            if (e & 1u) r = r * base % md;
            base = base * base % md;
        }
        t.pow2_neg_top[i] = (uint32_t)r;
    }
    for (int i = 0; i < N; i++) {
        t.recip_rd_m[i] = h.recip_rd_m[i];
        t.recip_ru_m[i] = h.recip_ru_m[i];
    }
    t.eval_acc_fx[0] = h.eval_acc_fx[0];
    t.eval_acc_fx[1] = h.eval_acc_fx[1];
    t.unit_upp_recip = h.unit_upp_recip;
    t.unit_low_recip = h.unit_low_recip;
    t.unit_upp_inv = h.unit_upp_inv;
    t.unit_low_inv = h.unit_low_inv;
}

template <int N>
cudaError_t upload_all(const HostTables &h, const int *dpow2, const int *dpow2_inv, const int *dceil,
                       const int *dhost_log2) {
    Tables<N> t;
    fill_tables<N>(h, dpow2, dpow2_inv, dceil, dhost_log2, t);
    cudaError_t e;
    if ((e = upload_tables_dot(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_gemv(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_gemm(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_elementwise(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_convert(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_batch(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_solver(N, &t)) != cudaSuccess) return e;
    if ((e = upload_tables_probe_fx(N, &t)) != cudaSuccess) return e;
    return upload_tables_spmv(N, &t);
}

/* requires g_mu held */
int init_locked(int nmod) {
    const int slot = set_slot(nmod);
    if (slot < 0) return fail(MPRES_ERR_INVALID_VALUE, "unsupported moduli set size %d (8, 16 or 32)", nmod);
    SetState &st = g_sets[slot];
    if (!st.host_ready) {
        if (!compute_host_tables(nmod, st.host)) return fail(MPRES_ERR_INVALID_VALUE, "tables of set %d", nmod);
        st.host_ready = true;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (st.device_ready[dev]) return ok();
    const HostTables &h = st.host;
    const size_t pow2_bytes = sizeof(int) * (size_t)(h.log2m + 1) * nmod;
    const size_t inv_bytes = sizeof(int) * (size_t)kScaleBits * nmod;
    int *dpow2 = nullptr, *dinv = nullptr;
    if ((e = cudaMalloc(&dpow2, pow2_bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
    if ((e = cudaMalloc(&dinv, inv_bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
    std::vector<int> inv((size_t)kScaleBits * nmod);
    for (int r = 0; r < kScaleBits; r++)
        for (int j = 0; j < nmod; j++) inv[(size_t)r * nmod + j] = h.pow2_inv[r][j];
    if ((e = cudaMemcpy(dpow2, h.pow2, pow2_bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(tables)");
    if ((e = cudaMemcpy(dinv, inv.data(), inv_bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(tables)");
    int *&dceil = g_ceil_log2[dev < 64 ? dev : 0];
    if (!dceil) {
        if ((e = cudaMalloc(&dceil, sizeof(int) * 2098)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
        ceil_log2_pow2_kernel<<<(2098 + 255) / 256, 256>>>(dceil);
        if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail(e, "ceil_log2_pow2_kernel");
    }
    if (g_host_log2_state == 0) g_host_log2_state = host_ceil_log2_table(g_host_log2_tab) ? 1 : -1;
    int *&dhl = g_host_log2[dev < 64 ? dev : 0];
    if (!dhl && g_host_log2_state > 0) {
        if ((e = cudaMalloc(&dhl, sizeof(g_host_log2_tab))) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
        if ((e = cudaMemcpy(dhl, g_host_log2_tab, sizeof(g_host_log2_tab), cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpy(tables)");
    }
    if (nmod == 8) e = upload_all<8>(h, dpow2, dinv, dceil, dhl);
    if (nmod == 16) e = upload_all<16>(h, dpow2, dinv, dceil, dhl);
    if (nmod == 32) e = upload_all<32>(h, dpow2, dinv, dceil, dhl);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyToSymbol(tables)");
    st.device_tables[dev] = {dpow2, dinv};
    st.device_ready[dev] = true;
    return ok();
}

int require(int nmod) {
    const int slot = set_slot(nmod);
    if (slot < 0) return fail(MPRES_ERR_INVALID_VALUE, "unsupported moduli set size %d (8, 16 or 32)", nmod);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_sets[slot].device_ready.find(dev);
    if (it == g_sets[slot].device_ready.end() || !it->second)
        return fail(MPRES_ERR_NOT_INITIALIZED, "mpres_init(%d) was not called on device %d", nmod, dev);
    return MPRES_SUCCESS;
}

/* Workspace of (device, stream), grown on demand: the first call on a stream
 * (or a call needing more room than before) allocates; later calls do not.
 * The larger buffer is allocated before the old one is released, so a request
 * that cannot be met leaves the stream's existing workspace in place (and the
 * next smaller call does not allocate again).  On failure nothing is reported
 * here: the caller decides whether the call fails (status_cuda) or takes a
 * path without scratch. */
cudaError_t workspace_grow(cudaStream_t s, size_t bytes, Workspace &out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_mu);
    Workspace &w = g_ws[WsKey{dev, s}];
    if (w.bytes < bytes) {
        const size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
        void *p = nullptr;
        if ((e = cudaMalloc(&p, want)) != cudaSuccess) {
            cudaGetLastError(); /* the failed allocation is not a sticky error */
            return e;
        }
        if (w.ptr) {
            cudaStreamSynchronize(s); /* work queued on s may still use the old buffer */
            cudaFree(w.ptr);
        }
        w.ptr = p;
        w.bytes = want;
    }
    out = w;
    return cudaSuccess;
}
int workspace(cudaStream_t s, size_t bytes, Workspace &out) {
    const cudaError_t e = workspace_grow(s, bytes, out);
    return e == cudaSuccess ? MPRES_SUCCESS : cuda_fail(e, "cudaMalloc(workspace)");
}

size_t mp_size(int nmod) { return 4 * (size_t)nmod + 40; }

} // namespace

/* status reporting for the entry points of the other translation units */
namespace mpres {
int status_fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
int status_ok() { return ok(); }
int status_cuda(cudaError_t e, const char *what) { return cuda_fail(e, what); }
int status_require(int nmod) { return require(nmod); }
} // namespace mpres

extern "C" {

const char *mpres_last_error(void) { return g_err; }

size_t mpres_mp_float_size(int nmod) { return set_slot(nmod) < 0 ? 0 : mp_size(nmod); }

int mpres_init(int nmod) {
    std::lock_guard<std::mutex> lk(g_mu);
    return init_locked(nmod);
}

int mpres_get_int_constants(int nmod, int *out) {
    const int slot = set_slot(nmod);
    if (slot < 0 || !out) return fail(MPRES_ERR_INVALID_VALUE, "unsupported moduli set size %d", nmod);
    std::lock_guard<std::mutex> lk(g_mu);
    SetState &st = g_sets[slot];
    if (!st.host_ready) {
        if (!compute_host_tables(nmod, st.host)) return fail(MPRES_ERR_INVALID_VALUE, "tables of set %d", nmod);
        st.host_ready = true;
    }
    out[0] = st.host.mp_precision;
    out[1] = st.host.mp_h;
    out[2] = st.host.mp_j;
    out[3] = st.host.ref_factor;
    out[4] = st.host.log2m;
    return ok();
}

int mpres_array_init(int nmod, mp_array_t *a, size_t size) {
    if (!a || set_slot(nmod) < 0) return fail(MPRES_ERR_INVALID_VALUE, "mpres_array_init: bad arguments");
    std::memset(a, 0, sizeof(*a));
    const size_t n = size ? size : 1;
    cudaError_t e;
    if ((e = cudaMalloc(&a->digits, sizeof(int) * (size_t)nmod * n)) != cudaSuccess ||
        (e = cudaMalloc(&a->sign, sizeof(int) * n)) != cudaSuccess ||
        (e = cudaMalloc(&a->exp, sizeof(int) * n)) != cudaSuccess ||
        (e = cudaMalloc(&a->eval, sizeof(er_float_t) * 2 * n)) != cudaSuccess ||
        (e = cudaMalloc(&a->buf, sizeof(mpres_int4) * n)) != cudaSuccess ||
        (e = cudaMalloc(&a->len, sizeof(int))) != cudaSuccess)
        return cuda_fail(e, "mpres_array_init");
    int len = (int)size;
    if ((e = cudaMemcpy(a->len, &len, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "mpres_array_init");
    return ok();
}

int mpres_array_clear(mp_array_t *a) {
    if (!a) return fail(MPRES_ERR_INVALID_VALUE, "mpres_array_clear: null array");
    cudaFree(a->digits);
    cudaFree(a->sign);
    cudaFree(a->exp);
    cudaFree(a->eval);
    cudaFree(a->buf);
    cudaFree(a->len);
    std::memset(a, 0, sizeof(*a));
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_array_clear");
}

/* Bulk copies between host mp_float_t records and a device mp_array_t: the
 * records travel as they are, in chunks through a device staging buffer, and a
 * kernel packs them into (or out of) the SoA fields.  The reference issues one
 * cudaMemcpy per element for the digits and packs sign, exp and eval on the
 * host (src/mparray.cuh:76-160); like it, the copies are synchronous, and the
 * upper bounds are placed `size` elements after the lower ones. */
static int array_copy(const char *what, int nmod, bool to_device, mp_array_t *a, char *host, size_t size) {
    const size_t rec = mp_size(nmod);
    const size_t chunk = std::max<size_t>(1, std::min<size_t>(size, ((size_t)256 << 20) / rec));
    cudaError_t e;
    std::lock_guard<std::mutex> lk(g_copy_mu); /* one copy at a time uses the staging buffer */
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_fail(e, what);
    Workspace &w = g_staging[dev < 64 ? dev : 0];
    if (w.bytes < chunk * rec) {
        if (w.ptr) cudaFree(w.ptr);
        w.ptr = nullptr;
        w.bytes = 0;
        if ((e = cudaMalloc(&w.ptr, chunk * rec)) != cudaSuccess) return cuda_fail(e, what);
        w.bytes = chunk * rec;
    }
    void *staging = w.ptr;
    for (size_t off = 0; off < size; off += chunk) {
        const size_t c = std::min(chunk, size - off);
        if (to_device) {
            if ((e = cudaMemcpy(staging, host + off * rec, c * rec, cudaMemcpyHostToDevice)) != cudaSuccess ||
                (e = launch_pack(nmod, true, staging, *a, (long long)size, (long long)off, (long long)c, 0)) != cudaSuccess)
                return cuda_fail(e, what);
        } else {
            if ((e = launch_pack(nmod, false, staging, *a, (long long)size, (long long)off, (long long)c, 0)) != cudaSuccess ||
                (e = cudaMemcpy(host + off * rec, staging, c * rec, cudaMemcpyDeviceToHost)) != cudaSuccess)
                return cuda_fail(e, what);
        }
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail(e, what);
    return ok();
}

int mpres_array_host2device(int nmod, mp_array_t *dst, const void *host_src, size_t size) {
    if (!dst || (!host_src && size) || set_slot(nmod) < 0)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_array_host2device: bad arguments");
    if (size == 0) return ok();
    return array_copy("mpres_array_host2device", nmod, true, dst, (char *)host_src, size);
}

int mpres_array_device2host(int nmod, void *host_dst, const mp_array_t *src, size_t size) {
    if (!src || (!host_dst && size) || set_slot(nmod) < 0)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_array_device2host: bad arguments");
    if (size == 0) return ok();
    return array_copy("mpres_array_device2host", nmod, false, const_cast<mp_array_t *>(src), (char *)host_dst, size);
}

int mpres_csr_init(csr_t *csr, int m, int nnz) {
    if (!csr || m < 0 || nnz < 0) return fail(MPRES_ERR_INVALID_VALUE, "mpres_csr_init: bad arguments");
    cudaError_t e;
    if ((e = cudaMalloc(&csr->as, sizeof(double) * (size_t)(nnz ? nnz : 1))) != cudaSuccess ||
        (e = cudaMalloc(&csr->ja, sizeof(int) * (size_t)(nnz ? nnz : 1))) != cudaSuccess ||
        (e = cudaMalloc(&csr->irp, sizeof(int) * (size_t)(m + 1))) != cudaSuccess)
        return cuda_fail(e, "mpres_csr_init");
    return ok();
}

int mpres_csr_host2device(csr_t *dev, const csr_t *host, int m, int nnz) {
    if (!dev || !host || m < 0 || nnz < 0) return fail(MPRES_ERR_INVALID_VALUE, "mpres_csr_host2device: bad arguments");
    cudaError_t e;
    if ((nnz && (e = cudaMemcpy(dev->as, host->as, sizeof(double) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (nnz && (e = cudaMemcpy(dev->ja, host->ja, sizeof(int) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (e = cudaMemcpy(dev->irp, host->irp, sizeof(int) * (size_t)(m + 1), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "mpres_csr_host2device");
    return ok();
}

int mpres_csr_clear(csr_t *csr) {
    if (!csr) return fail(MPRES_ERR_INVALID_VALUE, "mpres_csr_clear: null");
    cudaFree(csr->as);
    cudaFree(csr->ja);
    cudaFree(csr->irp);
    std::memset(csr, 0, sizeof(*csr));
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_csr_clear");
}

int mpres_ell_init(ell_t *ell, int m, int maxnzr) {
    if (!ell || m < 0 || maxnzr < 0) return fail(MPRES_ERR_INVALID_VALUE, "mpres_ell_init: bad arguments");
    size_t slots = (size_t)m * maxnzr;
    cudaError_t e;
    if ((e = cudaMalloc(&ell->as, sizeof(double) * (slots ? slots : 1))) != cudaSuccess ||
        (e = cudaMalloc(&ell->ja, sizeof(int) * (slots ? slots : 1))) != cudaSuccess)
        return cuda_fail(e, "mpres_ell_init");
    return ok();
}

int mpres_ell_host2device(ell_t *dev, const ell_t *host, int m, int maxnzr) {
    if (!dev || !host || m < 0 || maxnzr < 0)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_ell_host2device: bad arguments");
    size_t slots = (size_t)m * maxnzr;
    cudaError_t e;
    if (slots && ((e = cudaMemcpy(dev->as, host->as, sizeof(double) * slots, cudaMemcpyHostToDevice)) != cudaSuccess ||
                  (e = cudaMemcpy(dev->ja, host->ja, sizeof(int) * slots, cudaMemcpyHostToDevice)) != cudaSuccess))
        return cuda_fail(e, "mpres_ell_host2device");
    return ok();
}

int mpres_ell_clear(ell_t *ell) {
    if (!ell) return fail(MPRES_ERR_INVALID_VALUE, "mpres_ell_clear: null");
    cudaFree(ell->as);
    cudaFree(ell->ja);
    std::memset(ell, 0, sizeof(*ell));
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_ell_clear");
}

/* the host tables of a set, computed on first use */
static int host_tables_of(int nmod, const char *what, const HostTables *&t) {
    const int slot = set_slot(nmod);
    if (slot < 0) return fail(MPRES_ERR_INVALID_VALUE, "%s: unsupported moduli set size %d", what, nmod);
    std::lock_guard<std::mutex> lk(g_mu);
    SetState &st = g_sets[slot];
    if (!st.host_ready) {
        if (!compute_host_tables(nmod, st.host)) return fail(MPRES_ERR_INVALID_VALUE, "tables of set %d", nmod);
        st.host_ready = true;
    }
    t = &st.host;
    return MPRES_SUCCESS;
}

int mpres_div(int nmod, const void *x, const void *y, void *r) {
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_div", t)) return st;
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_div: null argument");
    if (!host_mp_div(*t, x, y, r)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_div: division by zero");
    return ok();
}

int mpres_sqrt(int nmod, const void *x, void *r) {
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_sqrt", t)) return st;
    if (!x || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_sqrt: null argument");
    if (!host_mp_sqrt(*t, x, r)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_sqrt: negative operand");
    return ok();
}

int mpres_dsqrt(int nmod, const void *x, double *out) {
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_dsqrt", t)) return st;
    if (!x || !out) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dsqrt: null argument");
    if (!host_mp_dsqrt(*t, x, *out)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dsqrt: negative operand");
    return ok();
}

/* the cuda:: forms: operands and result in device memory, computed on the host */
int mpres_div_device(int nmod, const void *x, const void *y, void *r) {
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_div_device", t)) return st;
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_div_device: null argument");
    const size_t sz = mp_size(nmod);
    char a[168], b[168], q[168];
    cudaError_t e;
    if ((e = cudaMemcpy(a, x, sz, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(b, y, sz, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "mpres_div_device");
    if (!host_mp_div(*t, a, b, q)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_div_device: division by zero");
    if ((e = cudaMemcpy(r, q, sz, cudaMemcpyHostToDevice)) != cudaSuccess) return cuda_fail(e, "mpres_div_device");
    return ok();
}

int mpres_dsqrt_device(int nmod, const void *x, double *out) {
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_dsqrt_device", t)) return st;
    if (!x || !out) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dsqrt_device: null argument");
    char a[168];
    cudaError_t e = cudaMemcpy(a, x, mp_size(nmod), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpres_dsqrt_device");
    if (!host_mp_dsqrt(*t, a, *out)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dsqrt_device: negative operand");
    return ok();
}

/* ---- v2 vector kernels and conjugate gradients ---- */

static int v2_threads(int threads, const char *what) {
    if (threads < 1 || threads > 256)
        return status_fail(MPRES_ERR_INVALID_VALUE, "%s: threads %d out of range (1..256)", what, threads);
    return MPRES_SUCCESS;
}

static int v2_vec(const char *what, int nmod, int op, int n, const void *alpha, const void *x, const void *y, void *r,
                  int threads, void *stream) {
    if (int st = require(nmod)) return st;
    if (n <= 0) return ok();
    if (!x || !y || !r || (op != 0 && !alpha)) return fail(MPRES_ERR_INVALID_VALUE, "%s: null argument", what);
    if (int st = v2_threads(threads, what)) return st;
    cudaError_t e = launch_vec_v2(nmod, op, n, threads, alpha, x, y, r, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, what);
}

int mpres_v2_diff(int nmod, int n, const void *x, const void *y, void *r, int threads, void *stream) {
    return v2_vec("mpres_v2_diff", nmod, 0, n, nullptr, x, y, r, threads, stream);
}
int mpres_v2_axpy(int nmod, int n, const void *alpha, const void *x, const void *y, void *r, int threads,
                  void *stream) {
    return v2_vec("mpres_v2_axpy", nmod, 1, n, alpha, x, y, r, threads, stream);
}
int mpres_v2_maxpy(int nmod, int n, const void *alpha, const void *x, const void *y, void *r, int threads,
                   void *stream) {
    return v2_vec("mpres_v2_maxpy", nmod, 2, n, alpha, x, y, r, threads, stream);
}

int mpres_v2_dot(int nmod, int n, const void *x, const void *y, void *r, int blocks, int threads, void *stream) {
    if (int st = require(nmod)) return st;
    if (n <= 0) return ok();
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_v2_dot: null argument");
    if (int st = v2_threads(threads, "mpres_v2_dot")) return st;
    if (blocks < 1) return fail(MPRES_ERR_INVALID_VALUE, "mpres_v2_dot: blocks %d", blocks);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, (size_t)blocks * mp_size(nmod), ws)) return st;
    cudaError_t e = launch_reduce_v2(nmod, false, n, blocks, threads, x, y, ws.ptr, r, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_v2_dot");
}

int mpres_v2_norm2(int nmod, int n, const void *x, double *out, int blocks, int threads, void *stream) {
    if (int st = require(nmod)) return st;
    if (!x || !out) return fail(MPRES_ERR_INVALID_VALUE, "mpres_v2_norm2: null argument");
    if (int st = v2_threads(threads, "mpres_v2_norm2")) return st;
    if (blocks < 1) return fail(MPRES_ERR_INVALID_VALUE, "mpres_v2_norm2: blocks %d", blocks);
    const HostTables *t;
    if (int st = host_tables_of(nmod, "mpres_v2_norm2", t)) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, (size_t)(blocks + 1) * mp_size(nmod), ws)) return st;
    char *parts = static_cast<char *>(ws.ptr), *sum = parts + (size_t)blocks * mp_size(nmod);
    cudaError_t e = launch_reduce_v2(nmod, true, n > 0 ? n : 0, blocks, threads, x, x, parts, sum, s);
    char h[168];
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, sum, mp_size(nmod), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "mpres_v2_norm2");
    if (!host_mp_dsqrt(*t, h, *out)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_v2_norm2: negative sum");
    return ok();
}

static int cg_common(const char *what, int nmod, int n, const csr_t *A, const void *b, double tol, int maxit,
                     const double *M, void *x, double *resvec, int resvec_cap, int *iters, int threads,
                     int blocks_reduce, void *stream) {
    if (int st = require(nmod)) return st;
    if (n <= 0 || !A || !b || !x || (resvec_cap > 0 && !resvec))
        return fail(MPRES_ERR_INVALID_VALUE, "%s: bad arguments", what);
    if (int st = v2_threads(threads, what)) return st;
    if (blocks_reduce < 1) return fail(MPRES_ERR_INVALID_VALUE, "%s: blocks_reduce %d", what, blocks_reduce);
    const HostTables *t;
    if (int st = host_tables_of(nmod, what, t)) return st;
    return solve_cg(nmod, *t, n, *A, b, tol, maxit, M, x, resvec, resvec_cap, iters, threads, blocks_reduce,
                    static_cast<cudaStream_t>(stream));
}

int mpres_cg_csr(int nmod, int n, const csr_t *A, const void *b, double tol, int maxit, void *x, double *resvec,
                 int resvec_cap, int *iters, int threads, int blocks_reduce, void *stream) {
    return cg_common("mpres_cg_csr", nmod, n, A, b, tol, maxit, nullptr, x, resvec, resvec_cap, iters, threads,
                     blocks_reduce, stream);
}

int mpres_pcg_csr(int nmod, int n, const csr_t *A, const void *b, double tol, int maxit, int ptype, const double *M,
                  void *x, double *resvec, int resvec_cap, int *iters, int threads, int blocks_reduce, void *stream) {
    if (ptype != 1 || !M)
        return fail(MPRES_ERR_NOT_SUPPORTED, "mpres_pcg_csr: only the diagonal (Jacobi) preconditioner, ptype 1");
    return cg_common("mpres_pcg_csr", nmod, n, A, b, tol, maxit, M, x, resvec, resvec_cap, iters, threads,
                     blocks_reduce, stream);
}

int mpres_set_d(int nmod, const double *x, size_t count, void *out) {
    const int slot = set_slot(nmod);
    if (slot < 0 || (count && (!x || !out))) return fail(MPRES_ERR_INVALID_VALUE, "mpres_set_d: bad arguments");
    const HostTables *t;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        SetState &st = g_sets[slot];
        if (!st.host_ready) {
            if (!compute_host_tables(nmod, st.host)) return fail(MPRES_ERR_INVALID_VALUE, "tables of set %d", nmod);
            st.host_ready = true;
        }
        t = &st.host;
    }
    host_set_d(*t, x, count, out);
    return ok();
}

/* the device conversion; out_aos or (dst, offset) */
static int set_d_device(const char *what, int nmod, const double *x, size_t count, void *out_aos,
                        const mp_array_t *dst, size_t offset, void *stream) {
    if (int st = require(nmod)) return st;
    if (count == 0) return ok();
    if (!x || (!out_aos && !dst)) return fail(MPRES_ERR_INVALID_VALUE, "%s: null pointer", what);
    if (g_host_log2_state < 0)
        return fail(MPRES_ERR_NOT_SUPPORTED, "%s: the host log2 is not monotone near powers of two; use mpres_set_d",
                    what);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, 256, ws)) return st;
    int *flag = static_cast<int *>(ws.ptr);
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    if (e == cudaSuccess) e = launch_set_d(nmod, x, (long long)count, out_aos, dst, (long long)offset, flag, s);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (h) return fail(MPRES_ERR_NOT_SUPPORTED, "%s: an input met a host-evaluation path not replayed on the device", what);
    return ok();
}

int mpres_set_d_device(int nmod, const double *x, size_t count, void *out, void *stream) {
    return set_d_device("mpres_set_d_device", nmod, x, count, out, nullptr, 0, stream);
}

int mpres_array_set_d(int nmod, mp_array_t *dst, size_t offset, const double *x, size_t count, void *stream) {
    if (!dst) return fail(MPRES_ERR_INVALID_VALUE, "mpres_array_set_d: null array");
    return set_d_device("mpres_array_set_d", nmod, x, count, nullptr, dst, offset, stream);
}

int mpres_dot(int nmod, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy, mp_array_t *r,
              mp_array_t *buffer, int gridDim1, int blockDim1, int gridDim2, int gridDim3, int blockDim3,
              void *stream) {
    (void)buffer; (void)gridDim1; (void)blockDim1; (void)gridDim2;
    if (int st = require(nmod)) return st;
    if (n <= 0) return ok(); /* src/blas/dot.cuh:88-90 */
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dot: null array");
    if (gridDim3 <= 0 || blockDim3 <= 0 || blockDim3 > 1024)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_dot: gridDim3 %d / blockDim3 %d out of range", gridDim3, blockDim3);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, (size_t)gridDim3 * mp_size(nmod), ws)) return st;
    cudaError_t e = launch_dot(nmod, n, *x, incx, *y, incy, *r, gridDim3, blockDim3, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_dot");
}

int mpres_dot_noalloc(int nmod, int n, const mp_array_t *x, int incx, const mp_array_t *y, int incy, mp_array_t *r,
                      int gridDim3, int blockDim3, void *stream) {
    if (int st = require(nmod)) return st;
    if (n <= 0) return ok();
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_dot_noalloc: null array");
    if (gridDim3 <= 0 || gridDim3 > MPRES_DOT_NOALLOC_MAX_BLOCKS || blockDim3 <= 0 || blockDim3 > 1024)
        return fail(MPRES_ERR_INVALID_VALUE,
                    "mpres_dot_noalloc: gridDim3 %d must be in 1..%d and blockDim3 %d in 1..1024 (static scratch)",
                    gridDim3, MPRES_DOT_NOALLOC_MAX_BLOCKS, blockDim3);
    Workspace ws;
    cudaError_t e = dot_noalloc_scratch(ws);
    if (e != cudaSuccess) return cuda_fail(e, "mpres_dot_noalloc: scratch address");
    e = launch_dot(nmod, n, *x, incx, *y, incy, *r, gridDim3, blockDim3, ws, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_dot_noalloc");
}

int mpres_gemv(int nmod, int trans, int m, int n, const mp_array_t *alpha, const mp_array_t *A, int lda,
               const mp_array_t *x, int incx, const mp_array_t *beta, mp_array_t *y, int incy, mp_array_t *buffer1,
               mp_array_t *buffer2, int gridDim1, int blockDim1, int gridDim2, int blockDim3, void *stream) {
    (void)buffer1; (void)buffer2; (void)gridDim1; (void)blockDim1; (void)gridDim2;
    if (int st = require(nmod)) return st;
    /* src/blas/gemv.cuh:155-161 */
    if (m <= 0 || n <= 0) return ok();
    if (incx == 0 || incy == 0 || lda < (m > 1 ? m : 1)) return ok();
    if (!alpha || !A || !x || !beta || !y) return fail(MPRES_ERR_INVALID_VALUE, "mpres_gemv: null array");
    if (blockDim3 <= 0 || blockDim3 > 1024)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_gemv: blockDim3 %d out of range", blockDim3);
    const bool tr = (trans != MPRES_NO_TRANS);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, (size_t)(tr ? m : n) * mp_size(nmod), ws)) return st;
    cudaError_t e = launch_gemv(nmod, tr, m, n, *alpha, *A, lda, *x, incx, *beta, *y, incy, blockDim3, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_gemv");
}

int mpres_gemm(int nmod, int transa, int transb, int m, int n, int k, const mp_array_t *alpha, const mp_array_t *A,
               int lda, const mp_array_t *B, int ldb, const mp_array_t *beta, mp_array_t *C, int ldc,
               mp_array_t *buffer, int blockDim1x, int blockDim1y, int gridDim2x, int gridDim2y, int blockDim3,
               void *stream) {
    (void)buffer; (void)blockDim1x; (void)blockDim1y; (void)gridDim2x; (void)gridDim2y; (void)blockDim3;
    if (int st = require(nmod)) return st;
    /* src/blas/gemm.cuh:77-96 */
    if (m <= 0 || n <= 0 || k <= 0) return ok();
    if (transa == MPRES_NO_TRANS && lda < (m > 1 ? m : 1)) return ok();
    if (transa == MPRES_TRANS && lda < (k > 1 ? k : 1)) return ok();
    if (transb == MPRES_NO_TRANS && ldb < (k > 1 ? k : 1)) return ok();
    if (transb == MPRES_TRANS && ldb < (n > 1 ? n : 1)) return ok();
    if (ldc < (m > 1 ? m : 1)) return ok();
    if (transa != MPRES_NO_TRANS || transb != MPRES_NO_TRANS)
        return fail(MPRES_ERR_NOT_SUPPORTED, "mpres_gemm: only non-transposed matrices are supported");
    if (!alpha || !A || !B || !beta || !C) return fail(MPRES_ERR_INVALID_VALUE, "mpres_gemm: null array");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    /* MPRES_GEMM_NO_SCRATCH=1 selects the step-by-step chain, the path taken when
     * the workspace cannot grow (same bits, no scratch); MPRES_GEMM_NO_SPLIT=1 the
     * tiled lazy chain, taken when it can grow to W(A), W(B) but not to the split
     * form's scratch */
    const char *no_scratch = std::getenv("MPRES_GEMM_NO_SCRATCH");
    const char *no_split = std::getenv("MPRES_GEMM_NO_SPLIT");
    const bool scratch = !(no_scratch && no_scratch[0] == '1');
    const bool allow_split = !(no_split && no_split[0] == '1');
    /* the split form's scratch first (32 moduli), else W(A), W(B) alone */
    const size_t split = scratch && allow_split ? gemm_split_workspace_bytes(nmod, m, n, k) : 0;
    if (scratch && (split == 0 || workspace_grow(s, split, ws) != cudaSuccess) &&
        workspace_grow(s, gemm_workspace_bytes(nmod, m, n, k), ws) != cudaSuccess)
        ws = Workspace{}; /* no room for W(A), W(B): the step-by-step chain, no scratch */
    if (!allow_split && ws.bytes > gemm_workspace_bytes(nmod, m, n, k))
        ws.bytes = gemm_workspace_bytes(nmod, m, n, k); /* a stream's workspace may be larger from earlier calls */
    cudaError_t e = launch_gemm(nmod, m, n, k, *alpha, *A, lda, *B, ldb, *beta, *C, ldc, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_gemm");
}

int mpres_spmv_csr(int nmod, int m, const csr_t *csr, const void *x, void *y, int threads, void *stream) {
    (void)threads;
    if (int st = require(nmod)) return st;
    if (m <= 0) return ok();
    if (!csr || !x || !y) return fail(MPRES_ERR_INVALID_VALUE, "mpres_spmv_csr: null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, spmv_workspace_bytes(m), ws)) return st;
    cudaError_t e = launch_spmv_csr(nmod, m, *csr, x, y, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_spmv_csr");
}

int mpres_spmv_csrv(int nmod, int m, const csr_t *csr, const void *x, void *y, int threads, int threadsPerRow,
                    void *stream) {
    (void)threads;
    if (int st = require(nmod)) return st;
    if (threadsPerRow < 1 || threadsPerRow > 32 || (threadsPerRow & (threadsPerRow - 1)))
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_spmv_csrv: threadsPerRow %d not a power of two <= 32",
                    threadsPerRow);
    if (m <= 0) return ok();
    if (!csr || !x || !y) return fail(MPRES_ERR_INVALID_VALUE, "mpres_spmv_csrv: null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, spmv_workspace_bytes(m), ws)) return st;
    cudaError_t e = launch_spmv_csrv(nmod, m, threadsPerRow, *csr, x, y, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_spmv_csrv");
}

int mpres_spmv_ell(int nmod, int m, int maxnzr, const ell_t *ell, const void *x, void *y, int threads,
                   void *stream) {
    (void)threads;
    if (int st = require(nmod)) return st;
    if (m <= 0) return ok();
    if (maxnzr < 0 || !ell || !x || !y) return fail(MPRES_ERR_INVALID_VALUE, "mpres_spmv_ell: bad argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, spmv_workspace_bytes(m), ws)) return st;
    cudaError_t e = launch_spmv_ell(nmod, m, maxnzr, *ell, x, y, ws, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_spmv_ell");
}

int mpres_elementwise(int nmod, int op, const void *x, const void *y, void *r, size_t count, void *stream) {
    if (int st = require(nmod)) return st;
    if (op != MPRES_OP_ADD && op != MPRES_OP_MUL && op != MPRES_OP_MUL_D)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_elementwise: unknown op %d", op);
    if (count == 0) return ok();
    if (!x || !y || !r) return fail(MPRES_ERR_INVALID_VALUE, "mpres_elementwise: null pointer");
    cudaError_t e = launch_elementwise(nmod, op, x, y, r, (long long)count, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_elementwise");
}

int mpres_probe_check(int which, int nmod, const void *a, const void *b, void *out, size_t count, void *stream) {
    if (int st = require(nmod)) return st;
    if (count == 0) return ok();
    if (!a || !out || (which == 1 && !b)) return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_check: null pointer");
    cudaError_t e = launch_check(which, nmod, a, b, out, (long long)count, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_check");
}

int mpres_probe_chain(int nmod, int kind, const void *x, const void *y, int len, long long *cycles,
                      unsigned *rounds, void *result, void *stream) {
    if (int st = require(nmod)) return st;
    const int k = kind & 0xf, fixed = kind >> 4;
    if (k < 0 || k > 2 || fixed < 0 || fixed > 1 || len <= 0 || !x || (k != 1 && !y) || !cycles || !rounds ||
        !result)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_chain: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = fixed ? launch_chain_probe_fx(nmod, k, x, y, len, cycles, rounds, result, s)
                          : launch_chain_probe_fp64(nmod, k, x, y, len, cycles, rounds, result, s);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_chain");
}

int mpres_probe_rounding(int nmod, const int *digits, const unsigned *D, int count, long long *cycles, int *out,
                         void *stream) {
    if (int st = require(nmod)) return st;
    if (count <= 0 || !digits || !D || !cycles || !out)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_rounding: bad arguments");
    cudaError_t e = launch_round_probe(nmod, digits, D, count, cycles, out, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_rounding");
}

int mpres_probe_fraction_sum(int nmod, int which, const int *digits, long long count, void *result, int *out,
                             void *stream) {
    if (int st = require(nmod)) return st;
    if ((which != 0 && which != 1) || count <= 0 || !digits || !result || (which == 0 && !out))
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_fraction_sum: bad arguments");
    cudaError_t e = launch_psum_probe(nmod, which, digits, count, result, out, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_fraction_sum");
}

int mpres_probe_gemm_phases(int nmod, int m, int n, int k, const mp_array_t *alpha, const mp_array_t *A, int lda,
                            const mp_array_t *B, int ldb, const mp_array_t *beta, mp_array_t *C, int ldc, float *ms,
                            void *stream) {
    if (int st = require(nmod)) return st;
    if (!alpha || !A || !B || !beta || !C || !ms || m <= 0 || n <= 0 || k <= 0 || lda < m || ldb < k || ldc < m)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_gemm_phases: bad arguments");
    if (nmod != 32) return fail(MPRES_ERR_NOT_SUPPORTED, "mpres_probe_gemm_phases: the split form is for 32 moduli");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Workspace ws;
    if (int st = workspace(s, gemm_split_workspace_bytes(nmod, m, n, k), ws)) return st;
    constexpr int P = kGemmSplitPhases;
    cudaEvent_t ev[P + 1] = {};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i <= P && e == cudaSuccess; i++) e = cudaEventCreate(&ev[i]);
    if (e == cudaSuccess) e = launch_gemm_split_marked(nmod, m, n, k, *alpha, *A, lda, *B, ldb, *beta, *C, ldc, ws, s, ev);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[P]);
    for (int i = 0; i < P && e == cudaSuccess; i++) e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    for (int i = 0; i <= P; i++)
        if (ev[i]) cudaEventDestroy(ev[i]);
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_gemm_phases");
}

int mpres_probe_eval_phases(int nmod, const int *digits, int count, long long *cycles, int *out, void *stream) {
    if (int st = require(nmod)) return st;
    if (count <= 0 || !digits || !cycles || !out)
        return fail(MPRES_ERR_INVALID_VALUE, "mpres_probe_eval_phases: bad arguments");
    cudaError_t e = launch_eval_phase_probe(nmod, digits, count, cycles, out, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_probe_eval_phases");
}

int mpres_rns_scale2pow(int nmod, const int *digits, const unsigned *D, int *out, size_t count, void *stream) {
    if (int st = require(nmod)) return st;
    if (count == 0) return ok();
    if (!digits || !D || !out) return fail(MPRES_ERR_INVALID_VALUE, "mpres_rns_scale2pow: null pointer");
    cudaError_t e = launch_scale2pow(nmod, digits, D, out, (long long)count, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_rns_scale2pow");
}

int mpres_rns_eval(int nmod, int fast, const int *digits, void *low, void *upp, size_t count, void *stream) {
    if (int st = require(nmod)) return st;
    if (count == 0) return ok();
    if (!digits || !low || !upp) return fail(MPRES_ERR_INVALID_VALUE, "mpres_rns_eval: null pointer");
    cudaError_t e = launch_eval(nmod, fast, digits, static_cast<er_t *>(low), static_cast<er_t *>(upp),
                                (long long)count, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ok() : cuda_fail(e, "mpres_rns_eval");
}

} // extern "C"
