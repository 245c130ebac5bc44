"""Host-side checks of the CUDA library that need no GPU: it builds for sm_103a,
loads, exports every entry point its header declares, and its host code (the
constant tables and the double -> mp_float_t conversion) matches the reference's
golden vectors and the oracle."""
import ctypes
import re

import numpy as np
import pytest

import helpers
from oracle import ffi

GOLD = helpers.ROOT / "tests" / "golden"


def declared_symbols():
    text = "\n".join(p.read_text() for p in sorted((helpers.ROOT / "include").glob("*.h")))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mpres_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_hot_path():
    syms = declared_symbols()
    for s in ("mpres_init", "mpres_dot", "mpres_gemv", "mpres_gemm", "mpres_spmv_csr", "mpres_spmv_csrv",
              "mpres_spmv_ell", "mpres_array_init", "mpres_array_host2device", "mpres_set_d"):
        assert s in syms


def test_library_exports_every_declared_symbol(library):
    lib = ctypes.CDLL(str(library.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_library_loads_through_binding(library):
    assert library.lib().mpres_mp_float_size(8) == 72
    assert library.lib().mpres_mp_float_size(16) == 104
    assert library.lib().mpres_mp_float_size(32) == 168
    assert library.lib().mpres_mp_float_size(12) == 0


@pytest.mark.parametrize("n", [8, 16, 32])
def test_integer_constants_match_oracle(library, oracle, n):
    c = library.int_constants(n)
    t = oracle.tables(n, helpers.LOG2M[n])
    assert [c["mp_precision"], c["mp_h"], c["mp_j"]] == list(t["mp_consts"])
    assert c["ref_factor"] == int(t["ref_factor"][0])
    assert c["log2m"] == helpers.LOG2M[n]


@pytest.mark.parametrize("n", [8, 16, 32])
def test_host_conversion_matches_golden(library, n):
    g = np.load(GOLD / ("elem_%d.npz" % n))
    for key in ("x", "y"):
        got = library.set_d(n, g[key])
        mm = ffi.mismatches(got, g["m" + key])
        assert len(mm) == 0, mm[:5]


@pytest.mark.parametrize("n", [8, 16, 32])
def test_host_conversion_matches_oracle(library, oracle, n):
    rng = np.random.default_rng(helpers.SEED + 700 + n)
    x = np.concatenate([helpers.doubles(rng, 20000, -1000, 1000), rng.standard_normal(5000),
                        rng.integers(-2 ** 40, 2 ** 40, 3000).astype(np.float64)])
    assert len(ffi.mismatches(library.set_d(n, x), oracle.set_d(n, x))) == 0


def test_unsupported_set_is_an_error(library):
    with pytest.raises(library.MpresError):
        library.set_d(12, np.ones(3))


DRIVER = r"""
#define RNS_MODULI_SIZE 8
#include "mpres_gb300.hpp"
#include <vector>
/* the calling sequence of the reference's benchmark drivers
 * (tests/blas/performance/test_dot_performance.cu, tests/sparse/spmv/csr/test_mpres_spmv_csr.cuh) */
int main() {
    rns_const_init();
    mp_const_init();
    const int n = 1000;
    std::vector<mp_float_t> hx(n), hy(n), hr(1);
    mp_array_t x, y, r, buf;
    cuda::mp_array_init(x, n); cuda::mp_array_init(y, n); cuda::mp_array_init(r, 1); cuda::mp_array_init(buf, n);
    cuda::mp_array_host2device(x, hx.data(), n);
    cuda::mp_array_host2device(y, hy.data(), n);
    cuda::mp_dot<512, 128, 8192, 256, 64>(n, x, 1, y, 1, r, buf);
    cuda::mp_gemv<256, 128, 256, 32>(mblas_no_trans, 10, 100, r, x, 10, y, 1, r, y, 1, buf, buf);
    cuda::mp_gemm<32, 1, 128, 64, 16>(mblas_no_trans, mblas_no_trans, 10, 10, 10, r, x, 10, y, 10, r, x, 10, buf);
    csr_t csr;
    cuda::csr_init(csr, 10, 10);
    cuda::mp_spmv_csr<32>(10, csr, hx.data(), hy.data());
    cuda::mp_spmv_csrv<32, 4>(10, csr, hx.data(), hy.data());
    /* the solver drivers (tests/sparse/solver/*) and their v2 kernels */
    std::vector<double> resvec;
    int it = mp_cg_csr<32, 256>(10, csr, hx.data(), 1e-12, 20, hy.data(), resvec);
    std::vector<double> M(10, 1.0);
    it += mp_pcg_csr<64, 256>(10, csr, hx.data(), 1e-12, 20, diag, M.data(), hy.data(), resvec);
    cuda::mp_axpy(10, hx.data(), hx.data(), hy.data(), hy.data());
    cuda::mp_dot<256, 32>(10, hx.data(), hy.data(), hx.data());
    double nrm = cuda::mp_norm2<256, 32>(10, hx.data()) + mp_dsqrt(hx.data()) + cuda::mp_dsqrt(hx.data());
    mp_div(hx.data(), hx.data(), hy.data());
    cuda::csr_clear(csr);
    /* the Matrix Market reader */
    int m, n2, lines, maxnzr, nzmd;
    bool symm;
    std::string dtype;
    collect_mtx_stats("a.mtx", m, n2, lines, maxnzr, nzmd, symm, dtype);
    build_csr("a.mtx", m, lines, lines, symm, csr);
    cuda::mp_array_device2host(hr.data(), r, 1);
    cuda::mp_array_clear(x);
    return it + (int)nrm;
}
"""


def test_cpp_dropin_header_compiles_and_links(library, tmp_path):
    """A driver written like the reference's own, against include/mpres_gb300.hpp,
    compiles and links with plain g++ (it is not run here: no GPU)."""
    import subprocess
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    lib = library.LIB_PATH
    r = subprocess.run(["g++", "-std=c++17", "-I", str(helpers.ROOT / "include"), str(src), "-o",
                        str(tmp_path / "driver"), str(lib), "-Wl,-rpath," + str(lib.parent)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("n", [8, 32])
def test_tensor_array_upload_copy_download(library, oracle, n):
    """TensorArray.upload / copy_ / download keep mp_float_t records bit for bit
    (the GEMM benchmark restores C with them); torch tensors on the CPU."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(helpers.SEED + 11)
    host = oracle.set_d(n, np.concatenate([helpers.doubles(rng, 37, -40, 40), [0.0, -0.0, 1.0]]))
    a = library.TensorArray(n, len(host), device="cpu")
    a.upload(host)
    b = library.TensorArray(n, len(host), device="cpu")
    b.copy_(a)
    assert a.download().tobytes() == host.tobytes()
    assert b.download().tobytes() == host.tobytes()
    assert torch.equal(a.eval, b.eval)
