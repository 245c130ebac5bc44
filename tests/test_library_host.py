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
