"""A C++ driver written like the reference's own benchmark drivers, compiled
against the drop-in header include/mpres_gb300.hpp with plain g++ and run on the
GPU: its mp_dot, mp_gemv, mp_gemm and mp_spmv_csr outputs, read back from files,
are bit-identical to the oracle on the same seeded inputs."""
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu
SRC = helpers.ROOT / "tests" / "native" / "dropin_driver.cpp"


def build_driver(library, tmp_path, n):
    import build
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    cuda = build.cuda_home()
    exe = tmp_path / ("driver%d" % n)
    lib = library.LIB_PATH
    subprocess.run([gxx, "-std=c++17", "-O1", "-DRNS_MODULI_SIZE=%d" % n, "-I", str(helpers.ROOT / "include"),
                    "-I", str(cuda / "include"), str(SRC), "-o", str(exe), str(lib), "-Wl,-rpath," + str(lib.parent),
                    "-L", str(cuda / "lib64"), "-lcudart", "-Wl,-rpath," + str(cuda / "lib64")], check=True)
    return exe


def run(exe, *args):
    r = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_driver_matches_oracle(gpu, oracle, tmp_path):
    rng = np.random.default_rng(helpers.SEED + 808)
    f = lambda name: tmp_path / name  # noqa: E731
    # DOT and SpMV with 8 moduli (their benchmark set), GEMV with 16, GEMM with 32
    exe8, exe16, exe32 = (build_driver(gpu, tmp_path, n) for n in (8, 16, 32))

    n = 8
    cnt = 100003
    mx, my = (gpu.set_d(n, helpers.doubles(rng, cnt, -16, 16)) for _ in range(2))
    mx.tofile(f("x")), my.tofile(f("y"))
    run(exe8, "dot", cnt, f("x"), f("y"), f("r"))
    got = np.fromfile(f("r"), mx.dtype)
    assert got.tobytes() == oracle.dot(n, mx, my, g3=256, b3=64).tobytes()

    m = 20000
    irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m, kmax=300))
    sx = gpu.set_d(n, helpers.doubles(rng, m, -16, 16))
    irp.astype(np.int32).tofile(f("irp")), ja.astype(np.int32).tofile(f("ja")), vals.tofile(f("as"))
    sx.tofile(f("sx"))
    run(exe8, "spmv", m, len(ja), f("irp"), f("ja"), f("as"), f("sx"), f("sy"))
    assert np.fromfile(f("sy"), sx.dtype).tobytes() == oracle.spmv_csr(n, m, irp, ja, vals, sx).tobytes()

    n = 16
    m, k = 300, 517
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -32, 32))
    x, y = gpu.set_d(n, helpers.doubles(rng, k, -32, 32)), gpu.set_d(n, helpers.doubles(rng, m, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    for name, v in (("al", al), ("A", A), ("gx", x), ("be", be), ("gy", y)):
        v.tofile(f(name))
    run(exe16, "gemv", m, k, f("al"), f("A"), f("gx"), f("be"), f("gy"), f("gout"))
    want = oracle.gemv(n, gpu.NO_TRANS, m, k, al, A, m, x, be, y.copy(), b3=32)
    assert np.fromfile(f("gout"), y.dtype).tobytes() == want.tobytes()

    n = 32
    m, cols, k = 130, 70, 200
    A = gpu.set_d(n, helpers.doubles(rng, m * k, -32, 32))
    B = gpu.set_d(n, helpers.doubles(rng, k * cols, -32, 32))
    C = gpu.set_d(n, helpers.doubles(rng, m * cols, -32, 32))
    al, be = gpu.set_d(n, rng.uniform(-1, 1, 1)), gpu.set_d(n, rng.uniform(-1, 1, 1))
    for name, v in (("mal", al), ("mA", A), ("mB", B), ("mbe", be), ("mC", C)):
        v.tofile(f(name))
    run(exe32, "gemm", m, cols, k, f("mal"), f("mA"), f("mB"), f("mbe"), f("mC"), f("mout"))
    want = oracle.gemm(n, m, cols, k, al, A, m, B, k, be, C.copy(), m)
    assert np.fromfile(f("mout"), C.dtype).tobytes() == want.tobytes()
