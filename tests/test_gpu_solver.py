"""Conjugate gradients and the v2 vector kernels on the GPU against the
reference's own results (golden vectors made by the reference compiled for the
CPU): mp_add_abs through the sum of squares, the v2 dot and norm, axpy / maxpy /
diff, and mp_cg_csr / mp_pcg_csr -- solution records and residual history bit
for bit."""
import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu
GOLD = helpers.ROOT / "tests" / "golden"


def eq(a, b, what=""):
    mm = ffi.mismatches(a, b)
    assert len(mm) == 0, "%s: %d of %d records differ" % (what, len(mm), len(b))


@pytest.mark.parametrize("n", [8, 16])
def test_v2_reductions_match_reference(gpu, n):
    g = np.load(GOLD / ("v2_%d.npz" % n))
    x, y = gpu.DeviceBytes.from_numpy(g["x"]), gpu.DeviceBytes.from_numpy(g["y"])
    r = gpu.DeviceBytes(4 * n + 40)
    for blocks, threads in ((256, 32), (256, 64), (7, 33)):
        gpu.v2_dot(n, len(g["x"]), x, y, r, blocks, threads)
        eq(r.to_numpy(g["x"].dtype, 1), g["dot_%d_%d" % (blocks, threads)], "dot")
        nrm = gpu.v2_norm2(n, len(g["x"]), x, blocks, threads)
        want = gpu.dsqrt(n, g["sumsq_%d_%d" % (blocks, threads)])[0]
        assert nrm == want


def test_v2_vector_kernels_match_oracle(gpu, oracle):
    import torch
    n = 8
    rng = np.random.default_rng(helpers.SEED + 220)
    xs, ys = oracle.set_d(n, helpers.doubles(rng, 5000, -20, 20)), oracle.set_d(n, helpers.doubles(rng, 5000, -20, 20))
    al = oracle.set_d(n, rng.uniform(-1, 1, 1))
    x, y, a = gpu.DeviceBytes.from_numpy(xs), gpu.DeviceBytes.from_numpy(ys), gpu.DeviceBytes.from_numpy(al)
    r = gpu.DeviceBytes(xs.nbytes)
    neg = ys.copy()
    neg["sign"] ^= 1
    cases = {"diff": oracle.add(n, xs, neg), "axpy": oracle.add(n, oracle.mul(n, np.repeat(al, 5000), xs), ys)}
    mal = al.copy()
    mal["sign"] ^= 1
    cases["maxpy"] = oracle.add(n, oracle.mul(n, np.repeat(mal, 5000), xs), ys)
    for op, want in cases.items():
        gpu.v2_vec(n, op, 5000, x, y, r, alpha=a)
        torch.cuda.synchronize()
        eq(r.to_numpy(xs.dtype, 5000), want, op)


@pytest.mark.parametrize("kind", ["cg", "pcg"])
def test_cg_matches_reference(gpu, kind):
    import torch
    g = np.load(GOLD / "cg_8.npz")
    m = len(g["irp"]) - 1
    csr = gpu.DeviceCsr(m, g["irp"], g["ja"], g["vals"])
    b = gpu.DeviceBytes.from_numpy(g["b"])
    x = gpu.DeviceBytes.from_numpy(g["x0"])
    M = gpu.DeviceBytes.from_numpy(g["M"]) if kind == "pcg" else None
    k, res = gpu.cg_csr(8, m, csr, b, x, 1e-30, 40, M=M)
    torch.cuda.synchronize()
    assert k == int(g[kind + "_iters"][0])
    assert res.tobytes() == g[kind + "_res"].tobytes()
    eq(x.to_numpy(g["b"].dtype, m), g[kind + "_x"], kind + " solution")
