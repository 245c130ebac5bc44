"""mpres_dot_noalloc: the mp_dot entry point for callers that must not allocate
device memory after start-up (a serving process holding the whole device under
a fixed budget, a host whose own allocator owns the GPU, a loop that cannot take
cudaFree's device-wide synchronisation).  Through the C ABI, two calls in a row
must give exactly what mpres_dot gives for the same summation order, and must
leave the device's free memory unchanged.  Runs last (file name) so that a
stop-at-first-failure run has done every other test first; it also passes alone
in a fresh process."""
import ctypes

import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu


def _call_noalloc(lib, n, count, x, y, r, g3, b3):
    return lib.lib().mpres_dot_noalloc(n, count, x.ref, 1, y.ref, 1, r.ref, g3, b3, None)


# (moduli, count, gridDim3, blockDim3); the last case of the 32-moduli set
# writes all 4096 block sums of the largest record size, the whole static array
CASES = {
    8: [(200000, 256, 64), (77777, 4096, 32)],
    16: [(120001, 256, 64), (50000, 1000, 128)],
    32: [(60013, 96, 32), (200000, 4096, 1024)],
}


@pytest.mark.parametrize("n", [8, 16, 32])
def test_dot_noalloc_matches_dot_twice(gpu, n):
    import torch
    rng = np.random.default_rng(helpers.SEED + 4242 + n)
    data = []
    for count, g3, b3 in CASES[n]:
        mx = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
        my = gpu.set_d(n, helpers.doubles(rng, count, -16, 16))
        x, y = gpu.DeviceArray.from_host(n, mx), gpu.DeviceArray.from_host(n, my)
        want = gpu.DeviceArray(n, 1)
        gpu.dot(n, count, x, y, want, order=(1, 1, 1, g3, b3))  # the allocating entry point
        data.append((count, g3, b3, x, y, want.download()))
    torch.cuda.synchronize()
    for count, g3, b3, x, y, want in data:  # two calls in a row, different orders and sizes
        r = gpu.DeviceArray(n, 1)
        free_call = torch.cuda.mem_get_info()[0]
        gpu.check(_call_noalloc(gpu, n, count, x, y, r, g3, b3), "mpres_dot_noalloc")
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_call
        got = r.download()
        assert len(ffi.mismatches(got, want)) == 0
        r.free()


def test_dot_noalloc_rejects_grid_beyond_scratch(gpu):
    n = 8
    rec = gpu.set_d(n, np.ones(16))
    x = gpu.DeviceArray.from_host(n, rec)
    r = gpu.DeviceArray(n, 1)
    rc = _call_noalloc(gpu, n, 16, x, x, r, 4097, 64)
    assert rc == 1  # MPRES_ERR_INVALID_VALUE
    assert b"static scratch" in gpu.lib().mpres_last_error()
