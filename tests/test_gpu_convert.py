"""The device conversion double -> mp_float_t against the host conversion (the
reference's mp_set_d with its host interval evaluation), record for record, for
every moduli set: doubles over every binade, both signs, zeros, subnormals, the
benchmark distributions, and values whose evaluation starts just above a power
of two."""
import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu


def _inputs(rng, count):
    bits = rng.integers(0, 1 << 63, count, dtype=np.int64).astype(np.uint64)
    bits |= rng.integers(0, 2, count).astype(np.uint64) << np.uint64(63)
    wild = bits.view(np.float64)
    wild = wild[np.isfinite(wild)]
    edge = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 3.0, 5e-324, -5e-324, 2.0 ** -1022, 2.0 ** -1074 * 3,
                     np.finfo(float).max, -np.finfo(float).max, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0),
                     float(2 ** 53 - 1), -float(2 ** 52 + 1), 1e-300, 1e300])
    powers = np.ldexp(1.0, np.arange(-1074, 1024))
    near = np.concatenate([np.nextafter(powers, np.inf), np.nextafter(powers, 0)])
    near = near[np.isfinite(near)]
    small_int = rng.integers(-(1 << 20), 1 << 20, count // 4).astype(np.float64)
    return np.concatenate([edge, wild, powers, near, small_int,
                           helpers.doubles(rng, count, -16, 16), helpers.doubles(rng, count, -32, 32)])


@pytest.mark.parametrize("n", [8, 16, 32])
def test_device_conversion_matches_host(gpu, n):
    import torch
    rng = np.random.default_rng(helpers.SEED + 960 + n)
    x = _inputs(rng, 200000)
    want = gpu.set_d(n, x)
    got = gpu.set_d_device(n, torch.from_numpy(x).cuda()).to_numpy(want.dtype, len(x))
    mm = ffi.mismatches(got, want)
    assert len(mm) == 0, "%d of %d records differ, first x = %r" % (len(mm), len(x), float(x[mm[0]]))


@pytest.mark.parametrize("n", [8, 32])
def test_array_conversion_at_offset(gpu, n):
    import torch
    rng = np.random.default_rng(helpers.SEED + 970 + n)
    x = helpers.doubles(rng, 5000, -40, 40)
    host = gpu.set_d(n, rng.uniform(-1, 1, 12000))
    arr = gpu.DeviceArray.from_host(n, host)
    gpu.array_set_d(n, arr, 3000, torch.from_numpy(x).cuda())
    torch.cuda.synchronize()
    got = arr.download()
    want = host.copy()
    want[3000:8000] = gpu.set_d(n, x)
    assert len(ffi.mismatches(got, want)) == 0
    with pytest.raises(gpu.MpresError):
        gpu.array_set_d(n, arr, 10000, torch.from_numpy(x).cuda())
