"""The serving loop: mixed GEMV / DOT / SpMV requests submitted in bursts and
one by one, admitted under an HBM budget and batched while others run.  Every
result must equal the plain call's alone (bit for bit), the budget must hold at
every moment, and a request that can never fit must fail cleanly."""
import time

import numpy as np
import pytest

import helpers
from oracle import ffi

pytestmark = pytest.mark.gpu

N = 8


def _requests(gpu, rng, count):
    reqs = []
    for i in range(count):
        kind = ("gemv", "dot", "spmv")[i % 3]
        if kind == "gemv":
            m, n = (int(v) for v in np.exp(rng.uniform(np.log(32), np.log(700), 2)))
            reqs.append(dict(kind=kind, m=m, n=n, A=gpu.set_d(N, helpers.doubles(rng, m * n, -32, 32)),
                             x=gpu.set_d(N, helpers.doubles(rng, n, -32, 32)), y=gpu.set_d(N, helpers.doubles(rng, m, -32, 32)),
                             alpha=gpu.set_d(N, rng.uniform(-1, 1, 1)), beta=gpu.set_d(N, rng.uniform(-1, 1, 1))))
        elif kind == "dot":
            n = int(np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 16))))
            reqs.append(dict(kind=kind, n=n, x=gpu.set_d(N, helpers.doubles(rng, n, -16, 16)),
                             y=gpu.set_d(N, helpers.doubles(rng, n, -16, 16)), r=gpu.set_d(N, np.zeros(1))))
        else:
            m = int(np.exp(rng.uniform(np.log(1 << 9), np.log(1 << 13))))
            irp, ja, vals = helpers.random_csr(rng, m, m, helpers.power_law_rows(rng, m))
            reqs.append(dict(kind=kind, m=m, irp=irp, ja=ja, vals=vals, x=gpu.set_d(N, helpers.doubles(rng, m, -16, 16))))
    return reqs


def _device(gpu, r):
    d = dict(r)
    if r["kind"] == "gemv":
        for k in ("A", "x", "y", "alpha", "beta"):
            d[k] = gpu.DeviceArray.from_host(N, r[k])
    elif r["kind"] == "dot":
        for k in ("x", "y", "r"):
            d[k] = gpu.DeviceArray.from_host(N, r[k])
    else:
        d["csr"] = gpu.DeviceCsr(r["m"], r["irp"], r["ja"], r["vals"])
        d["x"] = gpu.DeviceBytes.from_numpy(r["x"])
        d["y"] = gpu.DeviceBytes(r["m"] * (4 * N + 40))
    return d


def _result(gpu, d):
    if d["kind"] == "gemv":
        return d["y"].download()
    if d["kind"] == "dot":
        return d["r"].download()
    return d["y"].to_numpy(gpu.mp_dtype(N), d["m"])


def _alone(gpu, r):
    import torch
    d = _device(gpu, r)
    if r["kind"] == "gemv":
        gpu.gemv(N, gpu.NO_TRANS, r["m"], r["n"], d["alpha"], d["A"], r["m"], d["x"], d["beta"], d["y"])
    elif r["kind"] == "dot":
        gpu.dot(N, r["n"], d["x"], d["y"], d["r"])
    else:
        gpu.spmv_csr(N, r["m"], d["csr"], d["x"], d["y"])
    torch.cuda.synchronize()
    return _result(gpu, d)


def _submit(srv, d):
    if d["kind"] == "gemv":
        return srv.submit_gemv(111, d["m"], d["n"], d["alpha"], d["A"], d["m"], d["x"], d["beta"], d["y"])
    if d["kind"] == "dot":
        return srv.submit_dot(d["n"], d["x"], d["y"], d["r"])
    return srv.submit_spmv_csr(d["m"], d["m"], d["csr"], d["x"], d["y"])


def test_mixed_requests_match_plain_calls(gpu):
    rng = np.random.default_rng(helpers.SEED + 4)
    reqs = _requests(gpu, rng, 60)
    want = [_alone(gpu, r) for r in reqs]
    devs = [_device(gpu, r) for r in reqs]
    srv = gpu.Server(N, budget_bytes=256 << 20, slots=3, max_batch_ops=16)
    ids = []
    for i, d in enumerate(devs):  # bursts of 10, then a pause
        ids.append(_submit(srv, d))
        if i % 10 == 9:
            time.sleep(0.002)
    srv.drain()
    st = srv.stats()
    t = srv.times(0, len(ids))
    srv.destroy()
    for r, d, w in zip(reqs, devs, want):
        got = _result(gpu, d)
        assert len(ffi.mismatches(got, w)) == 0, r["kind"]
    assert st["done"] == len(reqs) and st["errors"] == 0
    assert st["mean_batch"] > 1.0  # arrivals were batched
    assert st["peak_bytes"] <= 256 << 20
    assert (t[:, 0] <= t[:, 1]).all() and (t[:, 1] <= t[:, 2]).all()
    assert 0 < st["p50_s"] <= st["p99_s"]


def test_budget_serialises_and_rejects(gpu):
    rng = np.random.default_rng(helpers.SEED + 5)
    r = dict(kind="dot", n=20000, x=gpu.set_d(N, helpers.doubles(rng, 20000, -16, 16)),
             y=gpu.set_d(N, helpers.doubles(rng, 20000, -16, 16)), r=gpu.set_d(N, np.zeros(1)))
    want = _alone(gpu, r)
    one = 72 * (2 * 20000 + 257)  # the bytes the server counts for this request
    srv = gpu.Server(N, budget_bytes=one + 1000, slots=4, max_batch_ops=8)
    devs = [_device(gpu, r) for _ in range(5)]
    ids = [_submit(srv, d) for d in devs]
    big = dict(kind="dot", n=40000, x=gpu.set_d(N, helpers.doubles(rng, 40000, -16, 16)),
               y=gpu.set_d(N, helpers.doubles(rng, 40000, -16, 16)), r=gpu.set_d(N, np.zeros(1)))
    bid = _submit(srv, _device(gpu, big))
    for i in ids:
        srv.wait(i, 30.0)
    with pytest.raises(gpu.MpresError):
        srv.wait(bid, 30.0)
    st = srv.stats()
    assert st["peak_bytes"] <= one + 1000 and st["batches"] == 5  # one request at a time
    with pytest.raises(gpu.MpresError):
        srv.destroy()  # reports the failed request
    for d in devs:
        assert len(ffi.mismatches(_result(gpu, d), want)) == 0


def test_cancel_and_timeout(gpu):
    """A request withdrawn while it waits for admission completes as cancelled
    with its output untouched; waiting with a short limit on a request stuck
    behind a long one times out; everything else still completes."""
    rng = np.random.default_rng(helpers.SEED + 6)
    big = dict(kind="gemv", m=1500, n=1500, A=gpu.set_d(N, helpers.doubles(rng, 1500 * 1500, -32, 32)),
               x=gpu.set_d(N, helpers.doubles(rng, 1500, -32, 32)), y=gpu.set_d(N, helpers.doubles(rng, 1500, -32, 32)),
               alpha=gpu.set_d(N, rng.uniform(-1, 1, 1)), beta=gpu.set_d(N, rng.uniform(-1, 1, 1)))
    small = [dict(kind="dot", n=4096, x=gpu.set_d(N, helpers.doubles(rng, 4096, -16, 16)),
                  y=gpu.set_d(N, helpers.doubles(rng, 4096, -16, 16)), r=gpu.set_d(N, np.zeros(1))) for _ in range(4)]
    want = [_alone(gpu, r) for r in small]
    srv = gpu.Server(N, budget_bytes=1 << 30, slots=1, max_batch_ops=1)  # one request at a time
    bd = _device(gpu, big)
    devs = [_device(gpu, r) for r in small]
    ids = [_submit(srv, bd)] + [_submit(srv, d) for d in devs]
    cancelled = srv.cancel(ids[-1])
    with pytest.raises(gpu.MpresError):
        srv.wait(ids[-2], 1e-4)  # still behind the GEMV
    for i, d, w in zip(ids[1:], devs, want):
        if i == ids[-1] and cancelled:
            with pytest.raises(gpu.MpresError, match="cancelled"):
                srv.wait(i, 60.0)
            assert len(ffi.mismatches(_result(gpu, d), small[-1]["r"])) == 0  # untouched
        else:
            srv.wait(i, 60.0)
            assert len(ffi.mismatches(_result(gpu, d), w)) == 0
    srv.wait(ids[0], 60.0)
    srv.destroy()
