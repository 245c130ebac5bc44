#!/usr/bin/env python3
"""Benchmark of the RNS multiple-precision hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on stdout.  The headline workload is plain mp_gemm,
C = alpha*A*B + beta*C with m = n = k = 1024, column-major, 32 moduli, entries
u*2^e (u ~ U(-1,1), e ~ U{-32..32}), alpha, beta ~ U(-1,1); a step is one
mp_gemm call.  `value` is MP ops/s (one MP op = one multiple-precision multiply
or add; a GEMM step is 2*m*n*k + 3*m*n of them) with operands resident in HBM;
`e2e` is the same metric through the C ABI from host mp_float_t buffers in
pinned memory: every step uploads A, B and C (mp_array_host2device), runs
mp_gemm and downloads the product C (mp_array_device2host).  The line also
carries plain mp_dot (n = 2^20, 8 moduli) and mp_spmv_csr / csrv (tpr 4, 16,
32) / ell (2^20 rows, power-law row lengths, 8 moduli), each with its
roofline, e2e and CPU baselines, the batched GEMV form and the serving loop.

CPU baselines, timed on this host's cores on bounded samples of the same
workloads: `cpu_baseline` is the reference's own CPU path, its MPFR loops with
OpenMP at MP_PRECISION bits (oracle/mpfr_blas.c: mpfr_gemm, mpfr_dot,
mpfr_mpspmv_csr), kind "mpfr"; `cpu_baseline_port` is the oracle's C
restatement of the reference's multiple-precision arithmetic (the host
mp_float_t loop), kind "port".

--impl reference times the reference's CPU path for the headline workload (the
MPFR mpfr_gemm loop on all host cores, a bounded block of C per step; the port
where the host has no MPFR runtime).  It loads nothing of the CUDA library.

Multi-GPU (torchrun): the path does not shard (a GEMM's outputs are independent
but the benchmark does not split one); every rank runs an independent replica
and `value` is the sum of all ranks' work over the slowest rank's time.
"""
import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
PKG = ROOT / "mpres-blas_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

from workloads import doubles, power_law_rows, random_csr  # noqa: E402

METRIC = "MP ops/s (DOT,GEMM,SpMV) & batched-vs-plain speedup, bit-exact; p50/p99 lat"
SEED = 0x4D505245


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic(kernel, algo_bytes=None):
    """DRAM bytes (read + write) per launch of a kernel at the benchmark size, from
    the committed ncu capture (profiles/ncu_traffic.json); for a capture of a
    smaller case, scaled by algorithmic bytes when algo_bytes is given.  None if
    the kernel was not captured."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    e = json.loads(p.read_text()).get("kernels", {}).get(kernel)
    if not e:
        return None
    if algo_bytes is not None:
        return e["bytes_per_launch"] / e["algorithmic_bytes"] * algo_bytes if e.get("algorithmic_bytes") else None
    return e["bytes_per_launch"]


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as td
    dev = "cpu" if td.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def replica_rate(work_per_rank, secs, world):
    """Whole-job throughput of `world` independent replicas that each did
    work_per_rank units: all ranks' work over the slowest rank's time."""
    return world * work_per_rank / max_over_ranks(secs, world)


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


# --------------------------------------------------------------- workloads --

def gemm_doubles(m=1024):
    """The headline GEMM's seeded entries as doubles (A, B, C, alpha, beta)."""
    rng = np.random.default_rng(SEED + 1)
    d = {k: doubles(rng, m * m, -32, 32) for k in ("A", "B", "C")}
    d["alpha"] = rng.uniform(-1, 1, 1)
    d["beta"] = rng.uniform(-1, 1, 1)
    return d


def gemm_inputs(set_d, n=32, m=1024):
    """mp_float_t records of the headline GEMM, converted by set_d(n, doubles)
    (the library's host mp_set_d, or the oracle's in the reference arm)."""
    src = gemm_doubles(m)
    return {k: set_d(n, v) for k, v in src.items()}, src


def time_steps(torch, stream, fn, steps, warmup, world):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    stop.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    return start.elapsed_time(stop) / 1000.0


def probe_rates(torch, mp, stream):
    """Barrett-mulmod and directed-add throughput of this GPU (issue-bound microkernels)."""
    sink = torch.zeros(16, dtype=torch.uint8, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    out = {}
    for name, fn in (("mulmod", mp.lib().mpres_probe_mulmod), ("dadd_rd", mp.lib().mpres_probe_dadd)):
        it = iters if name == "mulmod" else iters // 16
        mp.check(fn(blocks, threads, it, sink.data_ptr(), stream.cuda_stream), "probe")
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        mp.check(fn(blocks, threads, it, sink.data_ptr(), stream.cuda_stream), "probe")
        e.record(stream)
        torch.cuda.synchronize()
        out[name] = blocks * threads * it * 8 / (s.elapsed_time(e) / 1000.0)
    return out


def gemm_roofline(torch, mp, stream, d, c_work, c_init, clocks, step_secs, rates, reps=3):
    """Roofline of the dominant kernel of mp_gemm's split form, the scalar
    chain: its launch timed live (mpres_probe_gemm_phases, events between the
    launches of one call, mean of `reps` calls on the same inputs), against
    the SMs' instruction issue rate at the SM clock sampled during the timed
    steps.  The kernel's work per launch is its warp instruction count for this
    workload, from the committed ncu capture (profiles/ncu_traffic.json): the
    kernel is bound by its integer pipe, and its interval arithmetic has no
    HBM or tensor bound."""
    m, n = 1024, 32
    phases = None
    for _ in range(reps):
        with torch.cuda.stream(stream):
            c_work.copy_(c_init)
        ph = mp.probe_gemm_phases(n, m, m, m, d["alpha"], d["A"], m, d["B"], m, d["beta"], c_work, m, stream=stream)
        phases = ph if phases is None else {k: phases[k] + ph[k] for k in ph}
    phases = {k: v / reps for k, v in phases.items()}
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or 2070.0
    peak = 4.0 * sms * mhz * 1e6  # warp instructions issued per second: four schedulers an SM
    entry = json.loads((ROOT / "profiles" / "ncu_traffic.json").read_text())["kernels"].get("gemm_scalar_chain", {}) \
        if (ROOT / "profiles" / "ncu_traffic.json").exists() else {}
    inst = entry.get("warp_instructions_per_launch")
    t = phases["scalar_chain"] / 1e3
    achieved = inst / t if inst else None
    # the second kernel, the modular product, is a bf16 tensor-core kernel: its limb products against the
    # measured cuBLAS bf16 rate (it runs the legacy mma.sync path)
    mp_path = ROOT / "MEASURED_PEAKS.json"
    bf16 = json.loads(mp_path.read_text()).get("bf16_tflops") if mp_path.exists() else None
    prod_flop = 16.0 * n * 2.0 * m ** 3
    t_prod = phases["residue_product"] / 1e3
    product = {"kernel": "gemm_mma_product", "bound": "tensor", "unit": "TFLOP/s", "achieved": prod_flop / t_prod / 1e12,
               "peak": bf16 or 1900.0, "peak_source": "measured" if bf16 else "fallback",
               "frac": prod_flop / t_prod / 1e12 / (bf16 or 1900.0), "kernel_ms": phases["residue_product"],
               "work": "16 bf16 limb products per modulus, %.2f TFLOP" % (prod_flop / 1e12)}
    return {"bound": "int", "kernel": "gemm_scalar_chain", "achieved": achieved / 1e9 if achieved else None,
            "peak": peak / 1e9, "unit": "G warp-instructions/s", "frac": achieved / peak if achieved else None,
            "traffic": entry.get("bytes_per_launch"), "kernel_ms": phases["scalar_chain"],
            "share_of_step": t / step_secs, "phases_ms": phases,
            "alu_pipe_active": entry.get("alu_pipe_active"), "product": product,
            "peak_source": "4 warp instructions per cycle per SM x %d SMs x the sampled SM clock" % sms,
            "work_note": "a split-form step: W(A), W(B) and their bf16 limb planes; the scalar chain (sign, "
                         "exponent and interval of every k step, the reference's expressions); the residues as one "
                         "modular product W(A) x W(B) per modulus on the tensor cores (16 limb products, %.2f TFLOP "
                         "of bf16 mma.sync); the epilogue" % (16 * n * 2 * m ** 3 / 1e12),
            "mulmod_peak_G": rates["mulmod"] / 1e9, "fp64_dadd_rd_peak_G": rates["dadd_rd"] / 1e9}


def gemm_config(world):
    """The headline workload, named identically by both arms."""
    return {"workload": "mp_gemm m=n=k=1024, 32 moduli (params.32_32bit), NN, column-major", "global_batch": 1,
            "seq_len": None, "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (3 x 176 MB)",
            "c_per_step": "every step starts from the same C (device copy in the resident timing, upload in e2e)"}


def pinned_copy(torch, arr):
    """A copy of a host record array in page-locked memory (allocated once,
    outside any timed region), so host<->device copies run at DMA speed."""
    buf = torch.empty(arr.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(arr.dtype)
    buf[...] = arr
    return buf


def e2e_time(torch, fn, steps, warmup, world):
    """Wall seconds (max over ranks) of `steps` calls of fn after `warmup`
    untimed ones; each call is synchronous (uploads, the operation, the read of
    its result), so the host clock brackets the device work."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    barrier(world)
    return max_over_ranks(secs, world)


def bench_gemm(torch, mp, stream, steps, warmup, world, rank, local):
    """C = alpha*A*B + beta*C, m = n = k = 1024, 32 moduli.  Every step starts
    from the same C, as the reference's own benchmark re-uploads C before each
    timed call (tests/blas/performance/test_gemm_performance.cu): C accumulated
    over steps would grow its residue representation by the bits of beta each
    time and make the later steps round in the epilogue.  In the resident timing
    the restore is a device-to-device copy inside the timed region; in e2e C is
    uploaded from the host every step and the product downloaded."""
    n, m = 32, 1024
    host, src = gemm_inputs(mp.set_d, n, m)
    d = {k: mp.DeviceArray.from_host(n, v) for k, v in host.items()}
    c_work, c_init = mp.TensorArray(n, m * m), mp.TensorArray(n, m * m)
    c_init.upload(host["C"])

    def step():
        with torch.cuda.stream(stream):
            c_work.copy_(c_init)
        mp.gemm(n, m, m, m, d["alpha"], d["A"], m, d["B"], m, d["beta"], c_work, m, stream=stream)

    with Clocks(local) as clk:
        secs = time_steps(torch, stream, step, steps, warmup, world)
    secs = max_over_ranks(secs, world)
    ops = 2.0 * m * m * m + 3.0 * m * m
    value = world * ops * steps / secs
    resident_c = c_work.download()
    rates = probe_rates(torch, mp, stream)
    roof = gemm_roofline(torch, mp, stream, d, c_work, c_init, clk.summary(), secs / steps, rates)

    # e2e: host mp_float_t arrays in pinned memory through the C ABI copies,
    # every step: upload A, B, C; mp_gemm into C; download the product
    pinned = {k: pinned_copy(torch, host[k]) for k in ("A", "B", "C")}
    c_out = pinned_copy(torch, host["C"])

    def e2e_step():
        d["A"].upload(pinned["A"])
        d["B"].upload(pinned["B"])
        d["C"].upload(pinned["C"])
        mp.gemm(n, m, m, m, d["alpha"], d["A"], m, d["B"], m, d["beta"], d["C"], m, stream=stream)
        stream.synchronize()
        d["C"].download(out=c_out)

    e2e_secs = e2e_time(torch, e2e_step, steps, 1, world)
    sz = 4 * n + 40
    e2e = {"value": world * ops * steps / e2e_secs, "unit": "MP ops/s", "h2d_bytes_per_step": 3 * m * m * sz,
           "d2h_bytes_per_step": m * m * sz, "steps": steps,
           "result_matches_resident": bool(c_out.tobytes() == resident_c.tobytes())}
    # per step: gemm_prescale for A and for B, the limb planes of each, the scalar chain, the modular product, the
    # epilogue and the per-output chain of the outputs that leave the split form (the restore of C is a torch copy)
    return dict(secs=secs, value=value, roofline=roof, e2e=e2e, clocks=clk.summary(), host=host, src=src,
                launches=8 * steps)


def chain_cycles(mp, n, kind, x, y, length):
    """Per-step SM cycles of one warp's chains run alone (mpres_probe_chain),
    best of three runs, with the steps' rounding counts."""
    best = None
    for _ in range(3):
        cyc, pr, sr, _ = mp.probe_chain(n, kind, x, y, length)
        if best is None or cyc.sum() < best[0].sum():
            best = (cyc, pr, sr)
    return best


def dot_floor(mp, mx, my, count, g3, b3, mhz):
    """Latency floor of mp_dot under the order key (g3, b3): the longest of a
    few warps' 32 chains of count/(g3*b3) fused steps (chains exactly as pass 1
    forms them), then the pass-1 tree, pass 2's chains of g3/b3 additions and
    its tree, at the add-only step latency; SM cycles at `mhz`."""
    K = g3 * b3
    steps = -(-count // K)
    chain = []
    for blk in (0, g3 // 3, (2 * g3) // 3, g3 - 1):
        lanes = blk * b3 + np.arange(32)
        idx = (lanes[:, None] + K * np.arange(steps)[None, :]).ravel()
        ok = idx < count
        idx = np.where(ok, idx, 0)
        cyc, pr, sr = chain_cycles(mp, 8, 0, mx[idx], my[idx], steps)
        fcyc, _, _ = chain_cycles(mp, 8, 0 + mp.PROBE_FIXED_POINT, mx[idx], my[idx], steps)
        chain.append((int(cyc.sum()), float((sr > 0).mean()), float(sr.sum() / (32.0 * steps)), int(fcyc.sum())))
    # additions of partial sums: products summed pairwise, as the trees do
    pr8 = mp.elementwise(8, mp.OP_MUL, mx[: 32 * 64], my[: 32 * 64])
    acyc, _, asr = chain_cycles(mp, 8, 1, pr8, None, 64)
    add_step = float(acyc.mean())
    levels = int(np.ceil(np.log2(max(b3, 2))))
    tree = (levels + -(-g3 // b3) + levels) * add_step
    worst = max(c[0] for c in chain)
    cycles = worst + tree
    return {"floor_ms": cycles / (mhz * 1e3), "chain_cycles_worst_warp": worst, "steps": steps,
            "step_cycles_mean": worst / steps, "add_step_cycles_mean": add_step,
            "warp_steps_with_a_rounding": max(c[1] for c in chain), "lane_rounding_rate": chain[0][2],
            "step_cycles_mean_fixed_point_eval": max(c[3] for c in chain) / steps,
            "sm_mhz": mhz, "method": "mpres_probe_chain: one warp alone, clock64 per step, best of 3; "
                                     "chain of the longest of 4 sampled warps + 2*log2(b3) + g3/b3 add steps"}


def bench_dot(torch, mp, stream, steps, warmup, world, hbm, mhz=None):
    """plain mp_dot, n = 2^20, 8 moduli, the reference benchmark's order
    <512,128,8192,256,64> (tests/blas/performance/test_dot_performance.cu:35-39)."""
    n, count = 8, 1 << 20
    rng = np.random.default_rng(SEED + 0)
    xd, yd = doubles(rng, count, -16, 16), doubles(rng, count, -16, 16)
    mx, my = mp.set_d(n, xd), mp.set_d(n, yd)
    x, y, r = mp.DeviceArray.from_host(n, mx), mp.DeviceArray.from_host(n, my), mp.DeviceArray(n, 1)
    order = (512, 128, 8192, 256, 64)

    def step():
        mp.dot(n, count, x, y, r, order=order, stream=stream)

    secs = max_over_ranks(time_steps(torch, stream, step, steps, warmup, world), world)
    per = secs / steps
    resident_r = r.download()
    algo = 2 * count * (4 * n + 40)
    px, py, pr = pinned_copy(torch, mx), pinned_copy(torch, my), pinned_copy(torch, mx[:1])

    def e2e_step():
        x.upload(px)
        y.upload(py)
        mp.dot(n, count, x, y, r, order=order, stream=stream)
        stream.synchronize()
        r.download(out=pr)

    e2e_secs = e2e_time(torch, e2e_step, steps, 1, world)
    floor = dot_floor(mp, mx, my, count, order[3], order[4], mhz or 2070.0)
    floor["achieved_over_floor"] = per * 1e3 / floor["floor_ms"]
    return {"workload": "mp_dot n=2^20, 8 moduli, order <512,128,8192,256,64>", "value": world * 2 * count / per,
            "chain_floor": floor,
            "unit": "MP ops/s", "ms_per_step": per * 1e3, "steps": steps, "launches": 2 * steps,
            "roofline": {"bound": "hbm", "achieved": algo / per / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": algo / per / 1e9 / hbm, "traffic": traffic("dot_pass1")},
            "e2e": {"value": world * 2 * count * steps / e2e_secs, "unit": "MP ops/s",
                    "h2d_bytes_per_step": 2 * count * (4 * n + 40), "d2h_bytes_per_step": 4 * n + 40,
                    "result_matches_resident": bool(pr.tobytes() == resident_r.tobytes())},
            "data": (xd, yd, mx, my)}


def ell_on_device(torch, mp, m, irp, ja, vals):
    """The ELLPACK form of a CSR matrix built on the device (column-major
    slots col*m + row, zero padded; the reference's build_ell layout)."""
    irp_t = torch.from_numpy(irp.astype(np.int64)).cuda()
    lens = irp_t[1:] - irp_t[:-1]
    maxnzr = int(lens.max().item())
    nnz = int(irp[-1])
    rows = torch.repeat_interleave(torch.arange(m, device="cuda"), lens)
    slot = (torch.arange(nnz, device="cuda") - irp_t[:-1][rows]) * m + rows
    del rows
    ell_ja = torch.zeros(maxnzr * m, dtype=torch.int32, device="cuda")
    ell_ja[slot] = torch.from_numpy(ja).cuda()
    ell_as = torch.zeros(maxnzr * m, dtype=torch.float64, device="cuda")
    ell_as[slot] = torch.from_numpy(vals).cuda()
    del slot
    return mp.DeviceEll.from_tensors(m, maxnzr, ell_ja, ell_as)


def spmv_floor(mp, irp, ja, vals, mx, mhz):
    """Latency floors of the SpMV kernels: a row is one chain (CSR, ELL) or
    tpr lane-strided chains and a log2(tpr)-level tree (CSRV), so no schedule
    finishes before the longest row's chain.  Measured on the warp holding the
    32 longest rows (kind 2 chains, one warp alone), scaled to the longest
    length; CSRV32 on the 32 lane chains of the longest row."""
    lens = np.diff(irp)
    order = np.argsort(lens)[::-1][:32]
    L = int(lens[order].min())
    Lmax = int(lens[order[0]])
    idx = np.concatenate([np.arange(irp[r], irp[r] + L) for r in order])
    cyc, _, sr = chain_cycles(mp, 8, 2, mx[ja[idx]], vals[idx], L)
    step = float(cyc.mean())
    fcyc, _, _ = chain_cycles(mp, 8, 2 + mp.PROBE_FIXED_POINT, mx[ja[idx]], vals[idx], L)
    r0 = int(order[0])
    sub = -(-Lmax // 32)
    lane_idx = np.array([[irp[r0] + l + 32 * t if l + 32 * t < Lmax else irp[r0] + l for t in range(sub)]
                         for l in range(32)]).ravel()
    cyc32, _, _ = chain_cycles(mp, 8, 2, mx[ja[lane_idx]], vals[lane_idx], sub)
    pr8 = mp.elementwise(8, mp.OP_MUL, mx[: 32 * 64], mx[32 * 64: 64 * 64])
    acyc, _, _ = chain_cycles(mp, 8, 1, pr8, None, 64)
    add_step = float(acyc.mean())
    out = {"longest_row": Lmax, "step_cycles_mean": step, "step_cycles_mean_fixed_point_eval": float(fcyc.mean()),
           "warp_steps_with_a_rounding": float((sr > 0).mean()),
           "lane_rounding_rate": float(sr.sum() / (32.0 * L)), "add_step_cycles_mean": add_step, "sm_mhz": mhz,
           "method": "mpres_probe_chain on the warp of the 32 longest rows (one warp alone, best of 3)"}
    out["csr_floor_ms"] = step * Lmax / (mhz * 1e3)
    for tpr in (4, 16):
        out["csrv%d_floor_ms" % tpr] = (step * -(-Lmax // tpr) + np.log2(tpr) * add_step) / (mhz * 1e3)
    out["csrv32_floor_ms"] = (float(cyc32.sum()) + 5 * add_step) / (mhz * 1e3)
    return out


def bench_spmv(torch, mp, stream, steps, warmup, world, hbm, mhz=None):
    """mp_spmv_csr, mp_spmv_csrv (tpr 4, 16, 32) and mp_spmv_ell on one
    2^20-row power-law matrix (row lengths 1..1024, mean 16), x as in the DOT,
    8 moduli.  e2e: every step uploads the matrix (CSR forms; the 12.9 GB ELL
    slots stay resident) and x from pinned host memory and reads y back."""
    n, m = 8, 1 << 20
    rec = 4 * n + 40
    rng = np.random.default_rng(SEED + 2)
    irp, ja, vals = random_csr(rng, m, m, power_law_rows(rng, m))
    xd = doubles(rng, m, -16, 16)
    mx = mp.set_d(n, xd)
    x = mp.DeviceBytes.from_numpy(mx)
    y = mp.DeviceBytes(m * rec)
    csr = mp.DeviceCsr(m, irp, ja, vals)
    nnz = int(irp[-1])
    algo = nnz * 12 + (m + 1) * 4 + 2 * m * rec
    ell = ell_on_device(torch, mp, m, irp, ja, vals)
    algo_ell = m * ell.maxnzr * 12 + 2 * m * rec
    p_irp, p_ja, p_vals = (pinned_copy(torch, v) for v in (irp, ja, vals))
    p_x, p_y = pinned_copy(torch, mx), pinned_copy(torch, mx)
    variants = [("csr", lambda: mp.spmv_csr(n, m, csr, x, y, stream=stream), "spmv_csr_kernel"),
                ("csrv4", lambda: mp.spmv_csrv(n, m, csr, x, y, 4, stream=stream), "spmv_csrv_kernel"),
                ("csrv16", lambda: mp.spmv_csrv(n, m, csr, x, y, 16, stream=stream), "spmv_csrv_kernel"),
                ("csrv32", lambda: mp.spmv_csrv(n, m, csr, x, y, 32, stream=stream), "spmv_csrv_kernel"),
                ("ell", lambda: mp.spmv_ell(n, m, ell, x, y, stream=stream), "spmv_ell_kernel")]
    out = {}
    ref_y = None
    for name, fn, kern in variants:
        secs = max_over_ranks(time_steps(torch, stream, fn, steps, warmup, world), world)
        per = secs / steps
        y_res = y.t[: m * rec].clone()
        is_ell = name == "ell"

        def e2e_step(fn=fn, is_ell=is_ell):
            if not is_ell:
                csr.upload(p_irp, p_ja, p_vals)
            x.t[: m * rec].copy_(torch.from_numpy(p_x.view(np.uint8).reshape(-1)), non_blocking=True)
            torch.cuda.current_stream().synchronize()
            fn()
            stream.synchronize()
            torch.from_numpy(p_y.view(np.uint8).reshape(-1)).copy_(y.t[: m * rec])

        e2e_secs = e2e_time(torch, e2e_step, steps, 1, world)
        a = algo_ell if is_ell else algo
        h2d = m * rec + (0 if is_ell else nnz * 12 + (m + 1) * 4)
        r = {"value": world * 2 * nnz / per, "unit": "MP ops/s", "ms_per_step": per * 1e3, "steps": steps,
             "launches": 4 * steps,
             "roofline": {"bound": "hbm", "achieved": a / per / 1e9, "peak": hbm, "unit": "GB/s",
                          "frac": a / per / 1e9 / hbm, "traffic": traffic(kern) if name in ("csr", "ell") else None},
             "e2e": {"value": world * 2 * nnz * steps / e2e_secs, "unit": "MP ops/s", "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": m * rec,
                     "matrix": "resident (12.9 GB of slots)" if is_ell else "uploaded every step",
                     "result_matches_resident": bool(torch.equal(torch.from_numpy(p_y.view(np.uint8).reshape(-1)),
                                                                 y_res.cpu()))}}
        if is_ell:
            r["maxnzr"] = ell.maxnzr
            r["roofline"]["vs_csr_bytes_frac"] = algo / per / 1e9 / hbm
            r["slots_bytes"] = m * ell.maxnzr * 12
        if name in ("csr", "ell"):
            if ref_y is None:
                ref_y = y_res
            else:
                r["bit_identical_to_csr"] = bool(torch.equal(ref_y, y_res))
        out[name] = r
    ell.free()
    del ell
    torch.cuda.empty_cache()
    floor = spmv_floor(mp, irp, ja, vals, mx, mhz or 2070.0)
    for name, key in (("csr", "csr_floor_ms"), ("csrv4", "csrv4_floor_ms"), ("csrv16", "csrv16_floor_ms"),
                      ("csrv32", "csrv32_floor_ms"), ("ell", "csr_floor_ms")):
        out[name]["achieved_over_floor"] = out[name]["ms_per_step"] / floor[key]
    return {"workload": "mp_spmv 2^20 rows, nnz=%d (power-law 1..1024), 8 moduli" % nnz, "results": out,
            "nnz": nnz, "chain_floor": floor, "data": (irp, ja, vals, xd, mx)}


def device_doubles(torch, gen, count, lo, hi):
    """u * 2^e with u ~ U(-1, 1) and e ~ U{lo..hi}, generated on the device."""
    u = torch.rand(count, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
    e = torch.randint(lo, hi + 1, (count,), generator=gen, device="cuda")
    return torch.ldexp(u, e)


def value_pool(torch, mp, nmod, count, lo, hi, seed):
    """count seeded u*2^e values converted on the device (bit-identical to the
    host conversion); the large operands are filled by random draws from it."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    pool = mp.TensorArray(nmod, count)
    chunk = 1 << 22
    for off in range(0, count, chunk):
        pool.set_d(device_doubles(torch, gen, min(chunk, count - off), lo, hi), off)
    return pool, gen


def fill_from_pool(torch, arr, pool, gen, offset=0, count=None):
    count = arr.size - offset if count is None else count
    chunk = 1 << 25
    for off in range(0, count, chunk):
        c = min(chunk, count - off)
        idx = torch.randint(0, pool.size, (c,), generator=gen, device="cuda")
        arr.gather_from(pool, idx, offset + off)


def log_uniform_ints(rng, shape, lo, hi):
    return np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), shape))), lo, hi).astype(np.int64)


def snapshot(a):
    return [t.clone() for t in (a.digits, a.sign, a.exp, a.eval)]


def restore(a, snap):
    for t, v in zip((a.digits, a.sign, a.exp, a.eval), snap):
        t.copy_(v)


def same(a, snap):
    import torch
    return all(torch.equal(t, v) for t, v in zip((a.digits, a.sign, a.exp, a.eval), snap))


def bench_batched_gemv(torch, mp, stream, hbm, count=4096, wave_bytes=96 << 30):
    """4096 mp_gemv y = alpha*A*x + beta*y (NO_TRANS, lda = m), m and n
    log-uniform in [32, 4096], entries u*2^e with e in [-32, 32], 16 moduli:
    one persistent launch per wave (graph replay, autotuned shape) against the
    4096 plain mpres_gemv calls, both timed with CUDA events with operands
    resident.  A is about 294 GB in all, so the instances run in waves of at
    most wave_bytes of A; every A, x, y is filled with random draws from 2^23
    seeded values converted on the device."""
    n, rec, b3 = 16, 104, 32
    sizes = log_uniform_ints(np.random.default_rng(SEED + 3), (count, 2), 32, 4096)
    pool, gen = value_pool(torch, mp, n, 1 << 23, -32, 32, SEED + 3)
    waves, cur, acc = [], [], 0
    for i, (m, k) in enumerate(sizes):
        b = int(m * k * rec)
        if cur and acc + b > wave_bytes:
            waves.append(cur)
            cur, acc = [], 0
        cur.append(i)
        acc += b
    waves.append(cur)
    t_plain = t_batch = 0.0
    identical, info, commit_s = True, None, 0.0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for w, idx in enumerate(waves):
        M, K = sizes[idx, 0], sizes[idx, 1]
        a_off = np.concatenate([[0], np.cumsum(M * K)])
        x_off = np.concatenate([[0], np.cumsum(K)])
        y_off = np.concatenate([[0], np.cumsum(M)])
        A, X, Y = mp.TensorArray(n, int(a_off[-1])), mp.TensorArray(n, int(x_off[-1])), mp.TensorArray(n, int(y_off[-1]))
        AB = mp.TensorArray(n, 2 * len(idx))
        for arr in (A, X, Y):
            fill_from_pool(torch, arr, pool, gen)
        AB.set_d(torch.rand(2 * len(idx), generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
        ops = [(int(M[j]), int(K[j]), AB.view(2 * j, 1), A.view(int(a_off[j]), int(M[j] * K[j])),
                X.view(int(x_off[j]), int(K[j])), AB.view(2 * j + 1, 1), Y.view(int(y_off[j]), int(M[j])))
               for j in range(len(idx))]
        torch.cuda.synchronize()

        def plain():
            for m, k, al, Av, xv, be, yv in ops:
                mp.gemv(n, mp.NO_TRANS, m, k, al, Av, m, xv, be, yv, order=(256, 128, 256, b3), stream=stream)

        batch = mp.Batch(n)
        for m, k, al, Av, xv, be, yv in ops:
            batch.add_gemv(mp.NO_TRANS, m, k, al, Av, m, xv, be, yv, b3=b3)
        t0 = time.perf_counter()
        batch.commit(mp.BATCH_GRAPH | (mp.BATCH_AUTOTUNE if w == 0 else 0), stream=stream)
        torch.cuda.synchronize()
        commit_s += time.perf_counter() - t0
        if w == 0:
            info = batch.info()
        # both forms timed from the same y; their outputs compared on every wave
        y0 = snapshot(Y)
        batch.run(stream)  # warm (graph upload)
        torch.cuda.synchronize()
        restore(Y, y0)
        torch.cuda.synchronize()
        ev[0].record(stream)
        plain()
        ev[1].record(stream)
        torch.cuda.synchronize()
        yp = snapshot(Y)
        restore(Y, y0)
        torch.cuda.synchronize()
        ev[2].record(stream)
        batch.run(stream)
        ev[3].record(stream)
        torch.cuda.synchronize()
        identical = identical and same(Y, yp)
        del y0, yp
        t_plain += ev[0].elapsed_time(ev[1]) / 1e3
        t_batch += ev[2].elapsed_time(ev[3]) / 1e3
        batch.destroy()
        del A, X, Y, AB, ops
        torch.cuda.empty_cache()
    mk = sizes[:, 0] * sizes[:, 1]
    ops_total = float(np.sum(2 * mk))
    algo = float(np.sum((mk + sizes[:, 1] + 2 * sizes[:, 0]) * rec))
    return {"workload": "4096 x mp_gemv NO_TRANS, m, n log-uniform in [32, 4096], 16 moduli, blockDim3 = 32",
            "value": ops_total / t_batch, "unit": "MP ops/s", "plain_value": ops_total / t_plain,
            "speedup_vs_plain": t_plain / t_batch, "ms_batched": t_batch * 1e3, "ms_plain": t_plain * 1e3,
            "waves": len(waves), "wave_bytes_max": wave_bytes, "launches_batched": 2 * len(waves),
            "launches_plain": 2 * count, "bit_identical_all_waves": identical, "shape": info,
            "commit_s": commit_s,
            "roofline": {"bound": "hbm", "achieved": algo / t_batch / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": algo / t_batch / 1e9 / hbm, "traffic": traffic("batch_kernel", algo)},
            "data": "A, x, y: random draws from 2^23 seeded u*2^e values (e in [-32, 32]) converted on the GPU; "
                    "alpha, beta ~ U(-1, 1)"}


def bench_batched_gemm(torch, mp, stream, count=256):
    """256 mp_gemm C = alpha*A*B + beta*C with m, n, k independently
    log-uniform in [32, 512], 32 moduli, entries u*2^e (e in [-32, 32]): one
    persistent launch (graph replay, autotuned shape, the W(A), W(B) pass
    before it) against the 256 plain mpres_gemm calls, both timed with CUDA
    events from the same C, outputs compared record for record."""
    n = 32
    sizes = log_uniform_ints(np.random.default_rng(SEED + 5), (count, 3), 32, 512)
    pool, gen = value_pool(torch, mp, n, 1 << 22, -32, 32, SEED + 5)
    M, Nc, K = sizes[:, 0], sizes[:, 1], sizes[:, 2]
    a_off = np.concatenate([[0], np.cumsum(M * K)])
    b_off = np.concatenate([[0], np.cumsum(K * Nc)])
    c_off = np.concatenate([[0], np.cumsum(M * Nc)])
    A, B, C = (mp.TensorArray(n, int(o[-1])) for o in (a_off, b_off, c_off))
    for arr in (A, B, C):
        fill_from_pool(torch, arr, pool, gen)
    AB = mp.TensorArray(n, 2 * count)
    AB.set_d(torch.rand(2 * count, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
    ops = [(int(M[j]), int(Nc[j]), int(K[j]), AB.view(2 * j, 1), A.view(int(a_off[j]), int(M[j] * K[j])),
            B.view(int(b_off[j]), int(K[j] * Nc[j])), AB.view(2 * j + 1, 1), C.view(int(c_off[j]), int(M[j] * Nc[j])))
           for j in range(count)]
    torch.cuda.synchronize()

    def plain():
        for m, c, k, al, Av, Bv, be, Cv in ops:
            mp.gemm(n, m, c, k, al, Av, m, Bv, k, be, Cv, m, stream=stream)

    batch = mp.Batch(n)
    for m, c, k, al, Av, Bv, be, Cv in ops:
        batch.add_gemm(m, c, k, al, Av, m, Bv, k, be, Cv, m)
    t0 = time.perf_counter()
    batch.commit(mp.BATCH_GRAPH | mp.BATCH_AUTOTUNE, stream=stream)
    torch.cuda.synchronize()
    commit_s = time.perf_counter() - t0
    c0 = snapshot(C)
    plain()  # warm: workspace growth and attributes
    batch.run(stream)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    t_plain = t_batch = 0.0
    reps = 3
    identical = True
    for _ in range(reps):
        restore(C, c0)
        torch.cuda.synchronize()
        ev[0].record(stream)
        plain()
        ev[1].record(stream)
        torch.cuda.synchronize()
        cp = snapshot(C)
        restore(C, c0)
        torch.cuda.synchronize()
        ev[2].record(stream)
        batch.run(stream)
        ev[3].record(stream)
        torch.cuda.synchronize()
        identical = identical and same(C, cp)
        t_plain += ev[0].elapsed_time(ev[1]) / 1e3 / reps
        t_batch += ev[2].elapsed_time(ev[3]) / 1e3 / reps
        del cp
    info = batch.info()
    batch.destroy()
    ops_total = float(np.sum(2.0 * M * Nc * K + 3.0 * M * Nc))
    return {"workload": "256 x mp_gemm NN, m, n, k log-uniform in [32, 512], 32 moduli", "value": ops_total / t_batch,
            "unit": "MP ops/s", "plain_value": ops_total / t_plain, "speedup_vs_plain": t_plain / t_batch,
            "ms_batched": t_batch * 1e3, "ms_plain": t_plain * 1e3, "launches_batched": 2, "launches_plain": 8 * count,
            "bit_identical": identical, "shape": info, "commit_s": commit_s,
            "data": "A, B, C: random draws from 2^22 seeded u*2^e values (e in [-32, 32]) converted on the GPU; "
                    "alpha, beta ~ U(-1, 1)"}


def bench_serving(torch, mp, rates=(100.0, 400.0, 1600.0), duration=1.5, budget=64 << 30):
    """Poisson request streams mixing mp_dot (n log-uniform 2^10..2^22),
    mp_gemv (m, n log-uniform 32..4096) and mp_spmv_csr (rows log-uniform
    2^12..2^20, power-law rows), 8 moduli, operands resident, through the
    serving loop (64 GB budget, 4 batches in flight).  Each request draws one
    of a pool of resident operand sets of its kind; GEMV and DOT outputs are
    its own.  Reports per offered rate: throughput, p50 / p99 latency."""
    n, rec = 8, 72
    rng = np.random.default_rng(SEED + 4)
    pool, gen = value_pool(torch, mp, n, 1 << 22, -16, 16, SEED + 4)
    dots = []
    for cnt in log_uniform_ints(rng, 8, 1 << 10, 1 << 22):
        x, y = mp.TensorArray(n, int(cnt)), mp.TensorArray(n, int(cnt))
        fill_from_pool(torch, x, pool, gen)
        fill_from_pool(torch, y, pool, gen)
        dots.append((int(cnt), x, y))
    gemvs = []
    for m, k in log_uniform_ints(rng, (8, 2), 32, 4096):
        A, x, y0 = mp.TensorArray(n, int(m * k)), mp.TensorArray(n, int(k)), mp.TensorArray(n, int(m))
        for a in (A, x, y0):
            fill_from_pool(torch, a, pool, gen)
        ab = mp.TensorArray(n, 2)
        ab.set_d(torch.rand(2, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
        gemvs.append((int(m), int(k), A, x, y0, ab))
    spmvs = []
    for m in log_uniform_ints(rng, 4, 1 << 12, 1 << 20):
        m = int(m)
        irp, ja, vals = random_csr(rng, m, m, power_law_rows(rng, m))
        xs = mp.TensorArray(n, m)  # x as AoS records (mp_float_t*) for the CSR kernel
        fill_from_pool(torch, xs, pool, gen)
        xa = mp.DeviceBytes.from_numpy(xs.download())
        spmvs.append((m, int(irp[-1]), mp.DeviceCsr(m, irp, ja, vals), xa, mp.DeviceBytes(m * rec)))
    torch.cuda.synchronize()
    results = []
    checks = []
    for rate in rates:
        count = max(60, int(rate * duration))
        kinds = rng.integers(0, 3, count)
        picks = rng.integers(0, 8, count)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
        outs_r = mp.TensorArray(n, count)
        gy_len = [gemvs[p][0] if k == 1 else 0 for k, p in zip(kinds, picks)]
        gy_off = np.concatenate([[0], np.cumsum(gy_len)])
        outs_y = mp.TensorArray(n, max(1, int(gy_off[-1])))
        for i in range(count):  # every GEMV request starts from its operand set's y
            if kinds[i] == 1:
                y0 = gemvs[picks[i]][4]
                outs_y.gather_from(y0, torch.arange(y0.size, device="cuda"), int(gy_off[i]))
        y_init = snapshot(outs_y)
        torch.cuda.synchronize()
        srv = mp.Server(n, budget, slots=4, max_batch_ops=64)
        ops_total = 0.0
        t_start = time.perf_counter()
        for i in range(count):
            while time.perf_counter() - t_start < arrivals[i]:
                pass
            k, p = int(kinds[i]), int(picks[i])
            if k == 0:
                cnt, x, y = dots[p]
                srv.submit_dot(cnt, x, y, outs_r.view(i, 1))
                ops_total += 2.0 * cnt
            elif k == 1:
                m, kk, A, x, _, ab = gemvs[p]
                srv.submit_gemv(mp.NO_TRANS, m, kk, ab.view(0, 1), A, m, x, ab.view(1, 1),
                                outs_y.view(int(gy_off[i]), m))
                ops_total += 2.0 * m * kk
            else:
                m, nnz, csr, xa, ya = spmvs[p % len(spmvs)]
                srv.submit_spmv_csr(m, m, csr, xa, ya)
                ops_total += 2.0 * nnz
        srv.drain()
        st = srv.stats()
        t = srv.times(0, count)
        srv.destroy()
        span = float(t[:, 2].max() - t[:, 0].min())
        results.append({"offered_per_s": rate, "requests": count, "throughput_per_s": count / span,
                        "mp_ops_per_s": ops_total / span, "p50_ms": st["p50_s"] * 1e3, "p99_ms": st["p99_s"] * 1e3,
                        "mean_batch": st["mean_batch"], "max_in_flight": st["max_in_flight"],
                        "peak_admitted_gb": st["peak_bytes"] / 1e9})
        # a sample of requests rerun alone through the plain calls: identical records
        sample = [i for i in range(count) if kinds[i] != 2][:12]
        mix_y, mix_r = snapshot(outs_y), snapshot(outs_r)
        restore(outs_y, y_init)
        for i in sample:
            p = int(picks[i])
            if kinds[i] == 0:
                cnt, x, y = dots[p]
                mp.dot(n, cnt, x, y, outs_r.view(i, 1))
            else:
                m, kk, A, x, _, ab = gemvs[p]
                mp.gemv(n, mp.NO_TRANS, m, kk, ab.view(0, 1), A, m, x, ab.view(1, 1), outs_y.view(int(gy_off[i]), m))
        torch.cuda.synchronize()
        for i in sample:
            arr, snap, off, cnt = ((outs_r, mix_r, i, 1) if kinds[i] == 0 else
                                   (outs_y, mix_y, int(gy_off[i]), gemvs[int(picks[i])][0]))
            checks.append(all(torch.equal(a[sl], b[sl]) for a, b, sl in _record_slices(arr, snap, off, cnt)))
        # SpMV requests: every request on an operand set writes the same y, so
        # the y left by the mix must equal one plain call's
        for p in sorted({int(picks[i]) % len(spmvs) for i in range(count) if kinds[i] == 2}):
            m, _, csr, xa, ya = spmvs[p]
            alone = mp.DeviceBytes(m * rec)
            mp.spmv_csr(n, m, csr, xa, alone)
            torch.cuda.synchronize()
            checks.append(torch.equal(alone.t[: m * rec], ya.t[: m * rec]))
            del alone
        del outs_r, outs_y
    return {"workload": "Poisson mix of mp_dot (n 2^10..2^22), mp_gemv (m, n 32..4096), mp_spmv_csr (rows 2^12..2^20), "
                        "8 moduli, 64 GB budget, 4 batches in flight",
            "rates": results, "alone_vs_mix_identical": bool(checks) and all(checks), "checked_requests": len(checks)}


def _record_slices(arr, snap, off, cnt):
    """(current tensor, snapshot tensor, slice) triples covering elements [off, off + cnt) of a TensorArray."""
    n = arr.nmod
    return [(arr.digits, snap[0], slice(off * n, (off + cnt) * n)), (arr.sign, snap[1], slice(off, off + cnt)),
            (arr.exp, snap[2], slice(off, off + cnt)), (arr.eval, snap[3], slice(off, off + cnt)),
            (arr.eval, snap[3], slice(arr.size + off, arr.size + off + cnt))]


# ------------------------------------------------------------ CPU baseline --
#
# Every sample grows until its timed loop takes about budget_s / 2 or more, so
# the whole default run stays within a few minutes.

def _grow_blocks(run, m, budget_s, rows=8, cols=2):
    """Runs run(rows, cols) on growing blocks of C until one takes at least
    budget_s / 2; returns (rows, cols, seconds)."""
    t = run(rows, cols)
    while t < budget_s / 2 and (cols < m or rows < m):
        if cols < m:
            cols = min(m, cols * 2)
        else:
            rows = min(m, rows * 2)
        t = run(rows, cols)
    return rows, cols, t


def cpu_gemm_mpfr(src, budget_s=8.0):
    """The reference's mpfr_gemm OpenMP loop (tests/blas/v2/gemm/test_mpfr_gemm.cuh:29-60)
    at MP_PRECISION = 480 bits on all host cores, on a block of C with the full
    k = 1024; None where the host has no MPFR runtime."""
    from oracle import ffi
    L = ffi.mpfr_blas()
    if L is None:
        return None
    m = 1024
    al, be = float(src["alpha"][0]), float(src["beta"][0])

    def run(rows, cols):
        return L.gemm(rows, cols, m, al, src["A"], m, src["B"], m, be, src["C"], m, ffi.mp_precision(32))[0]

    rows, cols, t = _grow_blocks(run, m, budget_s, 16, 4)
    ops = 2.0 * rows * cols * m + 3.0 * rows * cols
    return {"value": ops / t, "unit": "MP ops/s", "cores": L.threads(), "kind": "mpfr", "seconds": t,
            "sample": "reference mpfr_gemm loop (MPFR, 480 bits, OpenMP) on a %dx%d block of C, k = 1024, %.1f s"
                      % (rows, cols, t)}


def cpu_gemm_port(host, budget_s=8.0):
    """The oracle port (the reference's multiple-precision arithmetic restated
    in C, OpenMP) on a bounded block of the GEMM with full k = 1024 chains."""
    from oracle import ffi
    O = ffi.oracle()
    n, m = 32, 1024
    A, B, C = host["A"], host["B"], host["C"]

    # sub-problem: C(0:rows, 0:cols) = alpha * A(0:rows, :) * B(:, 0:cols) + beta * C(0:rows, 0:cols),
    # passed with the full leading dimensions so no copy is needed
    def run(rows, cols):
        t0 = time.perf_counter()
        O.gemm(n, rows, cols, m, host["alpha"], A, m, B, m, host["beta"], C[: m * cols], m)
        return time.perf_counter() - t0

    rows, cols, t = _grow_blocks(run, m, budget_s)
    ops = 2.0 * rows * cols * m + 3.0 * rows * cols
    return {"value": ops / t, "unit": "MP ops/s", "cores": O.threads(), "kind": "port", "seconds": t,
            "sample": "oracle mp_gemm on a %dx%d block of C (k = 1024, 32 moduli), %.1f s" % (rows, cols, t)}


def cpu_gemv_sample(torch, mp, budget_s=6.0):
    """The oracle port on the first instances of the batched-GEMV workload (sizes
    as there, fresh seeded entries), until budget_s; MP ops/s."""
    from oracle import ffi
    O = ffi.oracle()
    n = 16
    sizes = log_uniform_ints(np.random.default_rng(SEED + 3), (4096, 2), 32, 4096)
    rng = np.random.default_rng(SEED + 30)
    ops = t = 0.0
    done = 0
    for m, k in sizes:
        m, k = int(m), int(k)
        A = mp.set_d(n, doubles(rng, m * k, -32, 32))
        x, y = mp.set_d(n, doubles(rng, k, -32, 32)), mp.set_d(n, doubles(rng, m, -32, 32))
        ab = mp.set_d(n, rng.uniform(-1, 1, 2))
        t0 = time.perf_counter()
        O.gemv(n, mp.NO_TRANS, m, k, ab[:1], A, m, x, ab[1:], y, b3=32)
        t += time.perf_counter() - t0
        ops += 2.0 * m * k
        done += 1
        if t > budget_s:
            break
    return {"value": ops / t, "unit": "MP ops/s", "cores": O.threads(), "kind": "port",
            "sample": "oracle mp_gemv on the first %d of the 4096 instances, %.1f s" % (done, t)}


def cpu_dot_port(mx, my, budget_s=6.0):
    from oracle import ffi
    O = ffi.oracle()
    count = 1 << 16
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < budget_s or reps == 0:
        O.dot(8, mx[:count], my[:count], g3=256, b3=64)
        reps += 1
    t = time.perf_counter() - t0
    return {"value": 2.0 * count * reps / t, "unit": "MP ops/s", "cores": O.threads(), "kind": "port",
            "sample": "oracle mp_dot on the first 2^16 elements, %d runs in %.1f s" % (reps, t)}


def cpu_dot_mpfr(xd, yd, budget_s=6.0):
    """The reference's mpfr_dot OpenMP loop (tests/blas/performance/test_dot_performance.cu:152-174)
    at 120 bits over the whole n = 2^20, repeated until budget_s of loop time."""
    from oracle import ffi
    L = ffi.mpfr_blas()
    if L is None:
        return None
    t = 0.0
    reps = 0
    w0 = time.perf_counter()
    while (t < budget_s and time.perf_counter() - w0 < 3 * budget_s) or reps == 0:
        t += L.dot(xd, yd, ffi.mp_precision(8))[0]
        reps += 1
    return {"value": 2.0 * len(xd) * reps / t, "unit": "MP ops/s", "cores": L.threads(), "kind": "mpfr",
            "sample": "reference mpfr_dot loop (MPFR, 120 bits, OpenMP), n = 2^20, %d runs, %.1f s" % (reps, t)}


def _row_block(irp, rows):
    return irp[: rows + 1], int(irp[rows])


def cpu_spmv_mpfr(irp, ja, vals, xd, budget_s=6.0):
    """The reference's mpfr_mpspmv_csr OpenMP loop (tests/sparse/spmv/csr/test_mpfr_spmv_csr.cuh:33-51)
    at 120 bits on the first rows of the benchmark matrix."""
    from oracle import ffi
    L = ffi.mpfr_blas()
    if L is None:
        return None
    m = len(irp) - 1
    rows = 4096
    while True:
        sub, nnz = _row_block(irp, rows)
        t = L.spmv_csr(rows, sub, ja, vals, xd, ffi.mp_precision(8))[0]
        if t >= budget_s / 2 or rows >= m:
            break
        rows = min(m, rows * 2)
    reps = 1
    while t < budget_s / 2:  # the whole matrix takes less: repeat it
        t += L.spmv_csr(rows, sub, ja, vals, xd, ffi.mp_precision(8))[0]
        reps += 1
    return {"value": 2.0 * nnz * reps / t, "unit": "MP ops/s", "cores": L.threads(), "kind": "mpfr",
            "sample": "reference mpfr_mpspmv_csr loop (MPFR, 120 bits, OpenMP) on the first %d rows (%d nnz), "
                      "%d runs, %.1f s" % (rows, nnz, reps, t)}


def cpu_spmv_port(irp, ja, vals, mx, budget_s=6.0):
    """The oracle port of mp_spmv_csr on the first rows of the benchmark matrix."""
    from oracle import ffi
    O = ffi.oracle()
    m = len(irp) - 1
    rows = 4096
    while True:
        sub, nnz = _row_block(irp, rows)
        t0 = time.perf_counter()
        O.spmv_csr(8, rows, sub, ja, vals, mx)
        t = time.perf_counter() - t0
        if t >= budget_s / 2 or rows >= m:
            break
        rows = min(m, rows * 2)
    reps = 1
    while t < budget_s / 2:  # the whole matrix takes less: repeat it
        t0 = time.perf_counter()
        O.spmv_csr(8, rows, sub, ja, vals, mx)
        t += time.perf_counter() - t0
        reps += 1
    return {"value": 2.0 * nnz * reps / t, "unit": "MP ops/s", "cores": O.threads(), "kind": "port",
            "sample": "oracle mp_spmv_csr on the first %d rows (%d nnz), %d runs, %.1f s" % (rows, nnz, reps, t)}


# -------------------------------------------------------------------- main --

def reference_arm(args, world):
    """The reference's CPU path for the headline GEMM on this host's cores: the
    MPFR mpfr_gemm loop (the port where the host has no MPFR runtime), one
    bounded block of C per step.  Loads only oracle/ libraries."""
    from oracle import ffi
    ffi.build_oracle()
    src = gemm_doubles()
    budget = min(8.0, max(2.0, 150.0 / max(1, args.steps)))
    if ffi.mpfr_blas() is not None:
        def sample(b):
            return cpu_gemm_mpfr(src, b)
    else:
        host = {k: ffi.oracle().set_d(32, v) for k, v in src.items()}

        def sample(b):
            return cpu_gemm_port(host, b)
    for _ in range(args.warmup):
        sample(1.0)
    samples = [sample(budget) for _ in range(args.steps)]
    v = statistics.median(s["value"] for s in samples)
    cb = dict(samples[0])
    cb["value"] = v
    secs = [s["seconds"] for s in samples]
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "MP ops/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(secs) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "MPFR 480-bit (reference CPU path)" if cb["kind"] == "mpfr" else "int32 residues + f64 interval bounds",
        "data": "synthetic (seeded u*2^e entries; the reference publishes no dataset)",
        "config": gemm_config(world),
        "cpu_baseline": cb, "e2e": {"value": v, "unit": "MP ops/s", "h2d_bytes_per_step": 0,
                                    "d2h_bytes_per_step": 0}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extra", action="store_true", help="headline GEMM only")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-GEMV and serving workloads")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines")
    ap.add_argument("--only", choices=["dot", "spmv", "bgemv64", "bgemm"], default=None,
                    help="one secondary workload alone, its own JSON line (profiling runs; bgemv64: the first 64 "
                         "instances of the batched GEMV workload)")
    args = ap.parse_args()
    world, rank, local = dist()

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, world)
        return

    import torch
    if world > 1:
        import torch.distributed as td
        td.init_process_group(backend="nccl")
    torch.cuda.set_device(local)
    import build
    if rank == 0:
        build.build()
    barrier(world)
    import mpres_gb300 as mp
    for nmod in (8, 16, 32):
        mp.init(nmod)
    stream = torch.cuda.Stream()
    hbm, peak_src = peaks()

    if args.only:
        if args.only == "bgemv64":
            r = bench_batched_gemv(torch, mp, stream, hbm, count=64)
        elif args.only == "bgemm":
            r = bench_batched_gemm(torch, mp, stream)
        else:
            run = bench_dot if args.only == "dot" else bench_spmv
            r = run(torch, mp, stream, args.steps, max(3, args.warmup), world, hbm)
        if rank == 0:
            print(json.dumps({k: v for k, v in r.items() if k != "data"}))
        return
    g = bench_gemm(torch, mp, stream, args.steps, max(3, args.warmup), world, rank, local)
    extra = {}
    if not args.no_extra:
        mhz = g["clocks"].get("sm_mhz") or 2070.0
        dot = bench_dot(torch, mp, stream, 20, 3, world, hbm, mhz)
        spmv = bench_spmv(torch, mp, stream, 5, 3, world, hbm, mhz)
        extra["mp_dot"] = {k: v for k, v in dot.items() if k != "data"}
        extra["mp_spmv"] = {k: v for k, v in spmv.items() if k != "data"}
        if not args.no_batch:
            extra["batched_gemv"] = bench_batched_gemv(torch, mp, stream, hbm)
            extra["batched_gemm"] = bench_batched_gemm(torch, mp, stream)
            extra["serving"] = bench_serving(torch, mp)
    line = {
        "metric": METRIC, "value": g["value"], "unit": "MP ops/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": g["secs"] / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32 residues + f64 interval bounds",
        "data": "synthetic (seeded u*2^e entries; the reference publishes no dataset)",
        "config": gemm_config(world),
        "roofline": g["roofline"], "hbm_peak_source": peak_src, "e2e": g["e2e"], "clocks": g["clocks"],
        "gpu_launches": g["launches"],
    }
    line.update(extra)
    if rank == 0 and not args.no_cpu:
        mp_cb, port_cb = cpu_gemm_mpfr(g["src"]), cpu_gemm_port(g["host"])
        line["cpu_baseline"] = mp_cb or port_cb
        line["cpu_baseline_port"] = port_cb
        if not args.no_extra:
            xd, yd, mx, my = dot["data"]
            line["mp_dot"]["cpu_baseline"] = cpu_dot_mpfr(xd, yd) or cpu_dot_port(mx, my)
            line["mp_dot"]["cpu_baseline_port"] = cpu_dot_port(mx, my)
            irp, ja, vals, sxd, smx = spmv["data"]
            line["mp_spmv"]["cpu_baseline"] = cpu_spmv_mpfr(irp, ja, vals, sxd) or cpu_spmv_port(irp, ja, vals, smx)
            line["mp_spmv"]["cpu_baseline_port"] = cpu_spmv_port(irp, ja, vals, smx)
            if "batched_gemv" in line:
                line["batched_gemv"]["cpu_baseline"] = cpu_gemv_sample(torch, mp)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
