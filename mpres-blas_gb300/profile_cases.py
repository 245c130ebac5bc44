"""One launch of each hot kernel, for ncu captures (the summaries under
profiles/ name the command that made them).

    python mpres-blas_gb300/profile_cases.py [--full] [dot] [spmv] [gemv] [gemm] [batch]

Small cases (default) keep a `--set full` capture short: mp_dot n = 2^20
(8 moduli), mp_spmv_csr / csrv32 on 2^18 power-law rows (8 moduli), mp_gemv
1024 x 1024 (16 moduli), mp_gemm 256^3 (32 moduli), a batch of 64 GEMVs
(16 moduli).  --full runs the benchmark sizes instead (mp_spmv 2^20 rows,
mp_gemm 1024^3, a batch of 512 GEMVs with m, n log-uniform in [32, 1024]) for
single-pass captures such as the DRAM byte counters."""
import sys

import numpy as np

import build
import mpres_gb300 as mp
from workloads import doubles, power_law_rows, random_csr


def main(which, full):
    import torch
    build.build()
    for n in (8, 16, 32):
        mp.init(n)
    rng = np.random.default_rng(1)
    if "dot" in which:
        c = 1 << 20
        x = mp.DeviceArray.from_host(8, mp.set_d(8, doubles(rng, c, -16, 16)))
        y = mp.DeviceArray.from_host(8, mp.set_d(8, doubles(rng, c, -16, 16)))
        r = mp.DeviceArray(8, 1)
        mp.dot(8, c, x, y, r)
    if "spmv" in which:
        m = 1 << (20 if full else 18)
        irp, ja, vals = random_csr(rng, m, m, power_law_rows(rng, m))
        xv = mp.DeviceBytes.from_numpy(mp.set_d(8, doubles(rng, m, -16, 16)))
        yv = mp.DeviceBytes(m * 72)
        csr = mp.DeviceCsr(m, irp, ja, vals)
        mp.spmv_csr(8, m, csr, xv, yv)
        mp.spmv_csrv(8, m, csr, xv, yv, 32)
    if "gemv" in which:
        m = 1024
        A = mp.DeviceArray.from_host(16, mp.set_d(16, doubles(rng, m * m, -32, 32)))
        xg = mp.DeviceArray.from_host(16, mp.set_d(16, doubles(rng, m, -32, 32)))
        yg = mp.DeviceArray.from_host(16, mp.set_d(16, doubles(rng, m, -32, 32)))
        a = mp.DeviceArray.from_host(16, mp.set_d(16, np.array([0.7])))
        mp.gemv(16, mp.NO_TRANS, m, m, a, A, m, xg, a, yg)
    if "gemm" in which:
        k = 1024 if full else 256
        A = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        B = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        C = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        al = mp.DeviceArray.from_host(32, mp.set_d(32, np.array([0.7])))
        be = mp.DeviceArray.from_host(32, mp.set_d(32, np.array([-0.3])))
        mp.gemm(32, k, k, k, al, A, k, B, k, be, C, k)
    if "batch" in which:
        count = 512 if full else 64
        brng = np.random.default_rng(3)  # its own generator: the same batch whatever ran before
        sizes = np.exp(brng.uniform(np.log(32), np.log(1024), (count, 2))).astype(int)
        algo = int(np.sum((sizes[:, 0] * sizes[:, 1] + sizes[:, 1] + 2 * sizes[:, 0]) * 104))
        print("batch of %d GEMVs: %d algorithmic bytes" % (count, algo))
        a = mp.DeviceArray.from_host(16, mp.set_d(16, np.array([0.7])))
        b = mp.Batch(16)
        keep = []
        for m, n in sizes:
            A = mp.DeviceArray.from_host(16, mp.set_d(16, brng.uniform(-1, 1, m * n)))
            x = mp.DeviceArray.from_host(16, mp.set_d(16, brng.uniform(-1, 1, n)))
            y = mp.DeviceArray.from_host(16, mp.set_d(16, brng.uniform(-1, 1, m)))
            keep.append((A, x, y))
            b.add_gemv(mp.NO_TRANS, int(m), int(n), a, A, int(m), x, a, y, b3=32)
        b.commit(0)
        b.run()
    torch.cuda.synchronize()
    print("profile cases ok:", ",".join(which), "(full)" if full else "(small)")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--full"]
    main(tuple(args) or ("dot", "spmv", "gemv", "gemm", "batch"), "--full" in sys.argv[1:])
