"""One launch of every hot kernel on a small case, for ncu captures
(profiles/ summaries name the command).  Sizes keep a full-set capture short:
mp_dot n=2^20 (8 moduli), mp_spmv_csr/csrv32 on 2^18 power-law rows (8 moduli),
mp_gemv 1024x1024 (16 moduli), mp_gemm 256^3 (32 moduli)."""
import sys

import numpy as np

import build
import mpres_gb300 as mp
from workloads import doubles, power_law_rows, random_csr


def main(which=("dot", "spmv", "gemv", "gemm")):
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
        m = 1 << 18
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
        k = 256
        A = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        B = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        C = mp.DeviceArray.from_host(32, mp.set_d(32, doubles(rng, k * k, -32, 32)))
        al = mp.DeviceArray.from_host(32, mp.set_d(32, np.array([0.7])))
        be = mp.DeviceArray.from_host(32, mp.set_d(32, np.array([-0.3])))
        mp.gemm(32, k, k, k, al, A, k, B, k, be, C, k)
    torch.cuda.synchronize()
    print("profile cases ok:", ",".join(which))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("dot", "spmv", "gemv", "gemm"))
