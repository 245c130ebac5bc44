"""The identity mp_gemm's lazy-residue k chain rests on, checked on the oracle
(itself pinned to the reference) on the CPU.

With W(X) = (-1)^sign * digits * 2^exp mod m_i (2 is invertible modulo the odd
moduli, so negative exponents are fine), every step of a GEMM k chain satisfies
    W(a * b) = W(a) * W(b)                         unless mp_mul rounds,
    W(x + y) = nzx * W(x) + nzy * W(y)             unless mp_add rounds,
where nzx, nzy are mp_add's flags that drop a negligible operand
(src/arith/add.cuh:126-188).  The identity holds whatever the exponents and
whatever sign mp_add gives the sum, including the sign_estimate case.  So
between roundings the chain's residues are a modular dot product of W(A) and
W(B), and the digits come back as (-1)^sign * W * 2^-exp."""
import numpy as np
import pytest

import helpers
from oracle import ffi


def _i32(v):
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= 1 << 31 else v


def _w(rec, mods):
    s, e = int(rec["sign"]), int(rec["exp"])
    return [((-1) ** s * int(d) * pow(2, e, m)) % m for d, m in zip(rec["digits"], mods)]


def _chain(O, n, A, B, mp_j, mods, counts):
    x = np.zeros(1, ffi.mp_dtype(n))  # MP_ZERO
    W = [0] * n
    for i in range(len(A)):
        a, b = A[i:i + 1], B[i:i + 1]
        p = O.mul(n, a, b)
        r = O.add(n, x, p)
        ex, ey = int(x["exp"][0]), int(p["exp"][0])
        dexp = _i32(ex - ey)
        gamma, theta = max(dexp, 0), max(-dexp, 0)
        yev1, xev1 = p["eval"][0][1], x["eval"][0][1]
        nzx = int(yev1["frac"] == 0.0 or theta + int(yev1["exp"]) < mp_j)
        nzy = int(xev1["frac"] == 0.0 or gamma + int(xev1["exp"]) < mp_j)
        gamma *= nzy
        theta *= nzx
        exa, eya = _i32((ex - gamma) * nzx), _i32((ey - theta) * nzy)
        p_rounded = int(p["exp"][0]) != _i32(int(a["exp"][0]) + int(b["exp"][0]))
        r_rounded = int(r["exp"][0]) != (eya if exa == 0 else exa)
        if not p_rounded:
            assert _w(p[0], mods) == [(u * v) % m for u, v, m in zip(_w(a[0], mods), _w(b[0], mods), mods)]
        if not p_rounded and not r_rounded:
            W = [(nzx * w + nzy * q) % m for w, q, m in zip(W, _w(p[0], mods), mods)]
            assert W == _w(r[0], mods), (n, i, nzx, nzy)
            counts["lazy"] += 1
            counts["dropped"] += int(not (nzx and nzy))
        else:
            W = _w(r[0], mods)
            counts["rounded"] += 1
        x = r


@pytest.mark.parametrize("n", [8, 16, 32])
def test_chain_residues_are_a_modular_dot_product(oracle, n):
    mods = helpers.moduli(n)
    mp_j = int(oracle.tables(n, helpers.LOG2M[n])["mp_consts"][2])
    counts = {"lazy": 0, "dropped": 0, "rounded": 0}
    for trial in range(8):
        rng = np.random.default_rng(helpers.SEED + 100 * n + trial)
        k = 48
        lo, hi = [(-32, 32), (-400, 400), (-1000, 1000), (-2, 2)][trial % 4]
        a, b = helpers.doubles(rng, k, lo, hi), helpers.doubles(rng, k, lo, hi)
        if trial % 3 == 0:  # exact cancellations: the sum's sign comes from sign_estimate
            a[1::2] = a[0::2]
            b[1::2] = -b[0::2]
        a[rng.integers(0, k, 3)] = 0.0
        A, B = oracle.set_d(n, a), oracle.set_d(n, b)
        if trial % 4 == 3:  # wide residue integers: products and sums round
            A = oracle.mul(n, A, oracle.mul(n, A, A))
            B = oracle.mul(n, B, oracle.mul(n, B, B))
        _chain(oracle, n, A, B, mp_j, mods, counts)
    assert counts["lazy"] > 0 and counts["dropped"] > 0
    if n == 8:
        assert counts["rounded"] > 0
