"""The integer bounds behind mp_gemm's split form with 32 moduli, checked on the
predefined moduli themselves (CPU only).

The modular product W(A) x W(B) runs on the tensor cores as bf16 products of
8-bit limbs (gemm_mma_product, mpres-blas_gb300/csrc/gemm.cu): a residue
w < m is l0 + l1 2^8 + l2 2^16 + l3 2^24, each limb exact in bf16; the limb
products of one limb-sum group s = a + b are summed over a stage of 32 k steps
in fp32 started at 2^23, which is exact while every partial sum stays an
integer below 2^24, and the group's value, weighted by 2^(8s) mod m, enters a
64-bit accumulator folded every 128 stages.  These tests pin each bound the
kernel relies on, and the limb identity itself on random residues.
"""
import pathlib
import re

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
KC, FOLD_STAGES, GROUPS = 32, 128, 7


def moduli(n):
    text = (ROOT / "mpres-blas_gb300" / "csrc" / "moduli_sets.h").read_text()
    body = re.search(r"#define MPRES_SET%d_MODULI \{(.*?)\}" % n, text, re.S).group(1)
    vals = [int(v) for v in re.findall(r"\d+", body.replace("\\", " "))]
    assert len(vals) == n
    return vals


def limb_max(m):
    """the largest value each limb of a residue below m can take"""
    top = (m - 1) >> 24
    return [255, 255, 255, top]


def test_moduli_fit_the_limb_form():
    for m in moduli(32):
        assert m % 2 == 1
        assert m * m < 2 ** 60.6           # products of residues below 2^60.6 (the integer forms' fold rule)
        assert (m - 1) >> 24 <= 78          # the top limb


def test_group_sums_of_a_stage_stay_below_2_23():
    for m in moduli(32):
        lm = limb_max(m)
        for s in range(GROUPS):
            bound = sum(KC * lm[a] * lm[s - a] for a in range(4) if 0 <= s - a <= 3)
            assert bound < 2 ** 23, (m, s, bound)   # 2^23 + sum < 2^24: exact in fp32, sum in the significand


def test_accumulator_fold_budget():
    for m in moduli(32):
        c32 = (1 << 32) % m
        folded = ((1 << 32) - 1) * c32 + ((1 << 32) - 1)      # after a fold
        terms = FOLD_STAGES * GROUPS * ((1 << 23) - 1) * (m - 1)  # group values times weights below m
        assert folded + terms < 2 ** 64
        assert terms < 2 ** 64                                # the first run of stages, from zero


def test_limb_identity_on_random_residues():
    """sum_s 2^(8s) G_s = W(A) W(B) exactly (integers), so mod m as well"""
    rng = np.random.default_rng(20261204)
    for m in moduli(32)[::5]:
        a = rng.integers(0, m, size=(6, 40), dtype=np.int64)
        b = rng.integers(0, m, size=(40, 5), dtype=np.int64)
        la = [(a >> (8 * i)) & 255 for i in range(4)]
        lb = [(b >> (8 * i)) & 255 for i in range(4)]
        assert all(int(x.max()) <= lim for x, lim in zip(la, limb_max(m)))
        total = np.zeros((6, 5), dtype=object)
        for s in range(GROUPS):
            g = sum(la[i].astype(object).dot(lb[s - i].astype(object)) for i in range(4) if 0 <= s - i <= 3)
            total = total + g * pow(2, 8 * s, m)
        want = a.astype(object).dot(b.astype(object))
        assert np.all((total - want) % m == 0)
