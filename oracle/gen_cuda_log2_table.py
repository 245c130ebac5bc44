#!/usr/bin/env python3
"""Measures, on the GPU, where ceil(log2(x)) computed with the CUDA math library
differs from the exact ceil(log2(x)), and writes oracle/cuda_log2_table.h.

TEST INFRASTRUCTURE ONLY.  The reference's device code chooses the step of its
interval-evaluation refinement loop from ceil(log2(sumu)) (src/rns.cuh:848, :913),
evaluated with CUDA's log2, whose result may be one ulp off the exact value.
Where that changes the ceiling -- only within a few ulps of a power of two --
the reference's device results change too.  The oracle (plain C, on the host)
therefore takes the exact ceiling and corrects it with the deviations measured
here: for every binade e it probes every x within J(e) ulps of 2^e (J(e) covers
four result ulps of the logarithm, well beyond the documented one-ulp error) and
records the maximal runs of offsets where CUDA's ceiling differs, with the sign
of the difference.  A second pass checks a band beyond J(e) for deviations.

Run on a GPU machine:  python oracle/gen_cuda_log2_table.py <out.h>
"""
import math
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "mpres-blas_gb300"))

EMIN, EMAX = -1074, 1023


def zone(e):
    """Offsets (in ulps of x) probed on each side of 2^e."""
    r = abs(e)
    ulp_result = math.ulp(float(r)) if r else math.ulp(0.0)
    return 8 + int(math.ceil(4 * ulp_result * math.log(2) * 2.0 ** 52))


def points(e, lo, hi):
    """x = the values lo..hi steps of nextafter away from 2^e (negative = below)."""
    p = math.ldexp(1.0, e)
    bits = np.frombuffer(np.float64(p).tobytes(), np.int64)[0]
    offs = np.arange(lo, hi + 1, dtype=np.int64)
    xs = (bits + offs).view(np.float64)
    ok = (xs > 0) & np.isfinite(xs)
    return xs[ok], offs[ok]


def exact_ceil_log2(x):
    m, ex = np.frexp(x)  # x = m * 2^ex, m in [0.5, 1)
    return np.where(m == 0.5, ex - 1, ex).astype(np.float64)


def main():
    import mpres_gb300 as mp
    import build
    build.build()
    import torch
    torch.cuda.init()
    out_path = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else ROOT / "oracle" / "cuda_log2_table.h")
    runs = []
    beyond = 0
    total = 0
    for e in range(EMIN, EMAX + 1):
        J = zone(e)
        xs, offs = points(e, -J, J)
        got = mp.probe_ceil_log2(xs)
        want = exact_ceil_log2(xs)
        d = (got - want).astype(np.int64)
        total += len(xs)
        i = 0
        while i < len(d):
            if d[i] != 0:
                j = i
                while j + 1 < len(d) and d[j + 1] == d[i] and offs[j + 1] == offs[j] + 1:
                    j += 1
                runs.append((e, int(offs[i]), int(offs[j]), int(d[i])))
                i = j + 1
            else:
                i += 1
        # band beyond the zone: must show no deviation
        for lo, hi in ((-2 * J, -J - 1), (J + 1, 2 * J)):
            bx, _ = points(e, lo, hi)
            if len(bx):
                beyond += int((mp.probe_ceil_log2(bx) != exact_ceil_log2(bx)).sum())
    lines = [
        "/*",
        " * Deviations of ceil(log2(x)) computed with the CUDA math library on the GPU",
        " * from the exact ceil(log2(x)), measured by oracle/gen_cuda_log2_table.py",
        " * (%d points, every x within J(e) ulps of each power of two 2^e, e in [%d, %d];" % (total, EMIN, EMAX),
        " * %d deviations found in the bands beyond J(e))." % beyond,
        " * Each row {e, first, last, delta}: for x = 2^e moved by `first`..`last` ulps",
        " * (nextafter steps; negative = below 2^e), CUDA's ceiling is the exact one + delta.",
        " * Test infrastructure for the oracle; the library calls CUDA's log2 itself.",
        " */",
        "#ifndef ORACLE_CUDA_LOG2_TABLE_H",
        "#define ORACLE_CUDA_LOG2_TABLE_H",
        "static const int ORA_CUDA_LOG2_RUNS = %d;" % len(runs),
        "static const short ORA_CUDA_LOG2_TABLE[][4] = {",
    ]
    for r in runs:
        lines.append("    {%d, %d, %d, %d}," % r)
    if not runs:
        lines.append("    {0, 0, 0, 0},")
    lines += ["};", "#endif", ""]
    out_path.write_text("\n".join(lines))
    print("points", total, "runs", len(runs), "beyond-zone deviations", beyond, "->", out_path)


if __name__ == "__main__":
    main()
