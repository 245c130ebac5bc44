"""The Matrix Market reader against the reference's own (collect_mtx_stats,
build_csr, build_ell of src/sparse/utils/mtx_reader.cuh, compiled for the CPU):
identical statistics and identical CSR / ELL arrays -- entry order within rows
included, since it is the SpMV summation order -- for general and symmetric,
real and integer files with comments and unsorted, repeated-row entries, and
for the reference's fixture LF10.mtx where the reference checkout is present."""
import pathlib

import numpy as np
import pytest

import helpers
from oracle import ffi

_ROOT = ffi.reference_root()
LF10 = (_ROOT / "tests" / "sparse" / "matrices" / "LF10.mtx") if _ROOT else pathlib.Path("LF10.mtx.absent")


def write_mtx(path, m, n, entries, symmetric=False, dtype="real", comments=2):
    lines = ["%%%%MatrixMarket matrix coordinate %s %s" % (dtype, "symmetric" if symmetric else "general")]
    lines += ["%% comment line %d" % i for i in range(comments)]
    lines.append("%d %d %d" % (m, n, len(entries)))
    for r, c, v in entries:
        lines.append("%d %d %s" % (r, c, repr(int(v)) if dtype == "integer" else repr(float(v))))
    path.write_text("\n".join(lines) + "\n")
    return path


def random_entries(rng, m, n, count, symmetric=False):
    out, seen = [], set()
    while len(out) < count:
        r, c = int(rng.integers(1, m + 1)), int(rng.integers(1, n + 1))
        if symmetric and c > r:
            r, c = c, r
        if (r, c) in seen:
            continue
        seen.add((r, c))
        out.append((r, c, rng.normal() * 2.0 ** int(rng.integers(-20, 20))))
    return out  # random order: rows repeat and interleave


def cases(tmp_path):
    rng = np.random.default_rng(helpers.SEED + 60)
    yield write_mtx(tmp_path / "general.mtx", 300, 250, random_entries(rng, 300, 250, 3000))
    sym = random_entries(rng, 400, 400, 2500, symmetric=True) + [(i, i, rng.normal()) for i in range(1, 401, 3)]
    rng.shuffle(sym)
    yield write_mtx(tmp_path / "symmetric.mtx", 400, 400, sym, symmetric=True)
    ints = [(r, c, rng.integers(-9, 10)) for r, c, _ in random_entries(rng, 50, 60, 400)]
    yield write_mtx(tmp_path / "integer.mtx", 50, 60, ints, dtype="integer", comments=0)
    big_rows = [(1 + (i % 7), 1 + i % 500, rng.normal()) for i in range(3000)]  # long rows for the sort
    yield write_mtx(tmp_path / "long_rows.mtx", 7, 500, list(dict(((r, c), (r, c, v)) for r, c, v in big_rows).values()))
    if LF10.exists():
        yield LF10


@pytest.mark.skipif(not ffi.ref_available(8), reason="the reference is not built here")
def test_reader_matches_reference(library, tmp_path):
    mp = library
    for path in cases(tmp_path):
        st = mp.mtx_stats(path)
        rst, (rirp, rja, ras), (reja, reas) = ffi.ref_mtx(8, path)
        for k in ("m", "n", "lines", "maxnzr", "nzmd", "symmetric"):
            assert st[k] == rst[k], (path.name, k)
        irp, ja, vals = mp.mtx_csr(path, st)
        assert np.array_equal(irp, rirp) and np.array_equal(ja, rja), path.name
        assert vals.tobytes() == ras.tobytes(), path.name
        eja, eas = mp.mtx_ell(path, st)
        assert np.array_equal(eja, reja) and eas.tobytes() == reas.tobytes(), path.name


def test_reader_rows_and_errors(library, tmp_path):
    mp = library
    path = write_mtx(tmp_path / "s.mtx", 5, 5, [(2, 1, 1.5), (1, 1, 2.0), (5, 3, -1.0)], symmetric=True)
    st = mp.mtx_stats(path)
    assert (st["m"], st["nnz"], st["maxnzr"], st["nzmd"], st["datatype"]) == (5, 5, 2, 1, "real")
    irp, ja, vals = mp.mtx_csr(path, st)
    assert irp.tolist() == [0, 2, 3, 4, 4, 5]
    dense = np.zeros((5, 5))
    for r in range(5):
        for i in range(irp[r], irp[r + 1]):
            dense[r, ja[i]] += vals[i]
    assert np.array_equal(dense, dense.T) and dense[0, 0] == 2.0 and dense[4, 2] == -1.0
    (tmp_path / "p.mtx").write_text("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n")
    with pytest.raises(mp.MpresError, match="not supported"):
        mp.mtx_stats(tmp_path / "p.mtx")
    (tmp_path / "bad.mtx").write_text("hello\n")
    with pytest.raises(mp.MpresError):
        mp.mtx_stats(tmp_path / "bad.mtx")
    with pytest.raises(mp.MpresError, match="cannot open"):
        mp.mtx_stats(tmp_path / "missing.mtx")
