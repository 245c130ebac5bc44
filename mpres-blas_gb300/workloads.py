"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (the reference publishes no datasets; its SpMV drivers
read SuiteSparse matrices, replaced here by power-law CSR matrices)."""
import numpy as np

SEED = 0x4D505245  # configuration c uses SEED + c


def doubles(rng, count, emin, emax):
    """u * 2^e with u ~ U(-1, 1) and e ~ U{emin..emax}, exactly representable."""
    return np.ldexp(rng.uniform(-1.0, 1.0, count), rng.integers(emin, emax + 1, count))


def power_law_rows(rng, m, kmax=1024, alpha=1.6138):
    """Row lengths 1..kmax with P(k) ~ k^-alpha (mean 16 at alpha 1.6138, kmax 1024)."""
    k = np.arange(1, kmax + 1, dtype=np.float64)
    p = k ** -alpha
    p /= p.sum()
    return rng.choice(np.arange(1, kmax + 1), size=m, p=p).astype(np.int64)


def random_csr(rng, m, n, lengths):
    """CSR with the given row lengths, columns uniform without repeats and sorted
    within a row, values N(0, 1)."""
    lengths = np.minimum(lengths, n)
    irp = np.zeros(m + 1, np.int64)
    np.cumsum(lengths, out=irp[1:])
    nnz = int(irp[-1])
    rows = np.repeat(np.arange(m, dtype=np.int64), lengths)
    cols = rng.integers(0, n, nnz)
    while True:
        key = rows * n + cols
        order = np.argsort(key, kind="stable")
        key, rows, cols = key[order], rows[order], cols[order]
        dup = np.zeros(nnz, bool)
        dup[1:] = key[1:] == key[:-1]
        if not dup.any():
            break
        cols[dup] = rng.integers(0, n, int(dup.sum()))
    vals = rng.standard_normal(nnz)
    return irp.astype(np.int32), cols.astype(np.int32), vals


def csr_to_ell(m, irp, ja, vals):
    """ELLPACK slots col*m + row (column-major), zero padded."""
    lens = np.diff(irp).astype(np.int64)
    maxnzr = int(lens.max()) if m else 0
    ell_ja = np.zeros(maxnzr * m, np.int32)
    ell_as = np.zeros(maxnzr * m, np.float64)
    rows = np.repeat(np.arange(m, dtype=np.int64), lens)
    slot_in_row = np.arange(len(ja), dtype=np.int64) - np.repeat(irp[:-1].astype(np.int64), lens)
    idx = slot_in_row * m + rows
    ell_ja[idx] = ja
    ell_as[idx] = vals
    return maxnzr, ell_ja, ell_as
