/*
 * Matrix Market coordinate files -> the CSR and ELL arrays of the SpMV
 * kernels: the reference's collect_mtx_stats, build_csr and build_ell
 * (src/sparse/utils/mtx_reader.cuh:52-101, :200-253, :374-406), as host
 * functions behind the C ABI.
 *
 * The arrays must be what the reference builds from the same file, because
 * the order of a row's entries is the order of its SpMV chain:
 *   CSR  every data line in file order, the mirror (col, row) of each
 *        off-diagonal entry of a symmetric matrix appended after all lines,
 *        then the whole list sorted by row with std::sort (not a stable
 *        sort: the order within a row is what this standard library's
 *        introsort makes of that list, so the same call on the same list is
 *        used here), and the row pointers counted from it;
 *   ELL  column-major slots filled row by row in file order, a mirror placed
 *        right after the entry it mirrors; empty slots hold 0.0 and column -1.
 * Values are parsed as the reference's stream extraction parses them (to the
 * nearest double).  Files whose data type is not real or integer (pattern,
 * complex) are rejected: the reference would misread them.
 */
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpres_gb300.h"
#include "kernels.h"

using namespace mpres;

namespace {

struct Reader {
    FILE *f = nullptr;
    std::string dtype;
    bool symmetric = false;
    int m = 0, n = 0, lines = 0;
    ~Reader() {
        if (f) fclose(f);
    }
    /* header, comments and the size line; the file is left at the first data line */
    int open(const char *path, const char *what) {
        f = fopen(path, "r");
        if (!f) return status_fail(MPRES_ERR_INVALID_VALUE, "%s: cannot open %s", what, path);
        char head[64] = {0}, type[64] = {0}, fmt[64] = {0}, dt[64] = {0}, sym[64] = {0};
        if (fscanf(f, "%63s %63s %63s %63s %63s", head, type, fmt, dt, sym) != 5 || strcmp(head, "%%MatrixMarket") != 0 ||
            (strcmp(type, "matrix") != 0 && strcmp(type, "tensor") != 0) ||
            (strcmp(sym, "general") != 0 && strcmp(sym, "symmetric") != 0))
            return status_fail(MPRES_ERR_INVALID_VALUE, "%s: %s is not a general or symmetric Matrix Market matrix",
                               what, path);
        if (strcmp(fmt, "coordinate") != 0)
            return status_fail(MPRES_ERR_NOT_SUPPORTED, "%s: %s is not in coordinate format", what, path);
        dtype = dt;
        if (dtype != "real" && dtype != "integer")
            return status_fail(MPRES_ERR_NOT_SUPPORTED, "%s: data type %s is not supported", what, dt);
        symmetric = strcmp(sym, "symmetric") == 0;
        /* skip the rest of the header line and every comment line */
        int c;
        while ((c = fgetc(f)) != EOF && c != '\n') {
        }
        for (;;) {
            c = fgetc(f);
            if (c == '%') {
                while ((c = fgetc(f)) != EOF && c != '\n') {
                }
                continue;
            }
            if (c != EOF) ungetc(c, f);
            break;
        }
        if (fscanf(f, "%d %d %d", &m, &n, &lines) != 3 || m <= 0 || n <= 0 || lines < 0)
            return status_fail(MPRES_ERR_INVALID_VALUE, "%s: bad size line in %s", what, path);
        return MPRES_SUCCESS;
    }
    /* the next data line: 1-based row and column, value */
    bool next(int &row, int &col, double &v) {
        char buf[128];
        if (fscanf(f, "%d %d %127s", &row, &col, buf) != 3) return false;
        errno = 0;
        char *end = nullptr;
        v = strtod(buf, &end);
        return end != buf && row >= 1 && row <= m && col >= 1 && col <= n;
    }
};

} // namespace

extern "C" {

int mpres_mtx_stats(const char *path, int *m, int *n, int *lines, int *maxnzr, int *nzmd, int *symmetric,
                    char *datatype) {
    if (!path || !m || !n || !lines || !maxnzr || !nzmd || !symmetric)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_stats: null argument");
    Reader r;
    if (int st = r.open(path, "mpres_mtx_stats")) return st;
    std::vector<int> per_row((size_t)r.m, 0);
    int diag = 0;
    for (int l = 0; l < r.lines; l++) {
        int row, col;
        double v;
        if (!r.next(row, col, v)) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_stats: bad data line %d", l + 1);
        per_row[row - 1]++;
        if (row == col) diag++;
        if (r.symmetric && row != col) {
            if (col > r.m) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_stats: symmetric matrix not square");
            per_row[col - 1]++;
        }
    }
    *m = r.m;
    *n = r.n;
    *lines = r.lines;
    *maxnzr = *std::max_element(per_row.begin(), per_row.end());
    *nzmd = diag;
    *symmetric = r.symmetric;
    if (datatype) snprintf(datatype, 16, "%s", r.dtype.c_str());
    return status_ok();
}

int mpres_mtx_build_csr(const char *path, int m, int nnz, int lines, int symmetric, double *as, int *ja, int *irp) {
    if (!path || !as || !ja || !irp) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_csr: null argument");
    Reader r;
    if (int st = r.open(path, "mpres_mtx_build_csr")) return st;
    if (r.m != m || r.lines != lines || (bool)symmetric != r.symmetric)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_csr: arguments do not match %s", path);
    struct Entry {
        double v;
        int col, row;
    };
    std::vector<Entry> e((size_t)lines);
    std::vector<Entry> mirrors;
    for (int l = 0; l < lines; l++) {
        int row, col;
        double v;
        if (!r.next(row, col, v))
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_csr: bad data line %d", l + 1);
        e[l] = {v, col - 1, row - 1};
        if (symmetric && row != col) mirrors.push_back({v, row - 1, col - 1});
    }
    e.insert(e.end(), mirrors.begin(), mirrors.end());
    if ((long long)e.size() != nnz)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_csr: %zu entries, nnz = %d", e.size(), nnz);
    std::sort(e.begin(), e.end(), [](const Entry a, const Entry b) { return a.row < b.row; });
    for (int i = 0; i < nnz; i++) {
        as[i] = e[i].v;
        ja[i] = e[i].col;
    }
    /* irp[i] = first entry of row i or later */
    int p = 0;
    for (int i = 0; i <= m; i++) {
        while (p < nnz && e[p].row < i) p++;
        irp[i] = p;
    }
    return status_ok();
}

int mpres_mtx_build_ell(const char *path, int m, int maxnzr, int lines, int symmetric, double *as, int *ja) {
    if (!path || !as || !ja) return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_ell: null argument");
    Reader r;
    if (int st = r.open(path, "mpres_mtx_build_ell")) return st;
    if (r.m != m || r.lines != lines || (bool)symmetric != r.symmetric || maxnzr < 0)
        return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_ell: arguments do not match %s", path);
    const size_t slots = (size_t)m * (size_t)maxnzr;
    std::fill(ja, ja + slots, -1);
    std::fill(as, as + slots, 0.0);
    std::vector<int> used((size_t)m, 0);
    auto put = [&](int row, int col, double v) {
        if (used[row] >= maxnzr) return false;
        as[(size_t)used[row] * m + row] = v;
        ja[(size_t)used[row] * m + row] = col;
        used[row]++;
        return true;
    };
    for (int l = 0; l < lines; l++) {
        int row, col;
        double v;
        if (!r.next(row, col, v))
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_ell: bad data line %d", l + 1);
        if (!put(row - 1, col - 1, v) || (symmetric && row != col && !put(col - 1, row - 1, v)))
            return status_fail(MPRES_ERR_INVALID_VALUE, "mpres_mtx_build_ell: a row has more than maxnzr = %d entries",
                               maxnzr);
    }
    return status_ok();
}

} // extern "C"
