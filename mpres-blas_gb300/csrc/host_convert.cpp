/*
 * Host conversion double -> mp_float_t, the reference's mp_set_d
 * (src/arith/assign.cuh:54-81) with its host interval evaluation
 * rns_eval_compute (src/rns.cuh:645-716).
 *
 * The host evaluation is NOT the device one: it rounds with the emulated
 * directed rounding of src/dinterval.cuh (c -/+ (PHI1*|c| + ETA), evaluated in
 * round-to-nearest without fusing), multiplies residues through a double
 * quotient (src/modular.cuh:88-93, which may leave a residue off by one modulus)
 * and divides instead of multiplying by reciprocals in its refinement loop.
 * Converted inputs are part of every computation's result, so all of that is
 * reproduced exactly.  Compile without FP contraction (-ffp-contract=off).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "tables.h"

namespace mpres {

namespace {

const double kPhi1 = std::ldexp(1.0, -53) * (1 + 2 * std::ldexp(1.0, -53));
const double kEta = std::ldexp(1.0, -1074);

inline double emu_rd(double c) { return c - (kPhi1 * std::fabs(c) + kEta); }
inline double emu_ru(double c) { return c + (kPhi1 * std::fabs(c) + kEta); }
inline double emu_add_rd(double a, double b) { return emu_rd(a + b); }
inline double emu_add_ru(double a, double b) { return emu_ru(a + b); }

/* pairwise tree of src/pairwise.cuh:401-479 (host): span 2^k >= 8 holding len leaves */
template <class Add> double tree(const double *x, int len, int span, Add add) {
    if (span == 2) return add(x[0], len > 1 ? x[1] : 0.0);
    int h = span / 2;
    double s1 = tree(x, len, h, add);
    double s2 = len > h ? tree(x + h, len - h, h, add) : 0.0;
    return add(s1, s2);
}
template <class Add> double pairwise(const double *x, int len, Add add) {
    int span = 8;
    while (span <= len) span *= 2;
    return tree(x, len, span, add);
}

inline int mulmod_dq(int x, int y, int m, double d) {
    int64_t r = (int64_t)x * (int64_t)y;
    double q = (double)r * d;
    int i = (int)q;
    return (int)(r - (int64_t)i * (int64_t)m);
}

/* host mrd, src/rns.cuh:514-531 */
int host_mrd(const HostTables &t, const int *x) {
    int mixed[32];
    for (int i = 0; i < t.n; i++) {
        int v = x[i];
        for (int j = 0; j < i; j++) {
            if (v < mixed[j]) v = (int)((int64_t)t.moduli[i] - (int64_t)mixed[j] + (int64_t)v);
            else v = v - mixed[j];
            v = (int)(((int64_t)v * (int64_t)t.mrc_inv[j][i]) % t.moduli[i]);
        }
        mixed[i] = v;
    }
    return mixed[t.n - 1];
}

void set_er(er_t &r, double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    if (x != 0) {
        r.exp = (long long)((u & ~(1ull << 63)) >> 52) - 1023;
        u = (u & (((1ull << 52) - 1) | (1ull << 63))) | (1023ull << 52);
        std::memcpy(&r.frac, &u, 8);
    } else {
        r.exp = 0;
        r.frac = 0;
    }
}

/* host rns_eval_compute, src/rns.cuh:645-716 */
void host_eval(const HostTables &t, const int *x, er_t &low, er_t &upp) {
    const int n = t.n;
    bool zero = true;
    for (int i = 0; i < n; i++) zero = zero && x[i] == 0;
    if (zero) {
        low.frac = upp.frac = 0;
        low.exp = upp.exp = 0;
        return;
    }
    int s[32];
    double fl[32], fu[32];
    for (int i = 0; i < n; i++) s[i] = mulmod_dq(x[i], t.part_inv[i], t.moduli[i], 1.0 / t.moduli[i]);
    for (int i = 0; i < n; i++) {
        fl[i] = emu_rd(s[i] * t.recip_rd[i]);
        fu[i] = emu_ru(s[i] * t.recip_ru[i]);
    }
    double suml = pairwise(fl, n, emu_add_rd);
    double sumu = pairwise(fu, n, emu_add_ru);
    unsigned whl = (unsigned)suml, whu = (unsigned)sumu;
    suml = suml - whl;
    sumu = sumu - whu;
    set_er(low, suml);
    set_er(upp, sumu);
    int mr = -1;
    if (whl != whu) mr = host_mrd(t, x);
    if (mr > 0) {
        upp = t.inv_unit_upp;
        return;
    }
    if (mr == 0) low = t.unit_low;
    if (sumu >= t.eval_acc) return;
    int K = 0;
    for (int guard = 0; sumu < t.eval_acc && guard < 4096; guard++) {
        double a = -(std::ceil(std::log2(sumu)) + 1);
        int k = (int)(a > t.ref_factor ? a : (double)t.ref_factor);
        if (k > t.log2m) k = t.log2m;
        for (int i = 0; i < n; i++)
            s[i] = mulmod_dq(s[i], t.pow2[(size_t)k * n + i], t.moduli[i], 1.0 / t.moduli[i]);
        for (int i = 0; i < n; i++) fu[i] = emu_ru((double)s[i] / (double)t.moduli[i]);
        sumu = pairwise(fu, n, emu_add_ru);
        sumu -= (unsigned)sumu;
        K += k;
    }
    for (int i = 0; i < n; i++) fl[i] = emu_rd((double)s[i] / (double)t.moduli[i]);
    suml = pairwise(fl, n, emu_add_rd);
    suml -= (unsigned)suml;
    set_er(low, suml);
    set_er(upp, sumu);
    low.exp -= K;
    upp.exp -= K;
}

/* mp_set_d, src/arith/assign.cuh:54-81; out points to one mp_float_t (4n+40 bytes) */
void set_d(const HostTables &t, double x, char *out) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    int sign = (int)(u >> 63);
    int exp = (int)((u >> 52) & 2047);
    int64_t sig = (int64_t)(u & ((1ull << 52) - 1));
    if (exp != 0) sig |= (int64_t)1 << 52;
    exp = exp - 1023 - 52;
    if (sig != 0) {
        while ((sig & 1) == 0) {
            sig >>= 1;
            exp++;
        }
    } else {
        exp = 0;
    }
    int digits[32];
    for (int i = 0; i < t.n; i++) digits[i] = (int)(sig % (int64_t)t.moduli[i]);
    er_t ev[2];
    host_eval(t, digits, ev[0], ev[1]);
    /* a 53-bit significand stays below the rounding threshold of every set */
    std::memcpy(out, digits, 4 * t.n);
    std::memcpy(out + 4 * t.n, &sign, 4);
    std::memcpy(out + 4 * t.n + 4, &exp, 4);
    std::memcpy(out + 4 * t.n + 8, ev, sizeof(ev));
}

} // namespace

void host_eval_digits(const HostTables &t, const int *x, er_t &low, er_t &upp) { host_eval(t, x, low, upp); }

/* How ceil(std::log2(x)) -- the call of the refinement loop above -- behaves just
 * above each power of two 2^e, e = -1022..0.  out[2(e+1022)] = ceil(log2(2^e));
 * out[2(e+1022)+1] = the smallest j >= 1 with ceil(log2(2^e (1 + j 2^-52))) =
 * e + 1 (below it the rounded logarithm is still e).  Further from 2^e the
 * logarithm is at least one unit of its last place above e, so every log2
 * within one ulp gives the exact ceiling.  Returns false if the host's log2 is
 * not monotone over the probed window. */
bool host_ceil_log2_table(int *out) {
    for (int e = -1022; e <= 0; e++) {
        const double p = std::ldexp(1.0, e);
        out[2 * (e + 1022)] = (int)std::ceil(std::log2(p));
        int thr = 0;
        for (int j = 1; j < (1 << 20); j++) {
            const double x = p + std::ldexp((double)j, e - 52);
            const int c = (int)std::ceil(std::log2(x));
            if (c == e + 1) { thr = j; break; }
            if (c != e) return false;
        }
        if (thr == 0) return false;
        for (int j = thr; j < thr + 256; j++)
            if ((int)std::ceil(std::log2(p + std::ldexp((double)j, e - 52))) != e + 1) return false;
        out[2 * (e + 1022) + 1] = thr;
    }
    return true;
}

void host_set_d(const HostTables &t, const double *x, size_t count, void *out) {
    const size_t stride = 4 * (size_t)t.n + 40;
    char *o = static_cast<char *>(out);
    unsigned hw = std::thread::hardware_concurrency();
    size_t workers = count < 4096 ? 1 : (hw ? hw : 1);
    if (workers == 1) {
        for (size_t i = 0; i < count; i++) set_d(t, x[i], o + i * stride);
        return;
    }
    std::vector<std::thread> pool;
    size_t chunk = (count + workers - 1) / workers;
    for (size_t w = 0; w < workers; w++) {
        size_t lo = w * chunk, hi = lo + chunk < count ? lo + chunk : count;
        if (lo >= hi) break;
        pool.emplace_back([&, lo, hi] {
            for (size_t i = lo; i < hi; i++) set_d(t, x[i], o + i * stride);
        });
    }
    for (auto &th : pool) th.join();
}

} // namespace mpres
