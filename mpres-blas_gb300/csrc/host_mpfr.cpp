/*
 * The reference's host-side MPFR operations on multiple-precision numbers,
 * restated with exact integer arithmetic (GMP and MPFR are not needed):
 *   mp_div   (src/arith/div.cuh:33-45)   x / y,
 *   mp_sqrt  (src/arith/sqrt.cuh)        sqrt(x),
 *   mp_dsqrt (src/arith/sqrt.cuh)        sqrt(x) rounded to a double,
 * and their cuda:: forms, which copy the operands from the device, compute on
 * the host and copy the result back (src/arith/div.cuh:56-65).
 *
 * Every step is what MPFR does, bit for bit:
 *   - mp_get_mpfr (src/arith/assign.cuh:185-211): X = the integer of the
 *     residues (0 <= X < M), the value (-1)^sign X 2^exp rounded to nearest,
 *     ties to even, at MP_PRECISION bits (mpfr_set_str into a variable of that
 *     precision);
 *   - mpfr_div / mpfr_sqrt at MP_PRECISION bits, rounded to nearest-even
 *     (correctly rounded: the exact quotient or root, its remainder as sticky);
 *   - mp_set_mpfr (assign.cuh:86-127): the significand's binary digits with
 *     trailing zeros removed become X, the exponent follows, the residues are
 *     X mod m_i and the interval evaluation is the host rns_eval_compute.  Its
 *     string handling leaves zero as sign 0, exp -1 and negative zero as
 *     sign 1, exp 0; both are kept;
 *   - mpfr_get_d (mp_dsqrt): the MP_PRECISION-bit root rounded again to 53
 *     bits, nearest-even (a double rounding, as MPFR performs it).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "tables.h"

namespace mpres {

void host_eval_digits(const HostTables &t, const int *x, er_t &low, er_t &upp);

namespace {

/* non-negative integer, 32-bit limbs, least significant first, no leading zeros */
struct Big {
    std::vector<uint32_t> w;
    bool zero() const { return w.empty(); }
    void trim() {
        while (!w.empty() && w.back() == 0) w.pop_back();
    }
    int bits() const { return w.empty() ? 0 : (int)(32 * (w.size() - 1)) + (32 - __builtin_clz(w.back())); }
    bool bit(int i) const { return (size_t)(i / 32) < w.size() && ((w[i / 32] >> (i % 32)) & 1u); }
    /* any bit below position k set */
    bool any_below(int k) const {
        for (int i = 0; i < k / 32 && (size_t)i < w.size(); i++)
            if (w[i]) return true;
        if ((size_t)(k / 32) < w.size() && k % 32) return (w[k / 32] & ((1u << (k % 32)) - 1)) != 0;
        return false;
    }
    void mul_add(uint32_t m, uint32_t a) {
        uint64_t carry = a;
        for (uint32_t &v : w) {
            const uint64_t p = (uint64_t)v * m + carry;
            v = (uint32_t)p;
            carry = p >> 32;
        }
        if (carry) w.push_back((uint32_t)carry);
        trim();
    }
    uint32_t mod(uint32_t m) const {
        uint64_t r = 0;
        for (size_t i = w.size(); i-- > 0;) r = ((r << 32) | w[i]) % m;
        return (uint32_t)r;
    }
    void add_one() {
        for (uint32_t &v : w)
            if (++v != 0) return;
        w.push_back(1);
    }
};

Big shl(const Big &a, int k) {
    if (a.zero()) return a;
    Big r;
    r.w.assign(a.w.size() + k / 32 + 1, 0);
    const int s = k % 32;
    for (size_t i = 0; i < a.w.size(); i++) {
        const uint64_t v = (uint64_t)a.w[i] << s;
        r.w[i + k / 32] |= (uint32_t)v;
        r.w[i + k / 32 + 1] |= (uint32_t)(v >> 32);
    }
    r.trim();
    return r;
}

Big shr(const Big &a, int k) {
    Big r;
    const size_t q = (size_t)(k / 32);
    if (q >= a.w.size()) return r;
    const int s = k % 32;
    r.w.assign(a.w.size() - q, 0);
    for (size_t i = q; i < a.w.size(); i++) {
        uint64_t v = a.w[i];
        if (i + 1 < a.w.size()) v |= (uint64_t)a.w[i + 1] << 32;
        r.w[i - q] = (uint32_t)(v >> s);
    }
    r.trim();
    return r;
}

int cmp(const Big &a, const Big &b) {
    if (a.w.size() != b.w.size()) return a.w.size() < b.w.size() ? -1 : 1;
    for (size_t i = a.w.size(); i-- > 0;)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

/* a -= b, a >= b */
void sub_in(Big &a, const Big &b) {
    int64_t borrow = 0;
    for (size_t i = 0; i < a.w.size(); i++) {
        int64_t v = (int64_t)a.w[i] - borrow - (i < b.w.size() ? (int64_t)b.w[i] : 0);
        borrow = v < 0;
        a.w[i] = (uint32_t)(v + (borrow << 32));
    }
    a.trim();
}

/* q = a / b, r = a mod b (b != 0), binary long division */
void divmod(const Big &a, const Big &b, Big &q, Big &r) {
    q.w.clear();
    r.w.clear();
    const int n = a.bits();
    q.w.assign((size_t)(n / 32 + 1), 0);
    for (int i = n - 1; i >= 0; i--) {
        r = shl(r, 1);
        if (a.bit(i)) {
            if (r.w.empty()) r.w.push_back(1);
            else r.w[0] |= 1;
        }
        if (cmp(r, b) >= 0) {
            sub_in(r, b);
            q.w[i / 32] |= 1u << (i % 32);
        }
    }
    q.trim();
}

/* floor(sqrt(a)) and whether it is exact */
Big isqrt(const Big &a, bool &exact) {
    exact = true;
    if (a.zero()) return a;
    Big x;
    x.w.assign(1, 1);
    x = shl(x, (a.bits() + 1) / 2); /* >= sqrt(a) */
    for (;;) { /* Newton from above: y = (x + a / x) / 2 while it decreases */
        Big q, r;
        divmod(a, x, q, r);
        Big s = x;
        /* s = x + q */
        uint64_t carry = 0;
        const size_t len = std::max(s.w.size(), q.w.size());
        s.w.resize(len, 0);
        for (size_t i = 0; i < len; i++) {
            const uint64_t v = (uint64_t)s.w[i] + (i < q.w.size() ? q.w[i] : 0) + carry;
            s.w[i] = (uint32_t)v;
            carry = v >> 32;
        }
        if (carry) s.w.push_back((uint32_t)carry);
        s.trim();
        Big y = shr(s, 1);
        if (cmp(y, x) >= 0) break;
        x = y;
    }
    Big sq;
    { /* x*x == a ? */
        Big acc;
        for (size_t i = x.w.size(); i-- > 0;) {
            acc = shl(acc, 32);
            Big t = x;
            t.mul_add(x.w[i], 0);
            /* acc += t */
            uint64_t carry = 0;
            const size_t len = std::max(acc.w.size(), t.w.size());
            acc.w.resize(len, 0);
            for (size_t j = 0; j < len; j++) {
                const uint64_t v = (uint64_t)acc.w[j] + (j < t.w.size() ? t.w[j] : 0) + carry;
                acc.w[j] = (uint32_t)v;
                carry = v >> 32;
            }
            if (carry) acc.w.push_back((uint32_t)carry);
            acc.trim();
        }
        sq = acc;
    }
    exact = cmp(sq, a) == 0;
    return x;
}

/* a binary floating value: (-1)^neg * mant * 2^exp, mant with at most p bits */
struct Flt {
    bool neg = false;
    Big mant;
    long long exp = 0;
};

/* rounds mant * 2^exp (+ sticky below it) to p bits, nearest-even */
Flt round_to(bool neg, const Big &mant, long long exp, bool sticky, int p) {
    Flt f;
    f.neg = neg;
    const int L = mant.bits();
    if (L <= p) {
        f.mant = mant;
        f.exp = exp;
        return f; /* exact (sticky is never set with room to spare) */
    }
    const int drop = L - p;
    Big q = shr(mant, drop);
    const bool half = mant.bit(drop - 1);
    const bool rest = mant.any_below(drop - 1) || sticky;
    if (half && (rest || q.bit(0))) q.add_one();
    long long e = exp + drop;
    if (q.bits() > p) { /* carried into a new bit */
        q = shr(q, 1);
        e += 1;
    }
    f.mant = q;
    f.exp = e;
    return f;
}

/* mp_get_mpfr: the record's value at p bits */
Flt get(const HostTables &t, const char *rec, int p) {
    const int n = t.n;
    int digits[32], sign, exp;
    std::memcpy(digits, rec, 4 * n);
    std::memcpy(&sign, rec + 4 * n, 4);
    std::memcpy(&exp, rec + 4 * n + 4, 4);
    /* X from the residues by mixed-radix conversion */
    int mixed[32];
    for (int i = 0; i < n; i++) {
        int64_t v = digits[i];
        for (int j = 0; j < i; j++) {
            v = (v - mixed[j]) % t.moduli[i];
            if (v < 0) v += t.moduli[i];
            v = v * t.mrc_inv[j][i] % t.moduli[i];
        }
        mixed[i] = (int)v;
    }
    Big X;
    for (int i = n - 1; i >= 0; i--) X.mul_add((uint32_t)t.moduli[i], (uint32_t)mixed[i]);
    return round_to(sign == 1, X, exp, false, p);
}

/* mp_set_mpfr: the record of a p-bit value */
void set(const HostTables &t, const Flt &f, char *rec) {
    const int n = t.n;
    int digits[32] = {0};
    int sign, exp;
    if (f.mant.zero()) { /* the string handling of the reference for zeros */
        sign = f.neg ? 1 : 0;
        exp = f.neg ? 0 : -1;
    } else {
        int tz = 0;
        while (!f.mant.bit(tz)) tz++;
        const Big X = shr(f.mant, tz);
        for (int i = 0; i < n; i++) digits[i] = (int)X.mod((uint32_t)t.moduli[i]);
        sign = f.neg ? 1 : 0;
        exp = (int)(f.exp + tz);
    }
    er_t ev[2];
    host_eval_digits(t, digits, ev[0], ev[1]);
    std::memcpy(rec, digits, 4 * n);
    std::memcpy(rec + 4 * n, &sign, 4);
    std::memcpy(rec + 4 * n + 4, &exp, 4);
    std::memcpy(rec + 4 * n + 8, ev, sizeof(ev));
}

/* correctly rounded p-bit quotient */
bool div_p(const Flt &a, const Flt &b, int p, Flt &out) {
    if (b.mant.zero()) return false;
    if (a.mant.zero()) {
        out.neg = a.neg != b.neg;
        out.mant = Big();
        out.exp = 0;
        return true;
    }
    const int sh = p + 2 + b.mant.bits() - a.mant.bits() + 1;
    Big num = shl(a.mant, sh > 0 ? sh : 0), q, r;
    divmod(num, b.mant, q, r);
    out = round_to(a.neg != b.neg, q, a.exp - b.exp - (sh > 0 ? sh : 0), !r.zero(), p);
    return true;
}

/* correctly rounded p-bit square root (a >= 0) */
bool sqrt_p(const Flt &a, int p, Flt &out) {
    if (a.mant.zero()) {
        out = a;
        return true;
    }
    if (a.neg) return false;
    /* a = m 2^e; scale m by 2^(2k) with e - 2k even so the root has >= p + 2 bits */
    int k = p + 2 - (a.mant.bits() + 1) / 2 + 1;
    if (k < 0) k = 0;
    long long e = a.exp - 2LL * k;
    Big m = shl(a.mant, 2 * k);
    if (e % 2 != 0) {
        m = shl(m, 1);
        e -= 1;
    }
    bool exact;
    Big s = isqrt(m, exact);
    out = round_to(false, s, e / 2, !exact, p);
    return true;
}

double to_double(const Flt &f) {
    if (f.mant.zero()) return f.neg ? -0.0 : 0.0;
    const Flt d = round_to(f.neg, f.mant, f.exp, false, 53);
    uint64_t m = 0;
    for (size_t i = d.mant.w.size(); i-- > 0;) m = (m << 32) | d.mant.w[i];
    const double v = std::ldexp((double)m, (int)d.exp);
    return f.neg ? -v : v;
}

} // namespace

bool host_mp_div(const HostTables &t, const void *x, const void *y, void *r) {
    const int p = t.mp_precision;
    Flt q;
    if (!div_p(get(t, (const char *)x, p), get(t, (const char *)y, p), p, q)) return false;
    set(t, q, (char *)r);
    return true;
}

bool host_mp_sqrt(const HostTables &t, const void *x, void *r) {
    const int p = t.mp_precision;
    Flt s;
    if (!sqrt_p(get(t, (const char *)x, p), p, s)) return false;
    set(t, s, (char *)r);
    return true;
}

bool host_mp_dsqrt(const HostTables &t, const void *x, double &out) {
    const int p = t.mp_precision;
    Flt s;
    if (!sqrt_p(get(t, (const char *)x, p), p, s)) return false;
    out = to_double(s);
    return true;
}

} // namespace mpres
