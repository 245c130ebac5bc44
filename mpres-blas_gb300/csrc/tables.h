/*
 * Constant tables of one moduli set, shared by host code and kernels.
 *
 * They hold what the reference's rns_const_init() (src/rns.cuh:324-442) and
 * mp_const_init() (src/arith/arith_utils.cuh:44-90) compute, plus the Barrett
 * factors this library uses in place of 64-bit `%`.  Small tables live in
 * __constant__ memory of every translation unit that has kernels; the two large
 * ones (powers of two mod m_i, inverse powers of two) live in global memory.
 */
#ifndef MPRES_TABLES_H
#define MPRES_TABLES_H

#include <cstdint>

namespace mpres {

/* er_float_t of src/types.cuh:46-49 (frac, exp), 16 bytes */
struct er_t {
    double frac;
    long long exp;
};

constexpr int kScaleBits = 30; /* RNS_P2_SCALING_THRESHOLD of every predefined set */

template <int N>
struct Tables {
    int moduli[N];
    uint32_t mu[N];          /* Barrett factor floor(2^62 / m_i) */
    int part_inv[N];         /* RNS_PART_MODULI_PRODUCT_INVERSE: (M/m_i)^-1 mod m_i */
    double recip_rd[N];      /* RNS_MODULI_RECIP_RD */
    double recip_ru[N];      /* RNS_MODULI_RECIP_RU */
    int part_pow2_res30[N];  /* (M/m_i) mod 2^30; rows j < 30 of RNS_PART_MODULI_PRODUCT_POW2_RESIDUES are its low j bits */
    int m_pow2_res30;        /* M mod 2^30, likewise for RNS_MODULI_PRODUCT_POW2_RESIDUES */
    int mrc_inv[N][N];       /* MRC_MULT_INV: m_i^-1 mod m_j for j > i */
    double eval_acc;         /* RNS_EVAL_ACCURACY */
    int ref_factor;          /* RNS_EVAL_REF_FACTOR */
    int mp_h, mp_j, mp_precision, log2m;
    er_t unit_low, unit_upp;         /* RNS_EVAL_UNIT */
    er_t inv_unit_low, inv_unit_upp; /* RNS_EVAL_INV_UNIT */
    const int *pow2;     /* device: RNS_POW2[(log2m + 1)][N], 2^r mod m_i */
    const int *pow2_inv; /* device: RNS_POW2_INVERSE[30][N], (2^(r+1))^-1 mod m_i */
    /* integer forms for the fixed-point evaluation (fixed_eval.cuh) */
    uint64_t recip_rd_m[N];      /* RNS_MODULI_RECIP_RD[i] = recip_rd_m[i] * 2^-83 */
    uint64_t recip_ru_m[N];      /* RNS_MODULI_RECIP_RU[i] = recip_ru_m[i] * 2^-83 */
    uint64_t eval_acc_fx[2];     /* ceil(RNS_EVAL_ACCURACY * 2^83) as {low, high} 64-bit words */
    double unit_upp_recip;       /* nearest double to 1 / RNS_EVAL_UNIT.upp.frac */
    double unit_low_recip;       /* nearest double to 1 / RNS_EVAL_UNIT.low.frac */
    uint64_t unit_upp_inv;       /* floor(2^116 / Z), Z the 53-bit significand of RNS_EVAL_UNIT.upp.frac, at most 2^64-1 */
    uint64_t unit_low_inv;       /* the same for RNS_EVAL_UNIT.low.frac */
    const int *ceil_log2_pow2;   /* device: ceil(log2(2^e)) by CUDA's log2, e = -1074..1023 */
    /* the host conversion (double -> mp_float_t) replayed on the device */
    double recip_rn[N];          /* 1.0 / m_i rounded to nearest, as the host computes it */
    const int *host_ceil_log2;   /* device: host_ceil_log2_table() */
    uint32_t pow2_32[N];         /* 2^32 mod m_i: folds a 64-bit residue accumulator */
    uint64_t inv94[N];           /* floor(2^94 / m_i), 2^63 < inv94 < 2^64: the exact rank shortcut */
    uint32_t pow2_neg_top[N];    /* 2^-log2m mod m_i: 2^e for -log2m <= e < 0 as an RNS_POW2 row times this */
};

/* Host-side copy of every table in the reference's array shapes. */
struct HostTables {
    int n = 0, log2m = 0;
    int moduli[32];
    uint32_t mu[32];
    int part_inv[32];
    double recip_rd[32], recip_ru[32];
    int m_pow2_res[kScaleBits];
    int part_pow2_res[kScaleBits][32];
    int pow2_inv[kScaleBits][32];
    int mrc_inv[32][32];
    double eval_acc = 0;
    int ref_factor = 0, mp_h = 0, mp_j = 0, mp_precision = 0;
    er_t unit_low, unit_upp, inv_unit_low, inv_unit_upp;
    int *pow2 = nullptr; /* host, (log2m + 1) * n */
    uint64_t recip_rd_m[32], recip_ru_m[32], eval_acc_fx[2]; /* the Tables<N> integer forms */
    double unit_upp_recip = 0, unit_low_recip = 0;
    uint64_t unit_upp_inv = 0, unit_low_inv = 0;
};

/* Computes every table of the predefined set of n moduli (n in {8, 16, 32});
 * returns false for other sizes. */
bool compute_host_tables(int n, HostTables &t);

/* ceil(std::log2(x)) of the host just above powers of two (host_convert.cpp);
 * 2 * kHostLog2Entries ints */
constexpr int kHostLog2Entries = 1023;
bool host_ceil_log2_table(int *out);

} // namespace mpres

#endif
