/*
 * Minimal MPFR declarations for compiling the reference library's host code
 * against the runtime-only libmpfr.so.6 of this image.  Written from the public
 * MPFR manual: the mpfr_t layout, the rounding-mode enumeration and the
 * documented functions the reference's constant set-up and conversions call.
 *
 * Test infrastructure only (the oracle/_ref/ build and the MPFR baseline
 * oracle/mpfr_blas.c), never used by the product.
 */
#ifndef ORACLE_SHIM_MPFR_H
#define ORACLE_SHIM_MPFR_H

#include "gmp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;

typedef struct {
    mpfr_prec_t _mpfr_prec;
    mpfr_sign_t _mpfr_sign;
    mpfr_exp_t _mpfr_exp;
    mp_limb_t *_mpfr_d;
} __mpfr_struct;

typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct *mpfr_ptr;
typedef const __mpfr_struct *mpfr_srcptr;

typedef enum {
    MPFR_RNDN = 0,
    MPFR_RNDZ,
    MPFR_RNDU,
    MPFR_RNDD,
    MPFR_RNDA,
    MPFR_RNDF,
    MPFR_RNDNA = -1
} mpfr_rnd_t;

void mpfr_init(mpfr_ptr);
void mpfr_init2(mpfr_ptr, mpfr_prec_t);
void mpfr_clear(mpfr_ptr);
int mpfr_set4(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t, int);
int mpfr_set_ui(mpfr_ptr, unsigned long, mpfr_rnd_t);
int mpfr_set_d(mpfr_ptr, double, mpfr_rnd_t);
int mpfr_set_z(mpfr_ptr, mpz_srcptr, mpfr_rnd_t);
int mpfr_set_str(mpfr_ptr, const char *, int, mpfr_rnd_t);
int mpfr_add(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sub(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul_d(mpfr_ptr, mpfr_srcptr, double, mpfr_rnd_t);
int mpfr_div(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sqrt(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_log2(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
long mpfr_get_si(mpfr_srcptr, mpfr_rnd_t);
unsigned long mpfr_get_ui(mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d(mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d_2exp(long *, mpfr_srcptr, mpfr_rnd_t);
char *mpfr_get_str(char *, mpfr_exp_t *, int, size_t, mpfr_srcptr, mpfr_rnd_t);
void mpfr_free_str(char *);
mpfr_exp_t mpfr_get_z_2exp(mpz_ptr, mpfr_srcptr);

#ifdef __cplusplus
}
#endif

#define mpfr_set(a, b, r) mpfr_set4((a), (b), (r), (b)->_mpfr_sign)
#define mpfr_get_z_exp mpfr_get_z_2exp

#endif
