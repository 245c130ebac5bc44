/*
 * Minimal GMP declarations for compiling the reference library's host code
 * against the runtime-only libgmp.so.10 of this image (no development headers
 * are installed).  Written from the public GMP manual: the mpz_t layout and the
 * documented entry points, mapped onto the library's exported `__gmpz_*` names.
 *
 * Test infrastructure only: used to build the reference for the CPU under
 * oracle/_ref/, never by the product library.
 */
#ifndef ORACLE_SHIM_GMP_H
#define ORACLE_SHIM_GMP_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;
typedef long mp_exp_t;
typedef unsigned long mp_bitcnt_t;

typedef struct {
    int _mp_alloc;
    int _mp_size;
    mp_limb_t *_mp_d;
} __mpz_struct;

typedef __mpz_struct mpz_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;

/* random state: only its storage size matters to the reference's headers */
typedef struct { char _opaque[64]; } __gmp_randstate_struct;
typedef __gmp_randstate_struct gmp_randstate_t[1];

void __gmpz_init(mpz_ptr);
void __gmpz_init2(mpz_ptr, mp_bitcnt_t);
void __gmpz_clear(mpz_ptr);
void __gmpz_set(mpz_ptr, mpz_srcptr);
void __gmpz_set_ui(mpz_ptr, unsigned long);
void __gmpz_set_si(mpz_ptr, long);
int __gmpz_set_str(mpz_ptr, const char *, int);
char *__gmpz_get_str(char *, int, mpz_srcptr);
unsigned long __gmpz_get_ui(mpz_srcptr);
long __gmpz_get_si(mpz_srcptr);
void __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mul_si(mpz_ptr, mpz_srcptr, long);
void __gmpz_fdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long __gmpz_fdiv_q_ui(mpz_ptr, mpz_srcptr, unsigned long);
unsigned long __gmpz_fdiv_r_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mod(mpz_ptr, mpz_srcptr, mpz_srcptr);
int __gmpz_cmp_ui(mpz_srcptr, unsigned long);
void __gmp_get_memory_functions(void *(**)(size_t), void *(**)(void *, size_t, size_t),
                                void (**)(void *, size_t));
int __gmp_printf(const char *, ...);

#ifdef __cplusplus
}
#endif

#define mpz_init __gmpz_init
#define mpz_init2 __gmpz_init2
#define mpz_clear __gmpz_clear
#define mpz_set __gmpz_set
#define mpz_set_ui __gmpz_set_ui
#define mpz_set_si __gmpz_set_si
#define mpz_set_str __gmpz_set_str
#define mpz_get_str __gmpz_get_str
#define mpz_get_ui __gmpz_get_ui
#define mpz_get_si __gmpz_get_si
#define mpz_add __gmpz_add
#define mpz_add_ui __gmpz_add_ui
#define mpz_sub __gmpz_sub
#define mpz_mul __gmpz_mul
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_mul_si __gmpz_mul_si
#define mpz_fdiv_q __gmpz_fdiv_q
#define mpz_fdiv_q_ui __gmpz_fdiv_q_ui
#define mpz_fdiv_r_ui __gmpz_fdiv_r_ui
#define mpz_div_ui __gmpz_fdiv_q_ui
#define mpz_mod_ui __gmpz_fdiv_r_ui
#define mpz_mod __gmpz_mod
#define mpz_cmp_ui __gmpz_cmp_ui
#define mp_get_memory_functions __gmp_get_memory_functions
#define gmp_printf __gmp_printf

#endif
