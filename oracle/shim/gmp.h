/* Declaration-only stand-in for <gmp.h> (GMP 6.x public API).
 *
 * TEST INFRASTRUCTURE (oracle): lets the unmodified MDZ sources and the
 * oracle restatement compile in an image that ships libgmp.so.10 but no
 * development headers.  Only the types and functions that MDZ's hot path
 * names are declared; the struct layout and the __gmpf_* link names follow
 * the GMP manual ("Floating-point Functions") and libgmp's exported symbols.
 * Nothing here is compiled into the product library. */
#ifndef MDZ_SHIM_GMP_H
#define MDZ_SHIM_GMP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define __GNU_MP_VERSION 6
#define __GNU_MP_VERSION_MINOR 3

typedef unsigned long mp_limb_t;
typedef long mp_exp_t;
typedef unsigned long mp_bitcnt_t;
typedef long mp_size_t;

/* value = sign(_mp_size) * sum_i _mp_d[i] * 2^(64*(i - |_mp_size| + _mp_exp)) */
typedef struct {
    int _mp_prec;        /* limbs of precision, minus one */
    int _mp_size;        /* signed count of used limbs */
    mp_exp_t _mp_exp;    /* exponent, in limbs */
    mp_limb_t* _mp_d;    /* limbs, least significant first */
} __mpf_struct;

typedef __mpf_struct mpf_t[1];
typedef __mpf_struct* mpf_ptr;
typedef const __mpf_struct* mpf_srcptr;

#define mpf_init2    __gmpf_init2
#define mpf_clear    __gmpf_clear
#define mpf_set      __gmpf_set
#define mpf_set_si   __gmpf_set_si
#define mpf_set_str  __gmpf_set_str
#define mpf_set_prec __gmpf_set_prec
#define mpf_get_prec __gmpf_get_prec
#define mpf_add      __gmpf_add
#define mpf_sub      __gmpf_sub
#define mpf_mul      __gmpf_mul
#define mpf_mul_ui   __gmpf_mul_ui
#define mpf_div      __gmpf_div
#define mpf_ui_div   __gmpf_ui_div
#define mpf_abs      __gmpf_abs
#define mpf_cmp      __gmpf_cmp

void __gmpf_init2(mpf_ptr, mp_bitcnt_t);
void __gmpf_clear(mpf_ptr);
void __gmpf_set(mpf_ptr, mpf_srcptr);
void __gmpf_set_si(mpf_ptr, long);
int  __gmpf_set_str(mpf_ptr, const char*, int);
void __gmpf_set_prec(mpf_ptr, mp_bitcnt_t);
mp_bitcnt_t __gmpf_get_prec(mpf_srcptr);
void __gmpf_add(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_sub(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul_ui(mpf_ptr, mpf_srcptr, unsigned long);
void __gmpf_div(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_ui_div(mpf_ptr, unsigned long, mpf_srcptr);
void __gmpf_abs(mpf_ptr, mpf_srcptr);
int  __gmpf_cmp(mpf_srcptr, mpf_srcptr);

#ifdef __cplusplus
}
#endif
#endif
