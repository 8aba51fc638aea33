/* Declaration-only stand-in for <mpfr.h> (MPFR 4.x public API).
 *
 * TEST INFRASTRUCTURE (oracle): lets the unmodified MDZ sources and the
 * oracle restatement compile against the system libmpfr.so.6 when no
 * development headers are installed.  Only what MDZ's hot path and its
 * coordinate code name is declared; the layout of __mpfr_struct and the
 * special-exponent encoding follow the MPFR manual ("Nomenclature and
 * Types", "Internals").  MDZ_SHIM_LD_AS_D maps mpfr_get_ld to mpfr_get_d,
 * which is how the double-precision ("FP64") build of the reference is made
 * on x86-64 together with -mlong-double-64. */
#ifndef MDZ_SHIM_MPFR_H
#define MDZ_SHIM_MPFR_H

#include <stdio.h>
#include <stddef.h>
#include "gmp.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MPFR_VERSION_MAJOR 4
#define MPFR_VERSION_MINOR 2
#define MPFR_VERSION_PATCHLEVEL 1

typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;
typedef mpfr_prec_t mp_prec_t;

/* value = _mpfr_sign * 0.d[n-1] d[n-2] ... d[0] (binary) * 2^_mpfr_exp,
 * n = ceil(_mpfr_prec / 64), most significant limb last, top bit set.
 * Zero / NaN / Inf are flagged by _mpfr_exp = LONG_MIN+1 / +2 / +3. */
typedef struct {
    mpfr_prec_t _mpfr_prec;
    mpfr_sign_t _mpfr_sign;
    mpfr_exp_t _mpfr_exp;
    mp_limb_t* _mpfr_d;
} __mpfr_struct;

typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct* mpfr_ptr;
typedef const __mpfr_struct* mpfr_srcptr;

typedef enum {
    MPFR_RNDN = 0, MPFR_RNDZ, MPFR_RNDU, MPFR_RNDD, MPFR_RNDA, MPFR_RNDF,
    MPFR_RNDNA = -1
} mpfr_rnd_t;
typedef mpfr_rnd_t mp_rnd_t;
#define GMP_RNDN MPFR_RNDN
#define GMP_RNDZ MPFR_RNDZ
#define GMP_RNDU MPFR_RNDU
#define GMP_RNDD MPFR_RNDD

void mpfr_init2(mpfr_ptr, mpfr_prec_t);
void mpfr_clear(mpfr_ptr);
void mpfr_set_prec(mpfr_ptr, mpfr_prec_t);
mpfr_prec_t mpfr_get_prec(mpfr_srcptr);
int mpfr_prec_round(mpfr_ptr, mpfr_prec_t, mpfr_rnd_t);
int mpfr_set(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_set_si(mpfr_ptr, long, mpfr_rnd_t);
int mpfr_set_d(mpfr_ptr, double, mpfr_rnd_t);
int mpfr_set_str(mpfr_ptr, const char*, int, mpfr_rnd_t);
int mpfr_add(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sub(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sqr(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_div(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul_si(mpfr_ptr, mpfr_srcptr, long, mpfr_rnd_t);
int mpfr_div_si(mpfr_ptr, mpfr_srcptr, long, mpfr_rnd_t);
int mpfr_div_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_si_div(mpfr_ptr, long, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul_d(mpfr_ptr, mpfr_srcptr, double, mpfr_rnd_t);
int mpfr_div_d(mpfr_ptr, mpfr_srcptr, double, mpfr_rnd_t);
int mpfr_abs(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_neg(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_log2(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_greater_p(mpfr_srcptr, mpfr_srcptr);
int mpfr_cmp(mpfr_srcptr, mpfr_srcptr);
int mpfr_zero_p(mpfr_srcptr);
int mpfr_nan_p(mpfr_srcptr);
int mpfr_inf_p(mpfr_srcptr);
long mpfr_get_si(mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d(mpfr_srcptr, mpfr_rnd_t);
#ifdef MDZ_SHIM_LD_AS_D
#define mpfr_get_ld(x, r) mpfr_get_d((x), (r))
#else
long double mpfr_get_ld(mpfr_srcptr, mpfr_rnd_t);
#endif
mpfr_exp_t mpfr_get_exp(mpfr_srcptr);
char* mpfr_get_str(char*, mpfr_exp_t*, int, size_t, mpfr_srcptr, mpfr_rnd_t);
void mpfr_free_str(char*);
void mpfr_free_cache(void);
int mpfr_printf(const char*, ...);
/* the stream functions are exported under these names (they take a FILE*) */
#define mpfr_out_str __gmpfr_out_str
#define mpfr_fprintf __gmpfr_fprintf
size_t __gmpfr_out_str(FILE*, int, size_t, mpfr_srcptr, mpfr_rnd_t);
int __gmpfr_fprintf(FILE*, const char*, ...);
int mpfr_snprintf(char*, size_t, const char*, ...);
const char* mpfr_get_version(void);

#define MPFR_SIGN(x) ((x)->_mpfr_sign)

#ifdef __cplusplus
}
#endif
#endif
