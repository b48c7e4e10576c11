// fsg_mp.h -- the part of the MPFR 4.2 / MPC 1.3 C API this library calls,
// declared here because the system provides the shared libraries
// (libmpfr.so.6, libmpc.so.3, as dependencies of gcc) without their headers.
//
// Layout and calling convention of the public API on LP64 Linux (x86_64 and
// aarch64): mpfr_prec_t and mpfr_exp_t are long, a limb is 64 bits, a
// complex number is two mpfr numbers (real part first).  Only true functions
// are called (the headers also define some of them as macros).
#pragma once

#include <cstddef>

extern "C" {

typedef long fsg_mpfr_prec_t;
typedef long fsg_mpfr_exp_t;
typedef int fsg_mpfr_sign_t;

typedef struct {
    fsg_mpfr_prec_t prec;
    fsg_mpfr_sign_t sign;
    fsg_mpfr_exp_t exp;
    unsigned long *limbs;
} fsg_mpfr_struct;

typedef fsg_mpfr_struct *fsg_mpfr_ptr;
typedef const fsg_mpfr_struct *fsg_mpfr_srcptr;

typedef struct {
    fsg_mpfr_struct re[1];
    fsg_mpfr_struct im[1];
} fsg_mpc_struct;

typedef fsg_mpc_struct *fsg_mpc_ptr;
typedef const fsg_mpc_struct *fsg_mpc_srcptr;

typedef int fsg_mpfr_rnd_t;   // 0: round to nearest (MPFR_RNDN)
typedef int fsg_mpc_rnd_t;    // 0: nearest for both parts (MPC_RNDNN)

// MPFR
void mpfr_init2(fsg_mpfr_ptr, fsg_mpfr_prec_t);
void mpfr_clear(fsg_mpfr_ptr);
int mpfr_set_str(fsg_mpfr_ptr, const char *, int, fsg_mpfr_rnd_t);
int mpfr_set_si(fsg_mpfr_ptr, long, fsg_mpfr_rnd_t);
int mpfr_set_d(fsg_mpfr_ptr, double, fsg_mpfr_rnd_t);
int mpfr_set(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
double mpfr_get_d(fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
double mpfr_get_d_2exp(long *, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
char *mpfr_get_str(char *, fsg_mpfr_exp_t *, int, size_t, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
void mpfr_free_str(char *);
int mpfr_sqr(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_mul(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_add(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_sub(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_abs(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_mul_si(fsg_mpfr_ptr, fsg_mpfr_srcptr, long, fsg_mpfr_rnd_t);
int mpfr_add_si(fsg_mpfr_ptr, fsg_mpfr_srcptr, long, fsg_mpfr_rnd_t);
int mpfr_ui_div(fsg_mpfr_ptr, unsigned long, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_hypot(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_rec_sqrt(fsg_mpfr_ptr, fsg_mpfr_srcptr, fsg_mpfr_rnd_t);
int mpfr_sgn(fsg_mpfr_srcptr);
int mpfr_cmp(fsg_mpfr_srcptr, fsg_mpfr_srcptr);
int mpfr_cmp_d(fsg_mpfr_srcptr, double);
int mpfr_greaterequal_p(fsg_mpfr_srcptr, fsg_mpfr_srcptr);

// MPC
void mpc_init2(fsg_mpc_ptr, fsg_mpfr_prec_t);
void mpc_clear(fsg_mpc_ptr);
int mpc_set_fr_fr(fsg_mpc_ptr, fsg_mpfr_srcptr, fsg_mpfr_srcptr, fsg_mpc_rnd_t);
int mpc_set_si_si(fsg_mpc_ptr, long, long, fsg_mpc_rnd_t);
int mpc_sqr(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_add(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_sub(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_mul(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_div(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_mul_si(fsg_mpc_ptr, fsg_mpc_srcptr, long, fsg_mpc_rnd_t);
int mpc_mul_ui(fsg_mpc_ptr, fsg_mpc_srcptr, unsigned long, fsg_mpc_rnd_t);
int mpc_mul_fr(fsg_mpc_ptr, fsg_mpc_srcptr, fsg_mpfr_srcptr, fsg_mpc_rnd_t);
int mpc_add_ui(fsg_mpc_ptr, fsg_mpc_srcptr, unsigned long, fsg_mpc_rnd_t);
int mpc_pow_ui(fsg_mpc_ptr, fsg_mpc_srcptr, unsigned long, fsg_mpc_rnd_t);
int mpc_pow_d(fsg_mpc_ptr, fsg_mpc_srcptr, double, fsg_mpc_rnd_t);
int mpc_ui_div(fsg_mpc_ptr, unsigned long, fsg_mpc_srcptr, fsg_mpc_rnd_t);
int mpc_abs(fsg_mpfr_ptr, fsg_mpc_srcptr, fsg_mpfr_rnd_t);
int mpc_norm(fsg_mpfr_ptr, fsg_mpc_srcptr, fsg_mpfr_rnd_t);
void mpc_swap(fsg_mpc_ptr, fsg_mpc_ptr);

}  // extern "C"
