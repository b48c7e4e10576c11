/*
 * fsghost.h -- C-ABI of the arbitrary-precision host side: reference orbit,
 * ball-method period search, Newton nucleus search and nucleus size
 * estimate, on MPFR / MPC like the reference's Cython module.
 *
 * Each entry point replaces one function of the reference's
 * mpmath_utils/FP_loop.pyx (paths relative to src/fractalshades/) with the
 * same sequence of MPFR / MPC calls at the same precisions, so that its
 * results are those of the reference:
 *
 *   fsh_orbit_mn        <- perturbation_mandelbrot_FP_loop,
 *                          perturbation_mandelbrotN_FP_loop (FP_loop.pyx:237-421)
 *   fsh_orbit_bs        <- perturbation_nonholomorphic_FP_loop (:1828-1979)
 *   fsh_ball_mn         <- perturbation_mandelbrot(N)_ball_method (:605-760)
 *   fsh_ball_bs         <- perturbation_nonholomorphic_ball_method (:2357-2563)
 *   fsh_nucleus_m2      <- perturbation_mandelbrot_find_nucleus (:900-1116)
 *   fsh_any_nucleus_mn  <- perturbation_mandelbrot(N)_find_any_nucleus (:1119-1340)
 *   fsh_any_nucleus_bs  <- perturbation_nonholomorphic_find_any_nucleus (:2564-2756)
 *   fsh_size_mn         <- perturbation_mandelbrot(N)_nucleus_size_estimate (:457-604)
 *   fsh_size_bs         <- perturbation_nonholomorphic_nucleus_size_estimate (:1982-2100)
 *
 * Seeds are decimal strings (the reference's str(x).encode()); precisions
 * are in bits.  Arbitrary-precision results are returned exactly as
 * hexadecimal digit strings: value = sign * 0.d1 d2 ... (base 16) * 16^exp
 * (mpfr_get_str in base 16).  Xrange values are (mantissa, exponent) pairs
 * of mpfr_get_d_2exp, as the reference's mpc_t_to_Xrange (:424-456).
 * Functions return FSH_OK (or a count / index as stated) or a negative error
 * code; none throws.  They hold no global state and may run concurrently on
 * different threads.
 */
#ifndef FSGHOST_H
#define FSGHOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSH_OK 0
#define FSH_ERR_ARG (-1)      /* bad argument (seed string, precision, sizes) */
#define FSH_ERR_NOMEM (-3)

typedef struct fsh_registers fsh_registers;

/* The registers an orbit computation fills: the Xrange register (iterations
 * whose orbit value is below 1e-300 in modulus (M2, Mn) or in either
 * coordinate (Burning Ship), recorded only when asked for) and the partials
 * register (successive minima of |Z_n| below 1e-5).  Each entry holds the
 * iteration index and the (mantissa, exponent) pairs of the real and
 * imaginary parts (x and y for the Burning Ship family). */
int64_t fsh_registers_count(const fsh_registers *r, int32_t which);  /* 0 xr, 1 partials */
int fsh_registers_copy(const fsh_registers *r, int32_t which, int64_t *idx,
                       double *mantissas /* [2 * count] x, y interleaved */,
                       int64_t *exponents /* [2 * count] */);
void fsh_registers_free(fsh_registers *r);

/* Orbit of z -> z^exponent + c from z_0 = 0 (exponent 2: mpc_sqr, above:
 * mpc_pow_ui).  orbit: complex128 [max_iter + 1], orbit[0] = 0.  Stops after
 * the first |z_i| > M (double hypot of the rounded parts).  Returns the
 * reference's exit index i (max_iter + 1 when no escape) and *regs, to be
 * released with fsh_registers_free. */
int64_t fsh_orbit_mn(const char *seed_x, const char *seed_y, int64_t prec, int64_t max_iter,
                     uint32_t exponent, double M, int32_t need_xr, double *orbit,
                     fsh_registers **regs);

/* Burning Ship family orbit, flavor kind 1..5 (FP_loop.pyx:1343-1455):
 * (x, y) -> f_kind(x, y) + (a, -b). */
int64_t fsh_orbit_bs(const char *seed_x, const char *seed_y, int64_t prec, int64_t max_iter,
                     int32_t kind, double M, int32_t need_xr, double *orbit,
                     fsh_registers **regs);

/* First i <= maxiter with |z_i / (dz_i/dc)| / px < 1 (the ratio's modulus
 * rounded to 54 bits); 0 when the orbit escapes |z| > M_divergence first or
 * none is found (the reference returns -1 there); < 0 on error. */
int64_t fsh_ball_mn(const char *seed_x, const char *seed_y, int64_t prec, const char *seed_px,
                    uint32_t exponent, int64_t maxiter, double M_divergence);
/* Same with the 2 x 2 Jacobian: both |r_x|, |r_y| < 1 and hypot(r_x, r_y) < 1. */
int64_t fsh_ball_bs(const char *seed_x, const char *seed_y, int64_t prec, const char *seed_px,
                    int32_t kind, int64_t maxiter, double M_divergence);

/* Newton search of a period-order nucleus.  Writes the final c (hex digit
 * strings of at most out_len bytes including the terminating 0, and their
 * base-16 exponents) whether or not it converged; returns 1 when Newton
 * converged to a valid nucleus (|step| <= 64 eps_cv, then |z_order| <=
 * eps_valid, both at 54 bits), 0 when not, < 0 on error. */
int fsh_nucleus_m2(const char *seed_x, const char *seed_y, int64_t prec, int64_t order,
                   int64_t max_newton, const char *seed_eps_cv, const char *seed_eps_valid,
                   char *out_x, char *out_y, int64_t out_len, int64_t *exp_x, int64_t *exp_y);
int fsh_any_nucleus_mn(const char *seed_x, const char *seed_y, int64_t prec, uint32_t exponent,
                       int64_t order, int64_t max_newton, const char *seed_eps_cv,
                       const char *seed_eps_valid, char *out_x, char *out_y, int64_t out_len,
                       int64_t *exp_x, int64_t *exp_y);
int fsh_any_nucleus_bs(const char *seed_x, const char *seed_y, int64_t prec, int32_t kind,
                       int64_t order, int64_t max_newton, const char *seed_eps_cv,
                       const char *seed_eps_valid, char *out_x, char *out_y, int64_t out_len,
                       int64_t *exp_x, int64_t *exp_y);

/* Size estimate 1 / (b l^(n/(n-1))) of the period-order component (l^2 for
 * n = 2) as a complex Xrange: out[0] = re mantissa, out[1] = im mantissa,
 * eout[0], eout[1] their exponents. */
int fsh_size_mn(const char *seed_x, const char *seed_y, int64_t prec, uint32_t exponent,
                int64_t order, double *out, int64_t *eout);
/* Burning Ship: size (mantissa out[0], exponent eout[0]) and the skew matrix
 * skew[4] = {b_yy, b_xy, b_yx, b_xx} / sqrt(det b) (row-major 2 x 2). */
int fsh_size_bs(const char *seed_x, const char *seed_y, int64_t prec, int32_t kind,
                int64_t order, double *out, int64_t *eout, double *skew);

#ifdef __cplusplus
}
#endif

#endif
