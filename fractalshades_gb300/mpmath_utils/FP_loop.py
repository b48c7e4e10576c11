"""
Arbitrary-precision host functions with the entry points, arguments and
results of the reference's Cython module ``mpmath_utils/FP_loop.pyx``:
reference orbit, ball-method period search, Newton nucleus search and
nucleus size estimate for the power-2, power-n and Burning Ship models.

The arithmetic runs in libfsghost.so (csrc/host/fsg_host.cpp, declared in
include/fsghost.h) on MPFR / MPC, the libraries the reference links, with the
reference's sequence of calls and precisions.  This module converts the
results to the reference's Python types: mpmath numbers for nuclei and sizes,
Xrange values for the orbit registers.
"""
import mpmath
import numpy as np

from .. import _host
from ..numpy_utils.xrange import xr_from_mantissa_exp


def _xr_dict(entries):
    """{i: complex Xrange} from (i, mx, ex, my, ey) (mpc_t_to_Xrange,
    FP_loop.pyx:424-440)"""
    return {i: xr_from_mantissa_exp(mx, ex, my, ey) for (i, mx, ex, my, ey) in entries}


def _xy_dict(entries):
    """{i: ((mx, ex), (my, ey))}: the x and y Xrange values of the Burning
    Ship registers (FP_loop.pyx:1922-1951)"""
    return {i: ((mx, ex), (my, ey)) for (i, mx, ex, my, ey) in entries}


def _mpc(seed_prec, hx, hy):
    if hx is None or hy is None:
        return mpmath.mpc("nan", "nan")
    with mpmath.workprec(int(seed_prec)):
        return mpmath.mpc(mpmath.mpf(hx), mpmath.mpf(hy))


def _newton_result(seed_prec, r):
    ok, hx, hy = r
    if ok:
        return True, _mpc(seed_prec, hx, hy)
    return False, mpmath.mpc("nan", "nan")


# ---------------------------------------------------------------------------
# power-2 Mandelbrot (FP_loop.pyx:237-253, 457-470, 605-617, 900-1138)
# ---------------------------------------------------------------------------
def perturbation_mandelbrot_FP_loop(orbit, need_Xrange, max_iter, M, seed_x, seed_y,
                                    seed_prec):
    """Fill ``orbit`` (complex128 [max_iter + 1], or its float64 view) with
    z_n, z_0 = 0, z_{n+1} = z_n**2 + c.  Returns (i, partial_dict, xr_dict):
    the exit index (first invalid iteration), the successive minima of |z_n|
    below 1e-5 and, if need_Xrange, the iterations with |z_n| < 1e-300, both
    as Xrange values."""
    return perturbation_mandelbrotN_FP_loop(orbit, need_Xrange, max_iter, 2, M, seed_x,
                                            seed_y, seed_prec)


def perturbation_mandelbrot_ball_method(seed_x, seed_y, seed_prec, seed_px, maxiter,
                                        M_divergence):
    """First i such that the ball of radius px around c maps onto a ball
    containing 0 (|z_i / (dz_i/dc)| < px); -1 if none up to maxiter."""
    return _host.ball_mn(seed_x, seed_y, seed_prec, seed_px, 2, maxiter, M_divergence)


def perturbation_mandelbrot_find_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                         seed_eps_cv, seed_eps_valid):
    """Newton for f^order(0) = 0 with division by the roots of the divisor
    periods.  Returns (newton_cv, c)."""
    return _newton_result(seed_prec, _host.nucleus_m2(
        seed_x, seed_y, seed_prec, order, max_newton, seed_eps_cv, seed_eps_valid))


def perturbation_mandelbrot_find_any_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                             seed_eps_cv, seed_eps_valid):
    """Newton for f^order(0) = 0 accepting divisor periods."""
    return perturbation_mandelbrotN_find_any_nucleus(seed_x, seed_y, seed_prec, 2, order,
                                                     max_newton, seed_eps_cv, seed_eps_valid)


def perturbation_mandelbrot_nucleus_size_estimate(seed_x, seed_y, seed_prec, order):
    """Size estimate 1 / (beta lambda^2) of the period-``order`` component at
    c (lambda = dz_p/dz, beta = 1 + sum_i 1 / prod_{j<=i} dz_j/dz), complex."""
    return perturbation_mandelbrotN_nucleus_size_estimate(seed_x, seed_y, seed_prec, 2, order)


# ---------------------------------------------------------------------------
# power-n Mandelbrot (FP_loop.pyx:255-421, 472-604, 618-760, 1139-1340)
# ---------------------------------------------------------------------------
def _check_exponent(exponent):
    exponent = int(exponent)
    if exponent < 2:
        raise NotImplementedError(exponent)
    return exponent


def perturbation_mandelbrotN_FP_loop(orbit, need_Xrange, max_iter, exponent, M, seed_x,
                                     seed_y, seed_prec):
    """Orbit of z_{n+1} = z_n**exponent + c, z_0 = 0; outputs as
    perturbation_mandelbrot_FP_loop."""
    n = _check_exponent(exponent)
    i, xr, partials = _host.orbit_mn(orbit, need_Xrange, max_iter, n, M, seed_x, seed_y,
                                     seed_prec)
    return i, _xr_dict(partials), _xr_dict(xr)


def perturbation_mandelbrotN_ball_method(seed_x, seed_y, seed_prec, seed_px, exponent, maxiter,
                                         M_divergence):
    return _host.ball_mn(seed_x, seed_y, seed_prec, seed_px, _check_exponent(exponent), maxiter,
                         M_divergence)


def perturbation_mandelbrotN_find_any_nucleus(seed_x, seed_y, seed_prec, exponent, order,
                                              max_newton, seed_eps_cv, seed_eps_valid):
    return _newton_result(seed_prec, _host.any_nucleus_mn(
        seed_x, seed_y, seed_prec, _check_exponent(exponent), order, max_newton, seed_eps_cv,
        seed_eps_valid))


def perturbation_mandelbrotN_nucleus_size_estimate(seed_x, seed_y, seed_prec, exponent, order):
    """1 / (b l**(n / (n - 1))) (l**2 for n = 2), complex (mpmath)."""
    (mx, ex), (my, ey) = _host.size_mn(seed_x, seed_y, seed_prec, _check_exponent(exponent),
                                       order)
    with mpmath.workprec(int(seed_prec)):
        return mpmath.mpc(mpmath.ldexp(mx, ex), mpmath.ldexp(my, ey))


# ---------------------------------------------------------------------------
# Burning Ship family (FP_loop.pyx:1343-2100, 2357-2756)
# ---------------------------------------------------------------------------
def perturbation_nonholomorphic_FP_loop(orbit, need_Xrange, max_iter, M, seed_x, seed_y,
                                        seed_prec, kind=1):
    """Orbit (x_{n+1}, y_{n+1}) = f_kind(x_n, y_n) + (a, -b) of flavor kind
    1..5.  Returns (i, partial_dict, xr_dict), the registers holding
    ((mx, ex), (my, ey)) pairs; the Xrange register (if need_Xrange) the
    iterations where |x| or |y| < 1e-300."""
    i, xr, partials = _host.orbit_bs(orbit, need_Xrange, max_iter, int(kind), M, seed_x,
                                     seed_y, seed_prec)
    return i, _xy_dict(partials), _xy_dict(xr)


def perturbation_nonholomorphic_ball_method(seed_x, seed_y, seed_prec, seed_px, maxiter,
                                            M_divergence, kind=1):
    """Period from the 2 x 2 Jacobian ball method; -1 if none."""
    return _host.ball_bs(seed_x, seed_y, seed_prec, seed_px, int(kind), maxiter, M_divergence)


def perturbation_nonholomorphic_find_any_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                                 seed_eps_cv, seed_eps_valid, kind=1):
    """Newton on the 2 x 2 Jacobian for f^order(0) = 0.  Returns
    (newton_cv, c) with c = a + i b."""
    return _newton_result(seed_prec, _host.any_nucleus_bs(
        seed_x, seed_y, seed_prec, int(kind), order, max_newton, seed_eps_cv, seed_eps_valid))


def perturbation_nonholomorphic_nucleus_size_estimate(seed_x, seed_y, seed_prec, order, kind=1):
    """(size, skew): size = |det(L)^2 det(beta)|^(-1/2) with L the Jacobian of
    z_order w.r.t. z_1 and beta = I + sum_i L_i^-1, skew = beta / sqrt(det
    beta) as [[b_yy, b_xy], [b_yx, b_xx]]."""
    (m, e), skew = _host.size_bs(seed_x, seed_y, seed_prec, int(kind), order)
    with mpmath.workprec(int(seed_prec)):
        return mpmath.ldexp(m, e), np.array(skew, dtype=np.float64)
