"""
Fixed-point restatement of the reference's arbitrary-precision host functions
(mpmath_utils/FP_loop.pyx) -- TEST INFRASTRUCTURE: an independent check of
the package's MPFR implementation (fractalshades_gb300/csrc/host/fsg_host.cpp,
include/fsghost.h); only tests import it.

The arithmetic is binary fixed point on Python integers: a value v is held as
the integer round(v * 2**F) with F = seed_prec + 64 guard bits, so every
operation carries an absolute error below 2**-F, which is the accuracy that
matters for an iteration started from 0.  Results are returned as mpmath
numbers or float64 / Xrange values like the reference.  Where its Newton
iterate leaves the fixed-point range it takes one step in mpmath.
"""
import math

import mpmath
import numpy as np

from fractalshades_gb300.numpy_utils.xrange import xr_from_mantissa_exp

# settings.py:14 newton_zoom_level and :22 xrange_zoom_level (FP_loop.pyx:142-143)
PARTIAL_TSHOLD = 1.e-5
XR_TSHOLD = 1.e-300

GUARD_BITS = 64


# ---------------------------------------------------------------------------
# fixed point helpers
# ---------------------------------------------------------------------------
def _fix(v, F):
    """round(v * 2**F) for an mpmath number or a decimal string (parsed with
    F + 16 bits, like mpfr_set_str at the working precision)."""
    with mpmath.workprec(F + 16):
        v = mpmath.mpf(v)
    sign, man, exp, _bc = v._mpf_
    if sign:
        man = -man
    s = exp + F
    if s >= 0:
        return man << s
    # round to nearest
    return (man + (1 << (-s - 1))) >> (-s)


def _to_float(x, F):
    """float(x * 2**-F), correctly rounded (CPython's true division of
    integers rounds correctly, subnormal results included) like mpfr_get_d."""
    if x == 0:
        return 0.0
    return x / (1 << F)


def _to_mpf(x, F):
    return mpmath.mpf((x, -F)) if x else mpmath.mpf(0)


def _mantissa_exp(x, F):
    """(m, e) with x * 2**-F = m * 2**e, m in [0.5, 1) rounded to 53 bits
    (mpfr_get_d_2exp)."""
    if x == 0:
        return 0.0, 0
    b = abs(x).bit_length()
    m = x / (1 << b)                # correctly rounded, |m| in [0.5, 1]
    if abs(m) == 1.0:
        return m / 2, b - F + 1
    return m, b - F


def _xr_of(zx, zy, F):
    """Xrange (complex mantissa, shared exponent) of z, as mpc_t_to_Xrange
    (FP_loop.pyx:424-440) does through Xrange addition."""
    mx, ex = _mantissa_exp(zx, F)
    my, ey = _mantissa_exp(zy, F)
    return xr_from_mantissa_exp(mx, ex, my, ey)


def _sq_add(zx, zy, cx, cy, F):
    """z**2 + c"""
    return (((zx * zx - zy * zy) >> F) + cx, ((zx * zy) >> (F - 1)) + cy)


# ---------------------------------------------------------------------------
# reference orbit (FP_loop.pyx:274-421)
# ---------------------------------------------------------------------------
def perturbation_mandelbrot_FP_loop(orbit, need_Xrange, max_iter, M, seed_x, seed_y,
                                    seed_prec):
    """Fill ``orbit`` (complex128 of length max_iter + 1, or its float64 view)
    with the FP64 values of z_n, z_0 = 0, z_{n+1} = z_n**2 + c.

    Returns (i, partial_dict, xr_dict): the exit index (first invalid
    iteration), the successive minima of |z_n| below PARTIAL_TSHOLD and the
    iterations with |z_n| < XR_TSHOLD as Xrange (only if need_Xrange)."""
    orb = orbit.view(np.complex128) if orbit.dtype != np.complex128 else orbit
    if orb.shape[0] != max_iter + 1:
        raise ValueError("orbit length must be max_iter + 1")
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    zx, zy = 0, 0
    orb[0] = 0.
    xr_dict = {}
    partial_dict = {}
    curr_partial = PARTIAL_TSHOLD
    curr_partial2 = None
    i = 0
    abs_i = 0.
    for i in range(1, max_iter + 1):
        zx, zy = _sq_add(zx, zy, cx, cy, F)
        x, y = _to_float(zx, F), _to_float(zy, F)
        orb[i] = complex(x, y)
        abs_i = math.hypot(x, y)
        if abs_i > M:
            break
        if need_Xrange and abs_i < XR_TSHOLD:
            xr_dict[i] = _xr_of(zx, zy, F)
        if abs_i <= curr_partial:
            a2 = zx * zx + zy * zy
            if curr_partial2 is None or a2 < curr_partial2:
                partial_dict[i] = _xr_of(zx, zy, F)
                curr_partial2 = a2
                curr_partial = abs_i
    if i == max_iter and abs_i <= M:
        i += 1
    return i, partial_dict, xr_dict


# ---------------------------------------------------------------------------
# ball method (FP_loop.pyx:631-760)
# ---------------------------------------------------------------------------
def perturbation_mandelbrot_ball_method(seed_x, seed_y, seed_prec, seed_px, maxiter,
                                        M_divergence):
    """First i such that |z_i / (dz_i/dc)| < px (a ball of radius px around c
    maps onto a ball containing 0).  Returns -1 if none up to maxiter."""
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    px = _fix(_dec(seed_px), F)
    px2 = px * px
    one = 1 << F
    zx = zy = 0
    dx = dy = 0
    for i in range(1, maxiter + 1):
        # dzndc <- 2 z dzndc + 1 (iter_deriv_M2 with var_c_z = 0), then z <- z^2 + c
        dx, dy = ((zx * dx - zy * dy) >> (F - 1)) + one, ((zx * dy + zy * dx) >> (F - 1))
        zx, zy = _sq_add(zx, zy, cx, cy, F)
        if math.hypot(_to_float(zx, F), _to_float(zy, F)) > M_divergence:
            return -1
        # |z / dzndc| / px < 1  <=>  |z|^2 < px^2 |dzndc|^2
        z2 = zx * zx + zy * zy
        d2 = dx * dx + dy * dy
        if (z2 << (2 * F)) < px2 * d2:
            return i
    return -1


# ---------------------------------------------------------------------------
# Newton nucleus search (FP_loop.pyx:900-1116, 1119-1340)
# ---------------------------------------------------------------------------
def _cdiv(ax, ay, bx, by, F):
    """(a / b) in fixed point"""
    den = bx * bx + by * by
    if den == 0:
        raise ZeroDivisionError
    nx = ax * bx + ay * by
    ny = ay * bx - ax * by
    return (nx << F) // den, (ny << F) // den


def _cmul(ax, ay, bx, by, F):
    return (ax * bx - ay * by) >> F, (ax * by + ay * bx) >> F


def _newton_step_float(c, order, divide_divisors, prec):
    """One Newton step in floating point (mpmath at ``prec`` bits): used when
    the current c escapes, where fixed point would overflow."""
    with mpmath.workprec(prec):
        zr = mpmath.mpc(0)
        dz = mpmath.mpc(0)
        h = mpmath.mpc(1)
        dh = mpmath.mpc(0)
        for i in range(1, order + 1):
            dz = 2 * dz * zr + 1
            zr = zr * zr + c
            if divide_divisors and i < order and order % i == 0:
                h *= zr
                dh += dz / zr
        f = zr / h
        df = (dz - zr * dh) / h
        return f / df, zr


def _find_nucleus(seed_x, seed_y, seed_prec, order, max_newton, seed_eps_cv,
                  seed_eps_valid, divide_divisors):
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    eps_cv = mpmath.mpf(_dec(seed_eps_cv)) * 64
    eps_valid = mpmath.mpf(_dec(seed_eps_valid))
    one = 1 << F
    big = F + 64          # |z| > 2**64: the orbit escapes
    order = int(order)
    newton_cv = False
    for _ in range(int(max_newton)):
        zx = zy = 0
        dx = dy = 0
        hx, hy = one, 0
        dhx = dhy = 0
        escaped = False
        for i in range(1, order + 1):
            dx, dy = ((zx * dx - zy * dy) >> (F - 1)) + one, (zx * dy + zy * dx) >> (F - 1)
            zx, zy = _sq_add(zx, zy, cx, cy, F)
            if zx.bit_length() > big or zy.bit_length() > big:
                escaped = True
                break
            if divide_divisors and i < order and order % i == 0:
                hx, hy = _cmul(hx, hy, zx, zy, F)
                qx, qy = _cdiv(dx, dy, zx, zy, F)
                dhx, dhy = dhx + qx, dhy + qy
        if escaped:
            step_c, zr = _newton_step_float(
                mpmath.mpc(_to_mpf(cx, F), _to_mpf(cy, F)), order, divide_divisors, F)
            sx, sy = _fix(step_c.real, F), _fix(step_c.imag, F)
            cx, cy = cx - sx, cy - sy
            continue
        # f = zr / h ; df = (dzrdc - zr * dh) / h ; step = f / df
        fx, fy = _cdiv(zx, zy, hx, hy, F)
        tx, ty = _cmul(zx, zy, dhx, dhy, F)
        gx, gy = _cdiv(dx - tx, dy - ty, hx, hy, F)
        sx, sy = _cdiv(fx, fy, gx, gy, F)
        cx, cy = cx - sx, cy - sy
        step = mpmath.sqrt(_to_mpf(sx, F) ** 2 + _to_mpf(sy, F) ** 2)
        if step <= eps_cv:
            az = mpmath.sqrt(_to_mpf(zx, F) ** 2 + _to_mpf(zy, F) ** 2)
            newton_cv = az <= eps_valid
            break
    if newton_cv:
        return True, mpmath.mpc(_to_mpf(cx, F), _to_mpf(cy, F))
    return False, mpmath.mpc("nan", "nan")


def perturbation_mandelbrot_find_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                         seed_eps_cv, seed_eps_valid):
    """Newton for f^order(0) = 0 with division by the roots of the divisor
    periods (FP_loop.pyx:900-1116).  Returns (newton_cv, c)."""
    return _find_nucleus(seed_x, seed_y, seed_prec, order, max_newton, seed_eps_cv,
                         seed_eps_valid, True)


def perturbation_mandelbrot_find_any_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                             seed_eps_cv, seed_eps_valid):
    """Newton for f^order(0) = 0 accepting divisor periods (FP_loop.pyx:1119-1340)."""
    return _find_nucleus(seed_x, seed_y, seed_prec, order, max_newton, seed_eps_cv,
                         seed_eps_valid, False)


# ---------------------------------------------------------------------------
# nucleus size estimate (FP_loop.pyx:487-604)
# ---------------------------------------------------------------------------
def perturbation_mandelbrot_nucleus_size_estimate(seed_x, seed_y, seed_prec, order):
    """Size estimate of the hyperbolic component of period ``order`` at c
    (the renormalisation estimate 1 / (beta * lambda**2) of the reference,
    with lambda = dz_p/dz and beta = sum_i 1 / prod_{j<=i} dz_j/dz)."""
    with mpmath.workprec(int(seed_prec)):
        c = mpmath.mpc(_dec(seed_x), _dec(seed_y))
        z = mpmath.mpc(0)
        l = mpmath.mpc(1)
        b = mpmath.mpc(1)
        for _ in range(1, int(order)):
            z = z * z + c
            l = 2 * z * l
            b = b + 1 / l
        size = 1 / (b * l * l)
        return size


# ---------------------------------------------------------------------------
# power-n Mandelbrot, z -> z^n + c (FP_loop.pyx:167-235, 255-421, 472-604,
# 618-760, 1139-1340): mpc_pow_ui for z^n and n dzdc z^(n-1) (+ 1) for the
# derivative; exponent 2 runs the power-2 functions above.
# ---------------------------------------------------------------------------
def _pow_fix(zx, zy, n, F):
    """z**n in fixed point (binary powering), n >= 1"""
    rx, ry = None, None
    px, py = zx, zy
    while True:
        if n & 1:
            if rx is None:
                rx, ry = px, py
            else:
                rx, ry = _cmul(rx, ry, px, py, F)
        n >>= 1
        if not n:
            return rx, ry
        px, py = _cmul(px, py, px, py, F)


def _check_exponent(exponent):
    exponent = int(exponent)
    if exponent < 2:
        raise NotImplementedError(exponent)
    return exponent


def perturbation_mandelbrotN_FP_loop(orbit, need_Xrange, max_iter, exponent, M, seed_x,
                                     seed_y, seed_prec):
    """Orbit of z_{n+1} = z_n**exponent + c, z_0 = 0 (FP_loop.pyx:255-421):
    same outputs as perturbation_mandelbrot_FP_loop."""
    n = _check_exponent(exponent)
    if n == 2:
        return perturbation_mandelbrot_FP_loop(orbit, need_Xrange, max_iter, M, seed_x, seed_y,
                                               seed_prec)
    orb = orbit.view(np.complex128) if orbit.dtype != np.complex128 else orbit
    if orb.shape[0] != max_iter + 1:
        raise ValueError("orbit length must be max_iter + 1")
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    zx, zy = 0, 0
    orb[0] = 0.
    xr_dict = {}
    partial_dict = {}
    curr_partial = PARTIAL_TSHOLD
    curr_partial2 = None
    i = 0
    abs_i = 0.
    for i in range(1, max_iter + 1):
        px, py = _pow_fix(zx, zy, n, F)
        zx, zy = px + cx, py + cy
        x, y = _to_float(zx, F), _to_float(zy, F)
        orb[i] = complex(x, y)
        abs_i = math.hypot(x, y)
        if abs_i > M:
            break
        if need_Xrange and abs_i < XR_TSHOLD:
            xr_dict[i] = _xr_of(zx, zy, F)
        if abs_i <= curr_partial:
            a2 = zx * zx + zy * zy
            if curr_partial2 is None or a2 < curr_partial2:
                partial_dict[i] = _xr_of(zx, zy, F)
                curr_partial2 = a2
                curr_partial = abs_i
    if i == max_iter and abs_i <= M:
        i += 1
    return i, partial_dict, xr_dict


def perturbation_mandelbrotN_ball_method(seed_x, seed_y, seed_prec, seed_px, exponent, maxiter,
                                         M_divergence):
    """First i with |z_i / (dz_i/dc)| < px for z -> z**exponent + c
    (FP_loop.pyx:618-760), -1 if none up to maxiter."""
    n = _check_exponent(exponent)
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    px = _fix(_dec(seed_px), F)
    px2 = px * px
    one = 1 << F
    zx = zy = 0
    dx = dy = 0
    for i in range(1, maxiter + 1):
        # dzndc <- n dzndc z^(n-1) + 1 with the current z, then z <- z^n + c
        wx, wy = _pow_fix(zx, zy, n - 1, F)
        tx, ty = _cmul(dx, dy, wx, wy, F)
        dx, dy = n * tx + one, n * ty
        zx, zy = _cmul(wx, wy, zx, zy, F)
        zx, zy = zx + cx, zy + cy
        if math.hypot(_to_float(zx, F), _to_float(zy, F)) > M_divergence:
            return -1
        z2 = zx * zx + zy * zy
        d2 = dx * dx + dy * dy
        if (z2 << (2 * F)) < px2 * d2:
            return i
    return -1


def _newton_step_float_n(c, order, n, prec):
    """Newton step c -> c - z_order / (dz_order/dc) in floating point
    (mpmath at ``prec`` bits), for orbits that leave the fixed-point range."""
    with mpmath.workprec(prec):
        zr = mpmath.mpc(0)
        dz = mpmath.mpc(0)
        for _ in range(1, order + 1):
            dz = n * dz * zr ** (n - 1) + 1
            zr = zr ** n + c
        return zr / dz, zr


def perturbation_mandelbrotN_find_any_nucleus(seed_x, seed_y, seed_prec, exponent, order,
                                              max_newton, seed_eps_cv, seed_eps_valid):
    """Newton for f^order(0) = 0, f = z**exponent + c, divisor periods
    accepted (FP_loop.pyx:1139-1340).  Returns (newton_cv, c)."""
    n = _check_exponent(exponent)
    if n == 2:
        return perturbation_mandelbrot_find_any_nucleus(seed_x, seed_y, seed_prec, order,
                                                        max_newton, seed_eps_cv, seed_eps_valid)
    F = int(seed_prec) + GUARD_BITS
    cx, cy = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    eps_cv = mpmath.mpf(_dec(seed_eps_cv)) * 64
    eps_valid = mpmath.mpf(_dec(seed_eps_valid))
    one = 1 << F
    big = F + 64
    order = int(order)
    newton_cv = False
    for _ in range(int(max_newton)):
        zx = zy = 0
        dx = dy = 0
        escaped = False
        for i in range(1, order + 1):
            wx, wy = _pow_fix(zx, zy, n - 1, F)
            tx, ty = _cmul(dx, dy, wx, wy, F)
            dx, dy = n * tx + one, n * ty
            zx, zy = _cmul(wx, wy, zx, zy, F)
            zx, zy = zx + cx, zy + cy
            if zx.bit_length() > big or zy.bit_length() > big:
                escaped = True
                break
        if escaped:
            step_c, _zr = _newton_step_float_n(
                mpmath.mpc(_to_mpf(cx, F), _to_mpf(cy, F)), order, n, F)
            sx, sy = _fix(step_c.real, F), _fix(step_c.imag, F)
            cx, cy = cx - sx, cy - sy
            continue
        sx, sy = _cdiv(zx, zy, dx, dy, F)
        cx, cy = cx - sx, cy - sy
        step = mpmath.sqrt(_to_mpf(sx, F) ** 2 + _to_mpf(sy, F) ** 2)
        if step <= eps_cv:
            az = mpmath.sqrt(_to_mpf(zx, F) ** 2 + _to_mpf(zy, F) ** 2)
            newton_cv = az <= eps_valid
            break
    if newton_cv:
        return True, mpmath.mpc(_to_mpf(cx, F), _to_mpf(cy, F))
    return False, mpmath.mpc("nan", "nan")


def perturbation_mandelbrotN_nucleus_size_estimate(seed_x, seed_y, seed_prec, exponent, order):
    """Size estimate of the period-``order`` component of z -> z**n + c
    (FP_loop.pyx:472-604): with l = dz_i/dz_1 and b = 1 + sum_i 1 / l,
    size = 1 / (b * l**(n / (n - 1))) (principal power; l**2 for n = 2)."""
    n = _check_exponent(exponent)
    if n == 2:
        return perturbation_mandelbrot_nucleus_size_estimate(seed_x, seed_y, seed_prec, order)
    with mpmath.workprec(int(seed_prec)):
        c = mpmath.mpc(_dec(seed_x), _dec(seed_y))
        z = mpmath.mpc(0)
        l = mpmath.mpc(1)
        b = mpmath.mpc(1)
        for _ in range(1, int(order)):
            z = z ** n + c
            l = n * l * z ** (n - 1)
            b = b + 1 / l
        # the exponent n / (n - 1) is a double in the reference (mpc_pow_d)
        return 1 / (b * l ** mpmath.mpf(n / (n - 1.)))


def _dec(s):
    if isinstance(s, (bytes, bytearray)):
        return s.decode("utf8")
    return s


# ---------------------------------------------------------------------------
# Burning Ship family orbit (FP_loop.pyx:1828-1979)
# ---------------------------------------------------------------------------
def perturbation_nonholomorphic_FP_loop(orbit, need_Xrange, max_iter, M, seed_x, seed_y,
                                        seed_prec, kind=1):
    """BS-family orbit (x_{n+1}, y_{n+1}) = f_kind(x_n, y_n) + (a, -b).
    Returns (i, partial_dict, xr_dict) with the Xrange register holding
    iterations where |x| or |y| < XR_TSHOLD (only if need_Xrange)."""
    orb = orbit.view(np.complex128) if orbit.dtype != np.complex128 else orbit
    if int(seed_prec) <= 53:
        # MPFR at 53 bits, round to nearest, is IEEE double arithmetic
        return _bs_loop_double(orb, max_iter, M, float(_dec(seed_x)), float(_dec(seed_y)), kind)
    F = int(seed_prec) + GUARD_BITS
    a, b = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    x = y = 0
    orb[0] = 0.
    xr_dict = {}
    i = 0
    abs_i = 0.
    for i in range(1, max_iter + 1):
        x2, y2, xy = (x * x) >> F, (y * y) >> F, (x * y) >> F
        if kind == 1:
            x, y = x2 - y2 + a, 2 * abs(xy) - b
        elif kind == 2:
            x, y = x2 - y2 + a, 2 * ((x * abs(y)) >> F) - b
        elif kind == 3:
            x, y = x2 - ((y * abs(y)) >> F) + a, 2 * xy - b
        elif kind == 4:
            x, y = abs(x2 - y2) + a, 2 * xy - b
        else:
            x, y = abs(x2 - y2) + a, 2 * abs(xy) - b
        fx, fy = _to_float(x, F), _to_float(y, F)
        orb[i] = complex(fx, fy)
        abs_i = math.hypot(fx, fy)
        if abs_i > M:
            break
        if need_Xrange and (abs(fx) < XR_TSHOLD or abs(fy) < XR_TSHOLD):
            xr_dict[i] = (_mantissa_exp(x, F), _mantissa_exp(y, F))
    if i == max_iter and abs_i <= M:
        i += 1
    return i, {}, xr_dict


def _bs_loop_double(orb, max_iter, M, a, b, kind):
    """BS-family orbit in IEEE double (the seed_prec <= 53 case)."""
    x = y = 0.
    orb[0] = 0.
    i = 0
    abs_i = 0.
    for i in range(1, max_iter + 1):
        if kind == 1:
            x, y = x * x - y * y + a, 2. * abs(x * y) - b
        elif kind == 2:
            x, y = x * x - y * y + a, 2. * x * abs(y) - b
        elif kind == 3:
            x, y = x * x - y * abs(y) + a, 2. * x * y - b
        elif kind == 4:
            x, y = abs(x * x - y * y) + a, 2. * x * y - b
        else:
            x, y = abs(x * x - y * y) + a, 2. * abs(x * y) - b
        orb[i] = complex(x, y)
        abs_i = math.hypot(x, y)
        if abs_i > M:
            break
    if i == max_iter and abs_i <= M:
        i += 1
    return i, {}, {}


# ---------------------------------------------------------------------------
# Burning Ship family: ball method, Newton search and size estimate
# (FP_loop.pyx:1343-1827 iterations, Jacobians, matsolve; 1982-2100 size
# estimate; 2357-2440 ball method; 2564-2720 Newton).  The same arithmetic
# serves fixed-point integers (mul = product >> F) and mpmath numbers.
# ---------------------------------------------------------------------------
def _sgn(v):
    """sign() of FP_loop.pyx:1778-1784: +1 for v >= 0, else -1"""
    return 1 if v >= 0 else -1


def _bs_iter(kind, x, y, a, b, mul):
    """One iteration of flavor ``kind`` (FP_loop.pyx:1358-1455):
    1 BS       x' = x^2 - y^2 + a,     y' = 2 |x y| - b
    2 pBS      x' = x^2 - y^2 + a,     y' = 2 x |y| - b
    3 shark    x' = x^2 - y |y| + a,   y' = 2 x y - b
    4 celtic   x' = |x^2 - y^2| + a,   y' = 2 x y - b
    5 buffalo  x' = |x^2 - y^2| + a,   y' = 2 |x y| - b"""
    x2, y2 = mul(x, x), mul(y, y)
    if kind == 1:
        xy = mul(x, y)
        return x2 - y2 + a, 2 * abs(xy) - b
    if kind == 2:
        return x2 - y2 + a, 2 * mul(x, abs(y)) - b
    if kind == 3:
        return x2 - mul(abs(y), y) + a, 2 * mul(x, y) - b
    if kind == 4:
        return abs(x2 - y2) + a, 2 * mul(x, y) - b
    if kind == 5:
        return abs(x2 - y2) + a, 2 * abs(mul(x, y)) - b
    raise NotImplementedError(kind)


def _bs_jac(kind, x, y, J, mul, one, var_c):
    """Jacobian recurrence of flavor ``kind`` at the point (x, y)
    (FP_loop.pyx:1458-1743).  J = (dxdu, dxdv, dydu, dydv); with var_c the
    derivatives are taken w.r.t. c = a + i b and pick up +1 on dxda and -1 on
    dydb (the -b of the y update)."""
    jxx, jxy, jyx, jyy = J
    if kind in (1, 2, 5):
        sy = _sgn(y)
        ay = abs(y)
        if kind == 2:
            cx_, cy_ = x * sy, ay              # dyn/d. = 2 (x sgn(y) dy + |y| dx)
        else:
            cx_, cy_ = abs(x) * sy, ay * _sgn(x)
    if kind in (4, 5):
        s = _sgn(mul(x, x) - mul(y, y))
    else:
        s = 1
    if kind == 3:
        ay = abs(y)
        txx, txy = mul(x, jxx) - mul(ay, jyx), mul(x, jxy) - mul(ay, jyy)
        tyx, tyy = mul(x, jyx) + mul(y, jxx), mul(x, jyy) + mul(y, jxy)
    elif kind == 4:
        txx, txy = s * (mul(x, jxx) - mul(y, jyx)), s * (mul(x, jxy) - mul(y, jyy))
        tyx, tyy = mul(x, jyx) + mul(y, jxx), mul(x, jyy) + mul(y, jxy)
    else:
        txx, txy = s * (mul(x, jxx) - mul(y, jyx)), s * (mul(x, jxy) - mul(y, jyy))
        tyx = mul(cx_, jyx) + mul(cy_, jxx)
        tyy = mul(cx_, jyy) + mul(cy_, jxy)
    J = [2 * txx, 2 * txy, 2 * tyx, 2 * tyy]
    if var_c:
        J[0] += one
        J[3] -= one
    return tuple(J)


def _bs_escaped(x, y, F):
    return x.bit_length() > F + 64 or y.bit_length() > F + 64


def perturbation_nonholomorphic_ball_method(seed_x, seed_y, seed_prec, seed_px, maxiter,
                                            M_divergence, kind=1):
    """First i for which the ball of radius px around c maps onto a ball that
    contains 0 to first order: (rx, ry) = J^-1 (x_i, y_i) / px with |rx| < 1,
    |ry| < 1 and hypot(rx, ry) < 1, J the Jacobian w.r.t. c
    (FP_loop.pyx:2357-2440).  -1 if the orbit escapes M_divergence or no
    such i <= maxiter exists."""
    F = int(seed_prec) + GUARD_BITS
    a, b = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    px = _fix(_dec(seed_px), F)
    one = 1 << F

    def mul(u, v):
        return (u * v) >> F

    x = y = 0
    J = (0, 0, 0, 0)
    for i in range(1, int(maxiter) + 1):
        J = _bs_jac(kind, x, y, J, mul, one, True)
        x, y = _bs_iter(kind, x, y, a, b, mul)
        if math.hypot(_to_float(x, F), _to_float(y, F)) > M_divergence:
            return -1
        jxx, jxy, jyx, jyy = J
        det = jxx * jyy - jyx * jxy                   # scale 2^(2F)
        if det == 0:
            continue                                  # MPFR: inf / nan, no cycle
        nx = jyy * x - jxy * y                        # (J^-1 X) * det, scale 2^(2F)
        ny = jxx * y - jyx * x
        lim = abs(det) * px                           # scale 2^(3F)
        if abs(nx) << F < lim and abs(ny) << F < lim:
            if (nx * nx + ny * ny) << (2 * F) < lim * lim:
                return i
    return -1


def _bs_newton_step_float(a, b, order, kind, prec):
    """One Newton step in mpmath at ``prec`` bits, for an orbit that escapes
    (where fixed point would overflow): returns (da, db, x_order, y_order)."""
    with mpmath.workprec(prec):
        one = mpmath.mpf(1)
        x = y = mpmath.mpf(0)
        J = (x, x, x, x)
        for _ in range(int(order)):
            J = _bs_jac(kind, x, y, J, lambda u, v: u * v, one, True)
            x, y = _bs_iter(kind, x, y, a, b, lambda u, v: u * v)
        jxx, jxy, jyx, jyy = J
        det = jxx * jyy - jyx * jxy
        return (jyy * x - jxy * y) / det, (jxx * y - jyx * x) / det, x, y


def perturbation_nonholomorphic_find_any_nucleus(seed_x, seed_y, seed_prec, order, max_newton,
                                                 seed_eps_cv, seed_eps_valid, kind=1):
    """Newton search for c with f_c^order(0) = 0 on the 2 x 2 Jacobian,
    divisor periods accepted (FP_loop.pyx:2564-2720).  Converged when the
    step is below 64 eps_cv; valid when |(x, y)_order| <= eps_valid.
    Returns (newton_cv, c) with c an mpmath mpc (nan when not converged)."""
    F = int(seed_prec) + GUARD_BITS
    a, b = _fix(_dec(seed_x), F), _fix(_dec(seed_y), F)
    eps_cv = mpmath.mpf(_dec(seed_eps_cv)) * 64
    eps_valid = mpmath.mpf(_dec(seed_eps_valid))
    one = 1 << F

    def mul(u, v):
        return (u * v) >> F

    newton_cv = False
    for _ in range(int(max_newton)):
        x = y = 0
        J = (0, 0, 0, 0)
        escaped = False
        for _i in range(int(order)):
            J = _bs_jac(kind, x, y, J, mul, one, True)
            x, y = _bs_iter(kind, x, y, a, b, mul)
            if _bs_escaped(x, y, F):
                escaped = True
                break
        if escaped:
            da, db, xo, yo = _bs_newton_step_float(_to_mpf(a, F), _to_mpf(b, F), order, kind, F)
            sa, sb = _fix(da, F), _fix(db, F)
            a, b = a - sa, b - sb
            continue
        jxx, jxy, jyx, jyy = J
        det = (jxx * jyy - jyx * jxy) >> F
        if det == 0:
            break
        sa = (jyy * x - jxy * y) // det                # scale 2^F
        sb = (jxx * y - jyx * x) // det
        a, b = a - sa, b - sb
        step = mpmath.sqrt(_to_mpf(sa, F) ** 2 + _to_mpf(sb, F) ** 2)
        if step <= eps_cv:
            az = mpmath.sqrt(_to_mpf(x, F) ** 2 + _to_mpf(y, F) ** 2)
            newton_cv = az <= eps_valid
            break
    if newton_cv:
        with mpmath.workprec(int(seed_prec)):
            return True, mpmath.mpc(_to_mpf(a, F), _to_mpf(b, F))
    return False, mpmath.mpc("nan", "nan")


def perturbation_nonholomorphic_nucleus_size_estimate(seed_x, seed_y, seed_prec, order, kind=1):
    """Size estimate of the period-``order`` component at c and its skew
    matrix (FP_loop.pyx:1982-2100): with L_i the Jacobian of z_i w.r.t. z_1
    (taken after each iteration) and beta = I + sum_i L_i^-1,
    size = |det(L)^2 det(beta)|^(-1/2) and skew = beta / sqrt(det beta),
    returned as [[b_yy, b_xy], [b_yx, b_xx]]."""
    with mpmath.workprec(int(seed_prec)):
        a, b = mpmath.mpf(_dec(seed_x)), mpmath.mpf(_dec(seed_y))
        one, zero = mpmath.mpf(1), mpmath.mpf(0)

        def mul(u, v):
            return u * v

        x = y = zero
        J = (one, zero, zero, one)
        bxx, bxy, byx, byy = one, zero, zero, one
        for _ in range(1, int(order)):
            x, y = _bs_iter(kind, x, y, a, b, mul)
            J = _bs_jac(kind, x, y, J, mul, one, False)
            jxx, jxy, jyx, jyy = J
            inv = 1 / (jxx * jyy - jyx * jxy)
            bxx += inv * jyy
            bxy -= inv * jxy
            byx -= inv * jyx
            byy += inv * jxx
        jxx, jxy, jyx, jyy = J
        d = (jxx * jyy - jyx * jxy) ** 2
        det_b = bxx * byy - byx * bxy
        size = 1 / mpmath.sqrt(abs(det_b * d))
        if det_b > 0:
            s = 1 / mpmath.sqrt(det_b)
            skew = np.array(((float(byy * s), float(bxy * s)),
                             (float(byx * s), float(bxx * s))), dtype=np.float64)
        else:
            skew = np.full((2, 2), np.nan)
        return size, skew
