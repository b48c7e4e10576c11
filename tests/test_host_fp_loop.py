"""
Host arbitrary-precision layer (mpmath_utils/FP_loop.py over libfsghost.so,
MPFR / MPC) against the known answers of the reference's
tests/test_FP_loop.py and its stored FP64 orbits (tests/REFERENCE_DATA), and
against the independent fixed-point restatement oracle/fp_loop_fixed.py.  The
known-answer values are copied from the reference's tests (they are its test
vectors, not computed here).
"""
import os
import pickle

import mpmath
import numpy as np
import pytest

from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
from oracle import fp_loop_fixed as fixed

HERE = os.path.dirname(os.path.abspath(__file__))


def test_ball_method_order_4252():
    """tests/test_FP_loop.py:166-193 of the reference."""
    x = ("-1.38489865821023436791757551552306535886843948840412919252407990736888"
         "673896107")
    y = ("0.02274991237672465768411681642741466833930426052197620974166612959128"
         "19114324773")
    order = fsFP.perturbation_mandelbrot_ball_method(
        x.encode(), y.encode(), int(78 * 3.33), "1.253026641642179625e-70".encode(),
        100000, 1000.0)
    assert order == 4252


def test_bs_orbit_is_double_recurrence_at_53_bits():
    """tests/test_FP_loop.py:278-309: at 53 bits the BS orbit is the IEEE
    double recurrence x' = x^2 - y^2 + a, y' = 2|xy| - b."""
    x, y = 0.1, 0.1
    npts = 10
    orbit = np.empty((npts,), dtype=np.complex128)
    fsFP.perturbation_nonholomorphic_FP_loop(orbit.view(np.float64), False, npts - 1, 1000.,
                                             str(x).encode(), str(y).encode(), 53, 1)
    z = complex(0.)
    for i in range(10):
        assert orbit[i] == z
        nx = z.real ** 2 - z.imag ** 2 + x
        ny = 2 * np.abs(z.real * z.imag) - y
        z = nx + 1j * ny


def test_orbit_matches_reference_stored_orbit():
    """The reference stores (tests/REFERENCE_DATA/perturb_REF/flake/dev_pt0.ref)
    an FP64 orbit of its 668-bit reference point, period 7884.  The host loop
    reproduces it bit-for-bit over the whole period (at the period the orbit
    returns to ~0, a value made of rounding noise)."""
    fx = os.path.join(HERE, "golden", "flake_orbit.npz")
    d = np.load(fx)
    order = int(d["order"])
    orbit = np.zeros(order + 1, dtype=np.complex128)
    i, _, _ = fsFP.perturbation_mandelbrot_FP_loop(
        orbit, False, order, 1e6, str(d["x"]), str(d["y"]), int(d["prec"]))
    assert i == order + 1
    assert np.array_equal(orbit[:order].view(np.uint64), d["orbit"][:order].view(np.uint64))


def test_newton_nucleus_and_size():
    """Newton with divisor deflation lands on a nucleus whose orbit returns to
    0 at the period; the ball method confirms the period."""
    from fractalshades_gb300 import synthetic as syn
    c = syn.find_nucleus(37, 60)
    with mpmath.workdps(60):
        z = mpmath.mpc(0)
        for _ in range(37):
            z = z * z + c
        assert abs(z) < mpmath.mpf(10) ** -25
        size = fsFP.perturbation_mandelbrot_nucleus_size_estimate(
            str(c.real), str(c.imag), mpmath.mp.prec, 37)
        assert 0 < abs(size) < 1e-3


@pytest.mark.slow
def test_newton_4252_reference_digits():
    """tests/test_FP_loop.py:231-272: Newton from a 80-digit start at order
    4252 and 11622-bit precision agrees with the reference's ~3500-digit
    nucleus.  Expected digits stored in tests/golden/newton_4252.npz."""
    d = np.load(os.path.join(HERE, "golden", "newton_4252.npz"))
    precision = int(3522 * 3.3)
    eps = mpmath.mpf(val=(2, -precision))
    eps_pix = mpmath.mpf(val=(2, -int(84 * 3.3)))
    with mpmath.workprec(precision):
        ok, val = fsFP.perturbation_mandelbrot_find_nucleus(
            str(d["x_start"]).encode(), str(d["y_start"]).encode(), precision, 4252, 80,
            str(eps).encode(), str(eps_pix).encode())
    assert ok
    with mpmath.workprec(precision - 10):
        assert mpmath.almosteq(mpmath.mpf(str(d["x_nucleus"])), val.real)


BS_KATS = [("-1.7545128115395", "0.0015894811966473", "0.01"),
           ("0.88410156557344", "1.5218981991448", "0.012")]


@pytest.mark.parametrize("x, y, px", BS_KATS)
def test_bs_ball_method_order_3(x, y, px):
    """tests/test_FP_loop.py:311-341 of the reference: period 3 at both seeds
    (53 bits, px 0.01, maxiter 100, M 1000)."""
    order = fsFP.perturbation_nonholomorphic_ball_method(
        x.encode(), y.encode(), 53, b"0.01", 100, 1000., 1)
    assert order == 3


def _bs_orbit(c, n, kind=1):
    x = y = mpmath.mpf(0)
    for _ in range(n):
        x, y = fixed._bs_iter(kind, x, y, c.real, c.imag, lambda u, v: u * v)
    return x, y


@pytest.mark.parametrize("x, y, px", BS_KATS)
def test_bs_newton_period_3(x, y, px):
    """tests/test_FP_loop.py:343-382: Newton from the same seeds converges
    (53 bits, 40 steps); the point found is periodic, z_3 = 0."""
    eps_cv = mpmath.mpf(val=(2, -53))
    ok, c = fsFP.perturbation_nonholomorphic_find_any_nucleus(
        x.encode(), y.encode(), 53, 3, 40, str(eps_cv).encode(), px.encode(), 1)
    assert ok
    with mpmath.workprec(200):
        zx, zy = _bs_orbit(c, 3)
        assert abs(zx) < 1e-12 and abs(zy) < 1e-12
    size, skew = fsFP.perturbation_nonholomorphic_nucleus_size_estimate(
        str(c.real).encode(), str(c.imag).encode(), 53, 3, 1)
    assert 1e-3 < float(size) < 1.
    assert np.all(np.isfinite(skew))


@pytest.mark.parametrize("kind", [1, 2, 3, 4, 5])
def test_bs_newton_deep_every_flavor(kind):
    """At 300 bits the Newton search converges to a point whose period-p
    orbit returns to 0 to the working precision, for every flavor (p from the
    ball method around a seeded point)."""
    rng = np.random.default_rng(kind)
    with mpmath.workprec(300):
        found = False
        for _ in range(40):
            c0 = mpmath.mpc(-2 + 2.5 * rng.random(), -1.5 + 2 * rng.random())
            order = fsFP.perturbation_nonholomorphic_ball_method(
                str(c0.real).encode(), str(c0.imag).encode(), 300, b"0.05", 200, 1e5, kind)
            if order < 2 or order > 60:
                continue
            ok, c = fsFP.perturbation_nonholomorphic_find_any_nucleus(
                str(c0.real).encode(), str(c0.imag).encode(), 300, order, 80,
                str(mpmath.mpf(val=(2, -300))).encode(), b"1e-60", kind)
            if not ok:
                continue
            zx, zy = _bs_orbit(c, order, kind)
            assert abs(zx) < 1e-60 and abs(zy) < 1e-60
            found = True
            break
        assert found


# ---------------------------------------------------------------------------
# power-n Mandelbrot (FP_loop.pyx:255-421, 472-604, 618-760, 1139-1340)
# ---------------------------------------------------------------------------
# period-10 nuclei of z^3 + c and z^4 + c to 20 digits (the seeds of the
# power-n golden vectors)
MN_NUCLEI = {3: ("0.64287667998175895118", "0.25145447487965245909"),
             4: ("-0.51534888699245770184", "0.46481172994907691405")}


@pytest.mark.parametrize("n", [3, 4])
def test_power_n_orbit_and_partials(n):
    mpmath.mp.dps = 40
    x, y = MN_NUCLEI[n]
    c = mpmath.mpc(x, y)
    orb = np.zeros(61, dtype=np.complex128)
    i, partials, xr = fsFP.perturbation_mandelbrotN_FP_loop(
        orb, True, 60, n, 2000., x.encode(), y.encode(), mpmath.mp.prec)
    assert i == 61 and not xr
    z = mpmath.mpc(0)
    for k in range(1, 61):
        z = z ** n + c
        assert orb[k] == complex(float(z.real), float(z.imag))
    # successive minima of |z_k| below 1e-5: the first return at the period
    assert list(partials)[0] == 10 and all(k % 10 == 0 for k in partials)


@pytest.mark.parametrize("n", [3, 4])
def test_power_n_ball_newton_size(n):
    mpmath.mp.dps = 40
    x, y = MN_NUCLEI[n]
    c = mpmath.mpc(x, y)
    prec = mpmath.mp.prec
    order = fsFP.perturbation_mandelbrotN_ball_method(
        x.encode(), y.encode(), prec, b"1e-7", n, 10000, 1e5)
    assert order == 10
    seed = c + mpmath.mpf("1e-9")
    ok, nucleus = fsFP.perturbation_mandelbrotN_find_any_nucleus(
        str(seed.real).encode(), str(seed.imag).encode(), prec, n, 10, 80,
        str(mpmath.mpf(2) ** -prec).encode(), b"1e-20")
    assert ok and abs(nucleus - c) < mpmath.mpf("1e-19")
    z = mpmath.mpc(0)
    for _ in range(10):
        z = z ** n + nucleus
    assert abs(z) < mpmath.mpf("1e-30")
    size = abs(fsFP.perturbation_mandelbrotN_nucleus_size_estimate(
        str(nucleus.real).encode(), str(nucleus.imag).encode(), prec, n, 10))
    # the component's size: at c + size / 4 along any direction the cycle
    # stays attracting (|d z_10 / d z_0| < 1 at the 10-cycle)
    assert mpmath.mpf("1e-7") < size < mpmath.mpf("1e-2")


def test_power_2_delegates_to_power_2_functions():
    mpmath.mp.dps = 30
    a = np.zeros(41, dtype=np.complex128)
    b = np.zeros(41, dtype=np.complex128)
    ra = fsFP.perturbation_mandelbrotN_FP_loop(a, False, 40, 2, 1e3, b"-0.1", b"0.65", 100)
    rb = fsFP.perturbation_mandelbrot_FP_loop(b, False, 40, 1e3, b"-0.1", b"0.65", 100)
    assert ra[0] == rb[0] and np.array_equal(a, b)
    with pytest.raises(NotImplementedError):
        fsFP.perturbation_mandelbrotN_FP_loop(a, False, 40, 1, 1e3, b"0", b"0", 100)


# ---------------------------------------------------------------------------
# the MPFR library against the fixed-point restatement and exact iteration
# ---------------------------------------------------------------------------
def _seeded_nucleus_400():
    from fractalshades_gb300 import synthetic as syn
    mpmath.mp.dps = 400
    return syn.nucleus(2562, 400)


def test_native_m2_orbit_registers_and_period_vs_fixed_point():
    """Period-2562 nucleus at 400 digits: the orbit (every double), the exit
    index and both registers equal the fixed-point restatement's, whose
    values are correctly rounded from 64 guard bits; the ball method finds
    the period in both."""
    c = _seeded_nucleus_400()
    prec = mpmath.mp.prec
    sx, sy = str(c.real).encode(), str(c.imag).encode()
    a = np.zeros(2563, dtype=np.complex128)
    b = np.zeros(2563, dtype=np.complex128)
    ra = fsFP.perturbation_mandelbrot_FP_loop(a, True, 2562, 2000., sx, sy, prec)
    rb = fixed.perturbation_mandelbrot_FP_loop(b, True, 2562, 2000., sx, sy, prec)
    assert ra[0] == rb[0] == 2563
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert sorted(ra[1]) == sorted(rb[1]) and sorted(ra[2]) == sorted(rb[2])
    for reg_a, reg_b in ((ra[1], rb[1]), (ra[2], rb[2])):
        for k in reg_a:
            if k < 2562:
                assert reg_a[k] == reg_b[k]
            else:
                # z_p of a 400-digit nucleus: rounding noise of either method
                for r in (reg_a[k], reg_b[k]):
                    assert r.e < -1200
    px = b"1e-300"
    assert fsFP.perturbation_mandelbrot_ball_method(sx, sy, prec, px, 3000, 1e5) == 2562
    assert fixed.perturbation_mandelbrot_ball_method(sx, sy, prec, px, 3000, 1e5) == 2562


def test_native_m2_newton_and_size_vs_fixed_point():
    c = _seeded_nucleus_400()
    prec = mpmath.mp.prec
    seed = c + mpmath.mpf("1e-200")
    eps = str(mpmath.mpf(2) ** -prec).encode()
    args = (str(seed.real).encode(), str(seed.imag).encode(), prec, 2562, 80, eps, b"1e-300")
    ok_a, ca = fsFP.perturbation_mandelbrot_find_nucleus(*args)
    ok_b, cb = fixed.perturbation_mandelbrot_find_nucleus(*args)
    assert ok_a and ok_b
    assert abs(ca - c) < mpmath.mpf(10) ** -395 and abs(ca - cb) < mpmath.mpf(10) ** -395
    sa = fsFP.perturbation_mandelbrot_nucleus_size_estimate(
        str(c.real).encode(), str(c.imag).encode(), prec, 2562)
    sb = fixed.perturbation_mandelbrot_nucleus_size_estimate(
        str(c.real).encode(), str(c.imag).encode(), prec, 2562)
    assert abs(sa - sb) < 1e-15 * abs(sb)


@pytest.mark.parametrize("kind", [1, 2, 3, 4, 5])
def test_native_bs_orbit_vs_fixed_point_and_exact(kind):
    """Burning Ship family at 300 bits: the orbit doubles equal the fixed-
    point restatement's and the correctly rounded values of a 600-bit
    iteration; the Xrange register records the coordinates below 1e-300."""
    with mpmath.workprec(300):
        a0, b0 = mpmath.mpf("-1.7545128115395"), mpmath.mpf("0.0015894811966473")
        sx, sy = str(a0).encode(), str(b0).encode()
    n = 400
    o = np.zeros(n + 1, dtype=np.complex128)
    f = np.zeros(n + 1, dtype=np.complex128)
    ia, pa, xa = fsFP.perturbation_nonholomorphic_FP_loop(o, True, n, 1e3, sx, sy, 300, kind)
    ib, _, _ = fixed.perturbation_nonholomorphic_FP_loop(f, True, n, 1e3, sx, sy, 300, kind)
    assert ia == ib
    assert np.array_equal(o[:ia].view(np.uint64), f[:ia].view(np.uint64))
    with mpmath.workprec(600):
        x = y = mpmath.mpf(0)
        a, b = mpmath.mpf(sx.decode()), mpmath.mpf(sy.decode())
        for k in range(1, min(ia, n) + 1):
            x, y = fixed._bs_iter(kind, x, y, a, b, lambda u, v: u * v)
            assert o[k] == complex(float(x), float(y)), (kind, k)
    assert all(k % 1 == 0 for k in pa)
    for k, ((mx, ex), (my, ey)) in xa.items():
        assert min(abs(o[k].real), abs(o[k].imag)) < 1e-300


def test_native_mn_matches_fixed_point():
    mpmath.mp.dps = 60
    x, y = MN_NUCLEI[3]
    a = np.zeros(301, dtype=np.complex128)
    b = np.zeros(301, dtype=np.complex128)
    ra = fsFP.perturbation_mandelbrotN_FP_loop(a, False, 300, 3, 1e3, x.encode(), y.encode(),
                                               mpmath.mp.prec)
    rb = fixed.perturbation_mandelbrotN_FP_loop(b, False, 300, 3, 1e3, x.encode(), y.encode(),
                                                mpmath.mp.prec)
    assert ra[0] == rb[0] and np.array_equal(a, b) and sorted(ra[1]) == sorted(rb[1])


def test_host_errors_are_reported():
    from fractalshades_gb300 import _host
    o = np.zeros(11, dtype=np.complex128)
    with pytest.raises(_host.HostError):
        fsFP.perturbation_mandelbrot_FP_loop(o, False, 10, 1e3, b"not-a-number", b"0", 100)
    with pytest.raises(ValueError):
        fsFP.perturbation_mandelbrot_FP_loop(o, False, 20, 1e3, b"0", b"0", 100)
