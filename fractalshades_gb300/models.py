"""
Fractal model classes with the reference's calculation API.

Mandelbrot (models/mandelbrot_M2.py:17-354), Perturbation_mandelbrot
(:361-877), Mandelbrot_N and Perturbation_mandelbrot_N
(models/mandelbrot_Mn.py:20-870), Burning_ship and Perturbation_burning_ship
(models/burning_ship.py:126-435, 862-1130).  Each ``calc_std_div`` keeps the
reference's keyword arguments, codes and defaults; its ``iterate()`` factory
returns the GPU calculation options instead of a numba closure.
"""
import enum
import typing
from typing import Optional

import mpmath
import numpy as np

from . import settings
from . import utils
from .core import Fractal
from .perturbation import PerturbationFractal
from .gpu import StdSpec, PerturbSpec
from .mpmath_utils import FP_loop as fsFP


def _orbit_backshift(calc_orbit, backshift):
    """The backshift the kernels use: 0 without calc_orbit (the reference
    divides by it when the orbit is stored, core.py:2985)."""
    if not calc_orbit:
        return 0
    if int(backshift) <= 0:
        raise ValueError("calc_orbit needs backshift > 0")
    return int(backshift)


def _no_initialize():
    def impl(*args):
        return None
    return impl


# ---------------------------------------------------------------------------
# Mandelbrot, power 2
# ---------------------------------------------------------------------------
class Mandelbrot(Fractal):

    def __init__(self, directory: str):
        """Standard power-2 Mandelbrot set, z_0 = 0, z_{n+1} = z_n^2 + c."""
        super().__init__(directory)
        self.potential_kind = "infinity"
        self.potential_d = 2
        self.potential_a_d = 1.
        self.potential_M_cutoff = 1000.
        self.holomorphic = True
        self.implements_dzndc = "always"
        self.implements_interior_detection = "always"
        self.implements_deepzoom = False

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str = "base_calc",
                     subset=None,
                     max_iter: int = 10000,
                     M_divergence: float = 1000.,
                     epsilon_stationnary: float = 0.01,
                     calc_d2zndc2: bool = False,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Escape-time iterations with dz/dz (interior detection) and dz/dc
        (mandelbrot_M2.py:61-176).  Exit codes 0 max_iter, 1 divergence,
        2 stationnary."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["zn", "dzndz", "dzndc"]
        if calc_d2zndc2:
            complex_codes += ["d2zndc2"]
        if calc_orbit:
            complex_codes += ["zn_orbit"]
        int_codes = []
        stop_codes = ["max_iter", "divergence", "stationnary"]

        def set_state():
            def impl(instance):
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.complex_type = np.complex128
                instance.potential_M = M_divergence
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = StdSpec(flavor=0, max_iter=max_iter, M_divergence=M_divergence,
                       epsilon_stationnary=epsilon_stationnary, calc_d2zndc2=calc_d2zndc2,
                       backshift=bs)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}


class Perturbation_mandelbrot(PerturbationFractal):

    def __init__(self, directory: str):
        """Arbitrary-precision power-2 Mandelbrot set (perturbation, BLA)."""
        super().__init__(directory)
        self.potential_kind = "infinity"
        self.potential_d = 2
        self.potential_a_d = 1.
        self.potential_M_cutoff = 1000.
        self.critical_pt = 0.
        self.FP_code = "zn"
        self.holomorphic = True
        self.implements_dzndc = "user"
        self.implements_interior_detection = "user"
        self.implements_deepzoom = True

    def FP_loop(self, NP_orbit, c0):
        """Full precision orbit, fills NP_orbit in place
        (mandelbrot_M2.py:408-430)."""
        max_orbit_iter = NP_orbit.shape[0] - 1
        return fsFP.perturbation_mandelbrot_FP_loop(
            NP_orbit.view(dtype=np.float64), self.xr_detect_activated, max_orbit_iter,
            self.M_divergence * 2, str(c0.real).encode("utf8"),
            str(c0.imag).encode("utf8"), mpmath.mp.prec)

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str,
                     subset,
                     max_iter: int,
                     M_divergence: float,
                     epsilon_stationnary: float,
                     BLA_eps: float = 1e-6,
                     interior_detect: bool = False,
                     calc_dzndc: bool = True,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Perturbation iterations (mandelbrot_M2.py:432-588).  Codes: zn,
        [dzndz], [dzndc]; int code ref_cycle_iter; exit codes 0 max_iter,
        1 divergence, 2 stationnary."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["zn"]
        code_int = 0
        dzndz = dzndc = i_znorbit = -1
        if interior_detect:
            code_int += 1
            complex_codes += ["dzndz"]
            dzndz = code_int
        if calc_dzndc:
            code_int += 1
            complex_codes += ["dzndc"]
            dzndc = code_int
        if calc_orbit:
            code_int += 1
            complex_codes += ["zn_orbit"]
            i_znorbit = code_int
        int_codes = ["ref_cycle_iter"]
        stop_codes = ["max_iter", "divergence", "stationnary"]
        BLA_activated = (BLA_eps is not None) and (self.dx < settings.newton_zoom_level)

        def set_state():
            def impl(instance):
                instance.complex_type = np.complex128
                instance.potential_M = M_divergence
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.calc_dZndz = interior_detect
                instance.calc_dZndc = calc_dzndc
                # the field-lines postproc reads it (the reference's power-2
                # model leaves it unset, mandelbrot_M2.py:529-539)
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = PerturbSpec(flavor=0, max_iter=max_iter, M_divergence=M_divergence,
                           epsilon_stationnary=epsilon_stationnary, calc_dzndc=calc_dzndc,
                           interior=interior_detect, bla=BLA_activated,
                           xr_detect_activated=self.xr_detect_activated,
                           i_dzndz=dzndz, i_dzndc=dzndc, nZ=len(complex_codes),
                           backshift=bs, i_znorbit=i_znorbit)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}

    # ------------------------------------------------------------------
    @staticmethod
    def _ball_method(c, px, maxiter, M_divergence):
        order = fsFP.perturbation_mandelbrot_ball_method(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), mpmath.mp.prec,
            str(px).encode("utf8"), maxiter, M_divergence)
        return None if order == -1 else order

    @staticmethod
    def find_nucleus(c, order, eps_pixel, max_newton=None, eps_cv=None):
        if order is None:
            raise ValueError("order shall be defined for Newton method")
        seed_prec = mpmath.mp.prec
        if max_newton is None:
            max_newton = 80
        if eps_cv is None:
            eps_cv = mpmath.mpf(val=(2, -seed_prec))
        return fsFP.perturbation_mandelbrot_find_nucleus(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), seed_prec, order,
            max_newton, str(eps_cv).encode("utf8"), str(eps_pixel).encode("utf8"))

    @staticmethod
    def find_any_nucleus(c, order, eps_pixel, max_newton=None, eps_cv=None):
        if order is None:
            raise ValueError("order shall be defined for Newton method")
        seed_prec = mpmath.mp.prec
        if max_newton is None:
            max_newton = 80
        if eps_cv is None:
            eps_cv = mpmath.mpf(val=(2, -seed_prec))
        return fsFP.perturbation_mandelbrot_find_any_nucleus(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), seed_prec, order,
            max_newton, str(eps_cv).encode("utf8"), str(eps_pixel).encode("utf8"))

    @staticmethod
    def _nucleus_size_estimate(c0, order):
        """(nucleus_size, julia_size) of the period-``order`` component at c0,
        julia_size = nucleus_size ** 0.75 (mandelbrot_M2.py:717-760)."""
        nucleus_size = abs(fsFP.perturbation_mandelbrot_nucleus_size_estimate(
            str(c0.real).encode("utf8"), str(c0.imag).encode("utf8"), mpmath.mp.prec, order))
        sqrt = mpmath.sqrt(nucleus_size)
        return nucleus_size, mpmath.sqrt(sqrt) * sqrt


# ---------------------------------------------------------------------------
# Mandelbrot, power n
# ---------------------------------------------------------------------------
def _check_exponent(exponent):
    exponent = int(exponent)
    if not 2 <= exponent <= nat_max_exponent():
        raise ValueError(f"exponent must be in 2 .. {nat_max_exponent()}, got {exponent}")
    return exponent


def nat_max_exponent():
    from . import _native
    return _native.FSG_MN_MAX_EXP


class Mandelbrot_N(Fractal):

    def __init__(self, directory: str, exponent: int):
        """Standard power-N Mandelbrot set, z_0 = 0, z_{n+1} = z_n^N + c
        (models/mandelbrot_Mn.py:20-380)."""
        super().__init__(directory)
        self.exponent = _check_exponent(exponent)
        self.potential_kind = "infinity"
        self.potential_d = exponent
        self.potential_a_d = 1.
        self.holomorphic = True
        self.implements_dzndc = "always"
        self.implements_interior_detection = "always"
        self.implements_deepzoom = False

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str,
                     subset=None,
                     max_iter: int,
                     M_divergence: float,
                     epsilon_stationnary: float,
                     calc_d2zndc2: bool = False,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Escape-time iterations of z^N + c with dz/dz and dz/dc
        (mandelbrot_Mn.py:60-175).  Codes zn, dzndz, dzndc; exit codes
        0 max_iter, 1 divergence, 2 stationnary."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["zn", "dzndz", "dzndc"]
        if calc_d2zndc2:
            complex_codes += ["d2zndc2"]
        if calc_orbit:
            complex_codes += ["zn_orbit"]
        int_codes = []
        stop_codes = ["max_iter", "divergence", "stationnary"]

        def set_state():
            def impl(instance):
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.complex_type = np.complex128
                instance.potential_M = M_divergence
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = StdSpec(flavor=0, max_iter=max_iter, M_divergence=M_divergence,
                       epsilon_stationnary=epsilon_stationnary, nexp=self.exponent,
                       calc_d2zndc2=calc_d2zndc2, backshift=bs)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}


class Perturbation_mandelbrot_N(PerturbationFractal):

    def __init__(self, directory: str, exponent: int):
        """Arbitrary-precision power-N Mandelbrot set: perturbation with the
        binomial expansion of (Z + z)^N - Z^N, BLA
        (models/mandelbrot_Mn.py:387-870)."""
        super().__init__(directory)
        self.exponent = _check_exponent(exponent)
        self.nexp = self.exponent
        self.potential_kind = "infinity"
        self.potential_d = exponent
        self.potential_a_d = 1.
        self.potential_M_cutoff = 1000.
        self.critical_pt = 0.
        self.FP_code = "zn"
        self.holomorphic = True
        self.implements_dzndc = "user"
        self.implements_interior_detection = "user"
        self.implements_deepzoom = True

    def FP_loop(self, NP_orbit, c0):
        """Full precision orbit of z^N + c, fills NP_orbit in place
        (mandelbrot_Mn.py:435-458)."""
        max_orbit_iter = NP_orbit.shape[0] - 1
        return fsFP.perturbation_mandelbrotN_FP_loop(
            NP_orbit.view(dtype=np.float64), self.xr_detect_activated, max_orbit_iter,
            self.exponent, self.M_divergence * 2, str(c0.real).encode("utf8"),
            str(c0.imag).encode("utf8"), mpmath.mp.prec)

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str,
                     subset,
                     max_iter: int,
                     M_divergence: float,
                     epsilon_stationnary: float,
                     BLA_eps: float = 1e-6,
                     interior_detect: bool = False,
                     calc_dzndc: bool = True,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Perturbation iterations for z^N + c (mandelbrot_Mn.py:460-623).
        Codes: zn, [dzndz], [dzndc]; int code ref_cycle_iter; exit codes
        0 max_iter, 1 divergence, 2 stationnary."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["zn"]
        code_int = 0
        dzndz = dzndc = i_znorbit = -1
        if interior_detect:
            code_int += 1
            complex_codes += ["dzndz"]
            dzndz = code_int
        if calc_dzndc:
            code_int += 1
            complex_codes += ["dzndc"]
            dzndc = code_int
        if calc_orbit:
            code_int += 1
            complex_codes += ["zn_orbit"]
            i_znorbit = code_int
        int_codes = ["ref_cycle_iter"]
        stop_codes = ["max_iter", "divergence", "stationnary"]
        BLA_activated = (BLA_eps is not None) and (self.dx < settings.newton_zoom_level)

        def set_state():
            def impl(instance):
                instance.complex_type = np.complex128
                instance.potential_M = M_divergence
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.calc_dZndz = interior_detect
                instance.calc_dZndc = calc_dzndc
                # the field-lines postproc reads it (the reference's power-2
                # model leaves it unset, mandelbrot_M2.py:529-539)
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = PerturbSpec(flavor=0, max_iter=max_iter, M_divergence=M_divergence,
                           epsilon_stationnary=epsilon_stationnary, calc_dzndc=calc_dzndc,
                           interior=interior_detect, bla=BLA_activated,
                           xr_detect_activated=self.xr_detect_activated,
                           i_dzndz=dzndz, i_dzndc=dzndc, nZ=len(complex_codes),
                           nexp=self.exponent, backshift=bs, i_znorbit=i_znorbit)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}

    # ------------------------------------------------------------------
    def _ball_method(self, c, px, maxiter, M_divergence):
        order = fsFP.perturbation_mandelbrotN_ball_method(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), mpmath.mp.prec,
            str(px).encode("utf8"), self.exponent, maxiter, M_divergence)
        return None if order == -1 else order

    def find_nucleus(self, c, order, eps_pixel, max_newton=None, eps_cv=None):
        """Not available for power N, as in the reference (mandelbrot_Mn.py:758-771)."""
        raise NotImplementedError(
            "Divide by undesired roots technique not implemented, Use 'find_any_nucleus'")

    def find_any_nucleus(self, c, order, eps_pixel, max_newton=None, eps_cv=None):
        if order is None:
            raise ValueError("order shall be defined for Newton method")
        seed_prec = mpmath.mp.prec
        if max_newton is None:
            max_newton = 80
        if eps_cv is None:
            eps_cv = mpmath.mpf(val=(2, -seed_prec))
        return fsFP.perturbation_mandelbrotN_find_any_nucleus(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), seed_prec, self.exponent,
            order, max_newton, str(eps_cv).encode("utf8"), str(eps_pixel).encode("utf8"))

    def _nucleus_size_estimate(self, c0, order):
        """(nucleus_size, julia_size), julia_size = nucleus_size **
        ((N + 1)(N - 1) / N^2) (mandelbrot_Mn.py:801-843)."""
        nucleus_size = abs(fsFP.perturbation_mandelbrotN_nucleus_size_estimate(
            str(c0.real).encode("utf8"), str(c0.imag).encode("utf8"), mpmath.mp.prec,
            self.exponent, order))
        expo = self.exponent
        julia_exp = (expo + 1.) * (expo - 1.) / expo / expo
        return nucleus_size, nucleus_size ** julia_exp


# ---------------------------------------------------------------------------
# Burning Ship family
# ---------------------------------------------------------------------------
BS_flavor_list = (
    "Burning ship",
    "Perpendicular burning ship",
    "Shark fin",
    "Celtic",
    "Buffalo",
)
BS_flavor_enum = enum.Enum("BS_flavor_enum", BS_flavor_list, module=__name__)


def get_flavor_int(flavor: str):
    """1-based index of the flavor (burning_ship.py:76-80)."""
    return getattr(BS_flavor_enum, flavor).value


class Burning_ship(Fractal):

    def __init__(self, directory: str,
                 flavor: typing.Literal[BS_flavor_enum] = "Burning ship"):
        """Burning Ship and its 'abs variations' (burning_ship.py:126-280):
        x' = x^2 - y^2 + a, y' = 2|xy| - b and four other flavors."""
        super().__init__(directory)
        self.flavor = flavor
        self.flavor_int = get_flavor_int(flavor)
        self.potential_kind = "infinity"
        self.potential_d = 2
        self.potential_a_d = 1.
        self.potential_M_cutoff = {"Burning ship": 1000., "Perpendicular burning ship": 1000,
                                   "Shark fin": 1.e20, "Celtic": 1000., "Buffalo": 1000}[flavor]
        self.holomorphic = False
        self.implements_dzndc = "always"
        self.implements_interior_detection = "no"
        self.implements_deepzoom = False

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str,
                     subset,
                     max_iter: int,
                     M_divergence: float,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Escape-time iterations with the Jacobian (burning_ship.py:282-346).
        Codes xn, yn, dxnda, dxndb, dynda, dyndb (float64)."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["xn", "yn", "dxnda", "dxndb", "dynda", "dyndb"]
        if calc_orbit:
            complex_codes += ["xn_orbit", "yn_orbit"]
        int_codes = []
        stop_codes = ["max_iter", "divergence", "stationnary"]

        def set_state():
            def impl(instance):
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.complex_type = np.float64
                instance.potential_M = M_divergence
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = StdSpec(flavor=self.flavor_int, max_iter=max_iter, M_divergence=M_divergence,
                       backshift=bs)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}


class Perturbation_burning_ship(PerturbationFractal):

    def __init__(self, directory: str,
                 flavor: typing.Literal[BS_flavor_enum] = "Burning ship"):
        """Arbitrary-precision Burning Ship family (perturbation with sign
        folding, 8-coefficient BLA)."""
        super().__init__(directory)
        self.flavor = flavor
        self.flavor_int = get_flavor_int(flavor)
        self.potential_kind = "infinity"
        self.potential_d = 2
        self.potential_a_d = 1.
        self.potential_M_cutoff = 1000.
        self.critical_pt = 0.
        self.FP_code = ["xn", "yn"]
        self.holomorphic = False
        self.implements_dzndc = "always"
        self.implements_interior_detection = "no"
        self.implements_deepzoom = True

    def FP_loop(self, NP_orbit, c0):
        max_orbit_iter = NP_orbit.shape[0] - 1
        return fsFP.perturbation_nonholomorphic_FP_loop(
            NP_orbit.view(dtype=np.float64), self.xr_detect_activated, max_orbit_iter,
            self.M_divergence * 2, str(c0.real).encode("utf8"),
            str(c0.imag).encode("utf8"), mpmath.mp.prec, kind=self.flavor_int)

    @utils.calc_options
    def calc_std_div(self, *,
                     calc_name: str,
                     subset,
                     max_iter: int,
                     M_divergence: float,
                     BLA_eps: float = 1e-6,
                     calc_hessian: bool = True,
                     calc_orbit: bool = False,
                     backshift: int = 0):
        """Perturbation iterations (burning_ship.py:971-1130).  Codes xn, yn
        [, dxnda, dxndb, dynda, dyndb]; int code ref_cycle_iter; exit codes
        0 max_iter, 1 divergence."""
        bs = _orbit_backshift(calc_orbit, backshift)
        complex_codes = ["xn", "yn"]
        if calc_hessian:
            complex_codes += ["dxnda", "dxndb", "dynda", "dyndb"]
        i_xnorbit = -1
        if calc_orbit:
            i_xnorbit = len(complex_codes)
            complex_codes += ["xn_orbit", "yn_orbit"]
        int_codes = ["ref_cycle_iter"]
        stop_codes = ["max_iter", "divergence"]
        BLA_activated = (BLA_eps is not None) and (self.dx < settings.newton_zoom_level)

        def set_state():
            def impl(instance):
                instance.complex_type = np.float64
                instance.potential_M = M_divergence
                instance.codes = (complex_codes, int_codes, stop_codes)
                instance.calc_hessian = calc_hessian
                instance.backshift = bs if calc_orbit else None
            return impl

        spec = PerturbSpec(flavor=self.flavor_int, max_iter=max_iter,
                           M_divergence=M_divergence, calc_dzndc=calc_hessian,
                           bla=BLA_activated, xr_detect_activated=self.xr_detect_activated,
                           nZ=len(complex_codes), backshift=bs, i_znorbit=i_xnorbit)
        return {"set_state": set_state, "initialize": _no_initialize,
                "iterate": lambda: spec}

    # Newton search & related (burning_ship.py:1168-1290)
    def _ball_method(self, c, px, maxiter, M_divergence):
        """Order-1 ball method on the 2 x 2 Jacobian (FP_loop.pyx:2357-2440)."""
        order = fsFP.perturbation_nonholomorphic_ball_method(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), mpmath.mp.prec,
            str(px).encode("utf8"), maxiter, M_divergence, kind=self.flavor_int)
        return None if order == -1 else order

    @staticmethod
    def find_nucleus(c, order, eps_pixel, max_newton=None, eps_cv=None):
        raise NotImplementedError("Divide by undesired roots technique "
                                  "not implemented for burning ship")

    def find_any_nucleus(self, c, order, eps_pixel, max_newton=None, eps_cv=None):
        """Newton search for f^order(0) = 0, divisor periods accepted
        (FP_loop.pyx:2564-2720)."""
        if order is None:
            raise ValueError("order shall be defined for Newton method")
        seed_prec = mpmath.mp.prec
        if max_newton is None:
            max_newton = 80
        if eps_cv is None:
            eps_cv = mpmath.mpf(val=(2, -seed_prec))
        return fsFP.perturbation_nonholomorphic_find_any_nucleus(
            str(c.real).encode("utf8"), str(c.imag).encode("utf8"), seed_prec, order,
            max_newton, str(eps_cv).encode("utf8"), str(eps_pixel).encode("utf8"),
            kind=self.flavor_int)

    def _nucleus_size_estimate(self, c0, order):
        """(nucleus_size, julia_size, skew) (FP_loop.pyx:1982-2100)."""
        nucleus_size, skew = fsFP.perturbation_nonholomorphic_nucleus_size_estimate(
            str(c0.real).encode("utf8"), str(c0.imag).encode("utf8"), mpmath.mp.prec, order,
            kind=self.flavor_int)
        sqrt = mpmath.sqrt(nucleus_size)
        return nucleus_size, mpmath.sqrt(sqrt) * sqrt, skew
