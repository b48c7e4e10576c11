"""
Projections of the screen coordinates (reference projection.py): Cartesian
(identity, scale 1) and Expmap (exponential mapping).  The GPU kernels apply
the mapping per pixel (fsg_tile.proj*, csrc/fsg_internal.cuh fsg_pixel) and
the perturbation loops its derivative modifier; Generic_mapping is outside
this package.
"""
import logging

import mpmath
import numpy as np

from . import settings

logger = logging.getLogger(__name__)


class Projection:
    """Base class (projection.py:20-145 of the reference)."""
    scale = 1.0
    dzndc_modifier = None
    df = None
    dfBS = None

    def adjust_to_zoom(self, fractal):
        self.make_impl()

    def make_impl(self):
        self.make_f_impl()
        self.make_df_impl()
        self.make_dfBS_impl()

    def make_f_impl(self):
        raise NotImplementedError

    def make_df_impl(self):
        self.df = None

    def make_dfBS_impl(self):
        self.dfBS = None

    def __eq__(self, other):
        return type(self) is type(other) and vars(self) == vars(other)

    def __hash__(self):
        return hash(type(self).__name__)


def cartesian_impl(z):
    return z


class Cartesian(Projection):
    #: kernel mapping kind (fsg_tile.proj)
    kernel_kind = 0

    """Identity projection (projection.py:156-223).  ``expmap_seam`` is not
    supported by the GPU path."""

    def __init__(self, expmap_seam=None):
        if expmap_seam is not None:
            raise NotImplementedError("expmap_seam is not supported by the GPU kernels")
        self.scale = 1.0
        self.expmap_seam = None

    def make_f_impl(self):
        self.f = cartesian_impl

    def bounding_box(self, xy_ratio):
        return 1., 1. / xy_ratio

    @property
    def min_local_scale(self):
        return 1.


class Expmap(Projection):
    """Exponential mapping pix -> exp(h_moy + dh pix) (projection.py:226-503):
    h runs from hmin to hmax along the screen's x axis ("horizontal") or y
    axis ("vertical"), the other axis carries the angle over [-pi, pi] (the
    zoom's xy_ratio and nx are adjusted for it).  Float h only: exp(hmax)
    up to 1 / xrange_zoom_level (hmax < ~690); the reference's Xrange h and
    its step-by-step rendering of larger mappings are not built."""
    kernel_kind = 1

    def __init__(self, hmin, hmax, rotates_df=True, orientation="horizontal"):
        if not (0 <= hmin < hmax):
            raise ValueError("Provide hmin, hmax with:  0 <= hmin < hmax for Expmap")
        if mpmath.exp(hmax) > (1. / settings.xrange_zoom_level):
            raise NotImplementedError("Expmap with exp(hmax) beyond the double range")
        self.use_step = False
        self.rotates_df = rotates_df
        self.orientation = orientation
        self.premul_1j = {"horizontal": False, "vertical": True}[orientation]
        self.hmin = float(hmin)
        self.hmax = float(hmax)
        self.hmoy = (hmin + hmax) * 0.5
        self.dh = hmax - hmin

    @property
    def init_kwargs(self):
        return {"hmin": self.hmin, "hmax": self.hmax, "rotates_df": self.rotates_df,
                "orientation": self.orientation}

    def __eq__(self, other):
        return type(self) is type(other) and self.init_kwargs == other.init_kwargs

    def __hash__(self):
        return hash((type(self).__name__,) + tuple(self.init_kwargs.values()))

    def __getstate__(self):
        # the mapping functions are rebuilt from the parameters (the
        # calculation fingerprint pickles the projection)
        return {k: v for k, v in vars(self).items() if k not in ("f", "df", "dfBS")}

    def __setstate__(self, state):
        self.__dict__.update(state)
        if hasattr(self, "xy_ratio"):
            self.make_impl()

    def nh(self, fractal):
        return fractal.ny if self.premul_1j else fractal.nx

    def nt(self, fractal):
        return fractal.nx if self.premul_1j else fractal.ny

    @property
    def pix_to_ht(self):
        """pixel -> h + i t factor (projection.py:306-314)"""
        return (1j * self.dh * self.xy_ratio) if self.premul_1j else self.dh

    def adjust_to_zoom(self, fractal):
        """xy_ratio so that t spans 2 pi (projection.py:339-361)."""
        if self.premul_1j:
            xy_ratio = (np.pi * 2.) / self.dh
            nx = int(fractal.nx * xy_ratio + 0.5)
        else:
            xy_ratio = self.dh / (np.pi * 2.)
            nx = fractal.nx
        fractal.xy_ratio = self.xy_ratio = xy_ratio
        fractal.zoom_kwargs["xy_ratio"] = xy_ratio
        fractal.nx = nx
        fractal.zoom_kwargs["nx"] = nx
        logger.info(f"Adjusted parameters for Expmap projection: nx {nx}, xy_ratio {xy_ratio}")
        self.make_impl()

    def make_f_impl(self):
        hmoy, pix_to_ht = self.hmoy, self.pix_to_ht

        def f(pix):
            return np.exp(hmoy + pix_to_ht * pix)
        self.f = f

    def make_df_impl(self):
        """The derivative of the mapping applied to dz/dc in post-processing
        (projection.py:375-393): exp(ht pix), or its modulus when not
        rotates_df.  (The reference's make_dfBS_impl then assigns df again,
        :412-435, which leaves its holomorphic df unusable; the intended
        function is kept here.)"""
        pix_to_ht = self.pix_to_ht
        if self.rotates_df:
            def df(pix):
                return np.exp(pix_to_ht * pix)
        else:
            def df(pix):
                return np.exp(np.real(pix_to_ht * pix))
        self.df = df

    def make_dfBS_impl(self):
        pix_to_ht = self.pix_to_ht
        if self.rotates_df:
            def dfBS(pix):
                ht = pix_to_ht * pix
                r = np.exp(np.real(ht))
                t = np.imag(ht)
                cr, sr = np.cos(t) * r, np.sin(t) * r
                return -sr, -cr, cr, -sr
        else:
            def dfBS(pix):
                r = np.exp(np.real(pix_to_ht * pix))
                return r, 0. * r, 0. * r, r
        self.dfBS = dfBS

    def dzndc_modifier(self, cpix):
        """exp(Re(ht pix) + h_moy), applied by the perturbation loops to the
        derivatives at exit (projection.py:455-473, perturbation.py:1387-1388)"""
        return np.exp(np.real(self.pix_to_ht * cpix) + self.hmoy)

    @property
    def scale(self):
        """exp(h_moy): the derivative paths' scale factor (projection.py:475-481)"""
        return mpmath.exp(self.hmoy)

    def bounding_box(self, xy_ratio):
        w = mpmath.exp(self.hmax)
        return w, w

    @property
    def min_local_scale(self):
        return mpmath.exp(self.hmin)

    def kernel_params(self):
        """(kind, h, Re ht, Im ht) of fsg_tile: f(pix) = exp(h + ht pix)"""
        ht = complex(self.pix_to_ht)
        return self.kernel_kind, float(self.hmoy), ht.real, ht.imag


def kernel_params(projection):
    """The fsg_tile projection fields of a projection."""
    if isinstance(projection, Expmap):
        return projection.kernel_params()
    return 0, 0., 0., 0.


def identity_lin_mat():
    return np.array(((1., -0.), (0., 1.)), dtype=np.float64)
