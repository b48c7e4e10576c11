"""
Projections of the screen coordinates (reference projection.py).  The
iteration path supports the Cartesian projection (identity, scale 1); the
non-linear ones (Expmap, Generic_mapping) are outside this package.
"""
import numpy as np


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


def identity_lin_mat():
    return np.array(((1., -0.), (0., 1.)), dtype=np.float64)
