"""
PerturbationFractal: arbitrary-precision reference orbit on the host, delta
iterations on the GPU.

Mirrors the reference's PerturbationFractal (perturbation.py:22-977): the
mpmath zoom, the reference-point search (ball method + Newton, dps boosts),
the orbit storage, ref_point_kc, get_path_data and get_cycle_indep_args.  The
derivative paths and the BLA tree are built on the GPU from the uploaded orbit
(fsg_ref_create), and ``numba_cycle_call`` runs the GPU perturbation kernel.
"""
import logging
import os
import pickle
import textwrap

import mpmath
import numpy as np

from . import settings
from . import utils
from . import gpu
from . import _native as nat
from . import projection as fsproj
from .core import Fractal
from .numpy_utils import xrange as fsx

logger = logging.getLogger(__name__)


def mpc_lin_proj_impl_noscale(lin_mat, x, y):
    x1 = lin_mat[0, 0] * x + lin_mat[0, 1] * y
    y1 = lin_mat[1, 0] * x + lin_mat[1, 1] * y
    return mpmath.mpc(x1, y1)


class _XrangeArrayCompat(np.ndarray):
    """Stands for the reference's Xrange_array (numpy_utils/xrange.py:65) when
    its pickles are read: the record array (mantissa, exp) it is made of."""


class _RefPointUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module == "fractalshades.numpy_utils.xrange" and name == "Xrange_array":
            return _XrangeArrayCompat
        return super().find_class(module, name)


class PerturbationFractal(Fractal):

    #: 0 for the power-2 closures, n for the power-n model (z -> z^n + c)
    nexp = 0

    def __init__(self, directory):
        """Base class for escape-time fractals computed by perturbation
        around an arbitrary-precision reference orbit (z_0 = 0,
        z_{n+1} = f(z_n) + c)."""
        super().__init__(directory)

    @utils.zoom_options
    def zoom(self, *,
             precision: int,
             x: mpmath.mpf,
             y: mpmath.mpf,
             dx: mpmath.mpf,
             nx: int,
             xy_ratio: float,
             theta_deg: float,
             projection: fsproj.Projection = fsproj.Cartesian(),
             has_skew: bool = False,
             skew_00: float = 1.,
             skew_01: float = 0.,
             skew_10: float = 0.,
             skew_11: float = 1.):
        """Zoom parameters (perturbation.py:43-135): precision in decimal
        digits, x, y, dx as strings or mpmath numbers."""
        mpmath.mp.dps = precision
        self.x = mpmath.mpf(x)
        self.y = mpmath.mpf(y)
        self.dx = dx = mpmath.mpf(dx)
        if isinstance(projection, str):
            self.projection = projection = fsproj.Cartesian()
        self._skew = None
        if has_skew:
            self._skew = np.array(((skew_00, skew_01), (skew_10, skew_11)), dtype=np.float64)
        self.dx_std = float(dx)
        self.dx_xr = fsx.mpf_to_Xrange(dx)
        self.lin_mat = self.get_lin_mat()
        projection.adjust_to_zoom(self)
        self.proj_impl = projection.f
        pix = projection.min_local_scale * self.dx / self.nx
        with mpmath.workdps(6):
            required_dps = int(-mpmath.log10(pix / nx) + 1)
        if required_dps > precision:
            raise ValueError(
                "Precision is too low for min. pixel size and shall be "
                f"increased to {required_dps} (current setting: {precision}).")

    @property
    def xr_detect_activated(self):
        """Xrange deltas needed (perturbation.py:152-155): dx < 1e-300."""
        return self.dx < settings.xrange_zoom_level

    # ------------------------------------------------------------------
    # reference point storage (perturbation.py:256-314)
    # ------------------------------------------------------------------
    def ref_point_file(self):
        return os.path.join(self.directory, "data", "ref_pt.dat")

    def save_ref_point(self, FP_params, Zn_path):
        self._FP_params = FP_params
        self._Zn_path = Zn_path
        save_path = self.ref_point_file()
        utils.mkdir_p(os.path.dirname(save_path))
        with open(save_path, 'wb+') as tmpfile:
            pickle.dump(FP_params, tmpfile, pickle.HIGHEST_PROTOCOL)
            pickle.dump(Zn_path, tmpfile, pickle.HIGHEST_PROTOCOL)

    def reload_ref_point(self, scan_only=False):
        """(FP_params, Zn_path) from data/ref_pt.dat -- also a file written by
        the reference, whose Xrange values unpickle as (mantissa, exp)
        record arrays (perturbation.py:276-289)."""
        with open(self.ref_point_file(), 'rb') as tmpfile:
            FP_params = _RefPointUnpickler(tmpfile).load()
            if scan_only:
                return FP_params
            Zn_path = _RefPointUnpickler(tmpfile).load()
        return FP_params, Zn_path

    @property
    def FP_params(self):
        if hasattr(self, "_FP_params"):
            return self._FP_params
        self._FP_params = self.reload_ref_point(scan_only=True)
        return self._FP_params

    @property
    def Zn_path(self):
        if hasattr(self, "_Zn_path"):
            return self._Zn_path
        FP_params, Zn_path = self.reload_ref_point()
        self._Zn_path = Zn_path
        return Zn_path

    def ref_point_matching(self):
        """Can the stored orbit be reused (perturbation.py:211-253)?"""
        init_kwargs = self.init_kwargs
        del init_kwargs["directory"]
        try:
            ref_point = self.FP_params["ref_point"]
            max_iter_ref = self.FP_params["max_iter"]
            init_kwargs_ref = self.FP_params["init_kwargs"]
        except (FileNotFoundError, KeyError):
            return False
        drift = (self.x + 1j * self.y) - ref_point
        match = (
            mpmath.mp.dps <= self.FP_params["dps"] + 3
            and abs(drift / self.dx) ** 2 < 1.e6
            and max_iter_ref >= self.max_iter
            and all(init_kwargs.get(k) == v for k, v in init_kwargs_ref.items())
        )
        return bool(match)

    def ref_point_kc(self):
        """Bound of |dc| over the view, with a 1.1 margin
        (perturbation.py:166-194), as an Xrange."""
        w, h = self.projection.bounding_box(self.xy_ratio)
        dx = self.dx
        mat = self.lin_mat
        corners = [mpc_lin_proj_impl_noscale(mat, sx * 0.5 * w, sy * 0.5 * h) * dx
                   for sx, sy in ((1, 1), (-1, 1), (-1, -1), (1, -1))]
        c0 = self.x + 1j * self.y
        shift = self.FP_params["ref_point"] - c0
        kc = max(abs(shift - c) for c in corners) * 1.1
        return fsx.mpf_to_Xrange(kc)

    # ------------------------------------------------------------------
    # reference orbit (perturbation.py:651-854)
    # ------------------------------------------------------------------
    def get_FP_orbit(self, c0=None, newton="cv", order=None, max_newton=None):
        if newton == "step":
            raise NotImplementedError("step option not Implemented (yet)")
        if self.ref_point_matching():
            logger.info("Reference point already stored, skipping calc")
            return
        if self.dx > settings.newton_zoom_level:
            self.compute_critical_orbit(self.critical_pt)
            return
        if c0 is None:
            c0 = self.x + 1j * self.y
        if settings.no_newton or (newton is None) or (newton == "None"):
            self.compute_FP_orbit(c0, None)
            return
        if order is None:
            order = self.ball_method(c0, self.dx * 1.0)
            if order is None:
                logger.warning("Ball method failed - Default to image center")
                self.compute_FP_orbit(c0, None)
                return
        max_attempt = 2
        eps_pixel = self.dx * (1. / self.nx)
        try:
            newton_cv, nucleus = self.find_nucleus(c0, order, eps_pixel, max_newton=max_newton)
        except NotImplementedError:
            newton_cv, nucleus = self.find_any_nucleus(c0, order, eps_pixel, max_newton=max_newton)
        attempt = 1
        if not newton_cv:
            while not newton_cv and attempt <= max_attempt:
                attempt += 1
                mpmath.mp.dps = int(1.25 * mpmath.mp.dps)
                eps_pixel = self.dx * (1. / self.nx)
                try:
                    no_div = True
                    newton_cv, nucleus = self.find_nucleus(c0, order, eps_pixel,
                                                           max_newton=max_newton)
                except NotImplementedError:
                    no_div = False
                    newton_cv, nucleus = self.find_any_nucleus(c0, order, eps_pixel,
                                                               max_newton=max_newton)
                if no_div and not newton_cv and attempt == max_attempt:
                    newton_cv, nucleus = self.find_any_nucleus(c0, order, eps_pixel,
                                                               max_newton=max_newton)
        if not newton_cv:
            order = None
            nucleus = c0
            logger.warning("Newton descent failed - Default to image center")
        self.compute_FP_orbit(nucleus, order)

    def compute_critical_orbit(self, crit):
        """Shallow zoom: a constant 'orbit' at the critical point, order 100
        (perturbation.py:770-805)."""
        div_iter = 100
        init_kwargs = self.init_kwargs
        del init_kwargs["directory"]
        FP_params = {"ref_point": mpmath.mpc(crit), "dps": mpmath.mp.dps, "order": 100,
                     "max_iter": self.max_iter, "FP_code": self.FP_code, "partials": {},
                     "xr": {}, "div_iter": div_iter, "init_kwargs": init_kwargs}
        Zn_path = np.zeros([div_iter + 1], dtype=np.complex128)
        Zn_path[:] = crit
        self.save_ref_point(FP_params, Zn_path)

    def compute_FP_orbit(self, ref_point, order=None):
        """Full precision orbit stored in FP64 (+ Xrange side table)
        (perturbation.py:808-854)."""
        max_iter = self.max_iter
        FP_params = {"ref_point": ref_point, "dps": mpmath.mp.dps, "order": order,
                     "max_iter": max_iter, "FP_code": self.FP_code}
        ref_orbit_len = max_iter + 1
        if order is not None:
            ref_orbit_len = min(order, ref_orbit_len)
        FP_params["ref_orbit_len"] = ref_orbit_len
        Zn_path = np.empty([ref_orbit_len], dtype=np.complex128)
        i, partial_dict, xr_dict = self.FP_loop(Zn_path, ref_point)
        FP_params["partials"] = partial_dict
        FP_params["xr"] = xr_dict
        FP_params["div_iter"] = i
        init_kwargs = self.init_kwargs
        del init_kwargs["directory"]
        FP_params["init_kwargs"] = init_kwargs
        self.save_ref_point(FP_params, Zn_path)

    def ball_method(self, c, px, kind=1, M_divergence=1.e5):
        return self._ball_method(c, px, self.max_iter, M_divergence)

    # ------------------------------------------------------------------
    # GPU-side data (perturbation.py:317-375, 431-562)
    # ------------------------------------------------------------------
    def get_path_data(self):
        FP_params = self.FP_params
        Zn_path = self.Zn_path
        ref_xr_python = FP_params["xr"]
        has_xr = len(ref_xr_python) > 0
        ref_order = FP_params["order"]
        ref_div_iter = FP_params["div_iter"]
        if ref_order is not None:
            ref_div_iter = self.max_iter + 1
        dx_xr = fsx.mpf_to_Xrange(self.dx)
        if self.holomorphic:
            drift_xr = fsx.mpc_to_Xrange((self.x + 1j * self.y) - FP_params["ref_point"])
            idx, m, e = fsx.xr_table(ref_xr_python)
            return (Zn_path, has_xr, idx, (m, e), ref_div_iter, ref_order, drift_xr, dx_xr)
        refp = FP_params["ref_point"]
        driftx_xr = fsx.mpf_to_Xrange(self.x - refp.real)
        drifty_xr = fsx.mpf_to_Xrange(self.y - refp.imag)
        idx, m, e = fsx.xr_table_xy(ref_xr_python)
        return (Zn_path, has_xr, idx, (m, e), ref_div_iter, ref_order,
                driftx_xr, drifty_xr, dx_xr)

    @staticmethod
    def numba_cycle_call(cycle_dep_args, cycle_indep_args):
        """numba_cycles_perturb(_BS) replacement (perturbation.py:414-428):
        iterate one tile on the GPU, arrays filled in place; returns 0 or
        USER_INTERRUPTED."""
        return gpu.run_perturb_pixels(cycle_dep_args, cycle_indep_args)

    def get_cycle_indep_args(self, initialize, iterate):
        """Reference orbit, derivative paths and BLA tree for this calculation
        (perturbation.py:431-562), the latter two built on the GPU."""
        holomorphic = self.holomorphic
        calc_deriv_c = self.calc_dZndc if holomorphic else self.calc_hessian
        calc_dZndz = self.calc_dZndz if holomorphic else False
        self.get_FP_orbit()
        pd = self.get_path_data()
        if holomorphic:
            (Zn_path, has_xr, ref_index_xr, ref_xr, ref_div_iter, ref_order,
             drift_xr, dx_xr) = pd
        else:
            (Zn_path, has_xr, ref_index_xr, ref_xr, ref_div_iter, ref_order,
             driftx_xr, drifty_xr, dx_xr) = pd
        if ref_order is None:
            ref_order = (1 << 62)
        # the derivative paths' scale: dx times the projection's
        # (perturbation.py:459-468)
        scale = dx_xr
        if self.projection.scale != 1.:
            # dx_xr * scale_xr as the reference's Xrange product: the
            # mantissas' double product
            sx = fsx.mpf_to_Xrange(self.projection.scale)
            scale = fsx.XrScalar(dx_xr.m * sx.m, dx_xr.e + sx.e)
        self.kc = kc = self.ref_point_kc()
        if kc.to_standard() == 0.:
            raise RuntimeError(
                "Resolution is too low for this zoom depth. Try to increase"
                "the reference calculation precicion.")
        bla_eps = self.BLA_eps
        xr = self.xr_detect_activated
        # Burning Ship below the double range: the Jacobian paths (double for
        # the FP32 + exponent form, Xrange records for the Xrange branch) at
        # the scale m (dx = m 2^e), the tiles add 2^e (fsg_tile.dzndc_scale_e):
        # the recurrences are linear in the scale and a power of two is exact
        dzndc_scale_e = 0
        if xr and not holomorphic:
            scale = fsx.XrScalar(dx_xr.m, 0)
            dzndc_scale_e = dx_xr.e
        ref = nat.Reference(
            gpu.context(), Zn_path, div_iter=ref_div_iter,
            order=(ref_order if ref_order < (1 << 62) else None),
            flavor=0 if holomorphic else self.flavor_int,
            xr_idx=ref_index_xr if has_xr else None,
            xr_m=ref_xr[0] if has_xr else None, xr_e=ref_xr[1] if has_xr else None,
            xr_paths=xr, calc_dzndc=calc_deriv_c,
            calc_dzndz=calc_dZndz, scale_m=scale.m, scale_e=scale.e,
            bla=bla_eps is not None, kc=kc.to_standard(),
            bla_eps=bla_eps if bla_eps is not None else 0.,
            nexp=self.nexp if holomorphic else 0)
        args = {"holomorphic": holomorphic, "spec": iterate, "ref": ref,
                "lin_mat": self.lin_mat, "dx_m": dx_xr.m, "dx_e": dx_xr.e,
                "interrupted": self._interrupted, "kc": kc,
                "ref_div_iter": ref_div_iter, "ref_order": ref_order, "has_xr": has_xr,
                "dzndc_scale_e": dzndc_scale_e,
                "proj": fsproj.kernel_params(self.projection)}
        if holomorphic:
            args.update(drift_m=drift_xr.m, drift_e=drift_xr.e)
        else:
            args.update(driftx_m=driftx_xr.m, driftx_e=driftx_xr.e,
                        drifty_m=drifty_xr.m, drifty_e=drifty_xr.e)
        return args

    def get_std_cpt(self, c_pix):
        """c of each pixel in double (perturbation.py:196-207 std_C_from_pix)."""
        center = complex(self.x + 1j * self.y)
        if getattr(self.projection, "kernel_kind", 0):
            c_pix = self.projection.f(np.asarray(c_pix))
        x, y = c_pix.real, c_pix.imag
        m = self.lin_mat
        x1 = m[0, 0] * x + m[0, 1] * y
        y1 = m[1, 0] * x + m[1, 1] * y
        return center + self.dx_std * (x1 + 1j * y1)

    @staticmethod
    def print_FP(FP_params, Zn_path):
        pp = "  Full precision orbit loaded, FP_params:"
        for k, v in FP_params.items():
            pp += f"  {k} --> {v}"
        pp += f"ref_path, shape: {Zn_path.shape}, {Zn_path.dtype}"
        logger.info(textwrap.shorten(pp, 2000))
