"""
GPU execution of the iteration path: a process-wide library context and the
calls that replace the reference's numba loops.

* ``StdSpec`` / ``PerturbSpec``: what the model's ``iterate()`` factory
  returns -- the calculation options of one calc_std_div call, in place of a
  numba closure.
* ``run_std_pixels`` / ``run_perturb_pixels``: one tile, reference contract
  (c_pix, Z, U, stop_reason, stop_iter filled in place) through the C-ABI with
  host buffers.
* ``run_image``: every tile of an image in one launch.
"""
import threading

import numpy as np

from . import settings
from . import tune
from . import _native as nat

_ctx_lock = threading.Lock()
_ctx = None


def context():
    """The library context of this process (device settings.gpu_device)."""
    global _ctx
    with _ctx_lock:
        if _ctx is None:
            _ctx = nat.Context(settings.gpu_device)
        return _ctx


_dev_name = None


def _shaped_calc(spec, perturb):
    """The spec's calculation with the launch shape the autotuner cached for
    its kernel kind (fractalshades_gb300.tune), if any."""
    global _dev_name
    if _dev_name is None:
        _dev_name = tune._device_name(context())
    return tune.apply(spec.calc(), perturb, _dev_name)


def cancel():
    if _ctx is not None:
        _ctx.cancel()


def clear_cancel():
    if _ctx is not None:
        _ctx.clear_cancel()


class StdSpec:
    """Options of a standard (non-perturbation) calculation."""

    def __init__(self, *, flavor, max_iter, M_divergence, epsilon_stationnary=0., nexp=0,
                 calc_d2zndc2=False, backshift=0):
        self.flavor = int(flavor)
        self.max_iter = int(max_iter)
        self.M_divergence = float(M_divergence)
        self.epsilon_stationnary = float(epsilon_stationnary)
        self.nexp = int(nexp)     # 0: power-2 model, n: power-n model
        self.calc_d2zndc2 = bool(calc_d2zndc2)
        self.backshift = int(backshift)   # > 0: calc_orbit

    def calc(self):
        return nat.make_calc(max_iter=self.max_iter, M_divergence=self.M_divergence,
                             epsilon_stationnary=self.epsilon_stationnary,
                             flavor=self.flavor, nexp=self.nexp,
                             calc_d2zndc2=self.calc_d2zndc2, backshift=self.backshift)

    @property
    def i_znorbit(self):
        """Z row of zn_orbit (xn_orbit for the Burning Ship family), after the
        reference's other codes (mandelbrot_M2.py:107-124, burning_ship.py:264-280)"""
        if self.flavor != 0:
            return 6
        return 3 + int(self.calc_d2zndc2)

    @property
    def nZ(self):
        if self.flavor != 0:
            return 6 + (2 if self.backshift > 0 else 0)
        return 3 + int(self.calc_d2zndc2) + int(self.backshift > 0)


class PerturbSpec:
    """Options of a perturbation calculation."""

    def __init__(self, *, flavor, max_iter, M_divergence, epsilon_stationnary=0.,
                 calc_dzndc=True, interior=False, bla=True, xr_detect_activated=False,
                 i_dzndz=-1, i_dzndc=-1, nZ=1, nexp=0, backshift=0, i_znorbit=0):
        self.flavor = int(flavor)
        self.max_iter = int(max_iter)
        self.M_divergence = float(M_divergence)
        self.epsilon_stationnary = float(epsilon_stationnary)
        self.calc_dzndc = bool(calc_dzndc)
        self.interior = bool(interior)
        self.bla = bool(bla)
        self.xr_detect_activated = bool(xr_detect_activated)
        self.i_dzndz = int(i_dzndz)
        self.i_dzndc = int(i_dzndc)
        self.nZ = int(nZ)
        self.nexp = int(nexp)     # 0: power-2 model, n: power-n model
        self.backshift = int(backshift)   # > 0: calc_orbit, orbit row(s) at i_znorbit
        self.i_znorbit = int(i_znorbit)

    @property
    def mode(self):
        m = settings.precision_mode
        if self.backshift > 0:
            # the orbit snapshots are kept by the reference's two delta forms
            if m == "fe32" or (self.flavor != 0 and self.xr_detect_activated):
                raise ValueError("calc_orbit runs in the FP64 / Xrange forms: precision_mode "
                                 "'auto', 'fp64' or 'xr64' (Burning Ship: above dx = 1e-300)")
        if self.nexp != 0:
            # power-n model: the reference's two delta forms (no FE32 kernel)
            if m == "fe32":
                raise ValueError("the power-n model runs with precision_mode 'auto', "
                                 "'fp64' or 'xr64'")
            if m == "auto":
                return "xr64" if self.xr_detect_activated else "fp64"
            return m
        if self.flavor != 0:
            # Burning Ship: the reference's two branches (Xrange below
            # dx = 1e-300), or the FP32 + exponent form
            if self.xr_detect_activated:
                if m == "fp64":
                    raise ValueError("Burning Ship below dx = 1e-300 runs with "
                                     "precision_mode 'auto', 'xr64' or 'fe32'")
                return "xr64" if m == "auto" else m
            return "fp64" if m in ("auto", "xr64") else m
        if m == "auto":
            return "xr64" if self.xr_detect_activated else "fp64"
        return m

    def calc(self):
        return nat.make_calc(max_iter=self.max_iter, M_divergence=self.M_divergence,
                             epsilon_stationnary=self.epsilon_stationnary, mode=self.mode,
                             calc_dzndc=self.calc_dzndc, interior=self.interior,
                             bla=self.bla, flavor=self.flavor,
                             xr_semantics=self.xr_detect_activated, nexp=self.nexp,
                             backshift=self.backshift)


def _check_rc(rc):
    return 1 if rc == nat.FSG_INTERRUPTED else 0


def run_std_pixels(cycle_dep_args, cycle_indep_args):
    """numba_cycles replacement (core.py:2935-2963): one tile of pixels given
    as the reference's c_pix array."""
    c_pix, Z, U, stop_reason, stop_iter = cycle_dep_args
    (_init, spec, center, proj, lin_mat, dx, interrupted) = cycle_indep_args
    if interrupted[0]:
        return 1
    if c_pix.size == 0:
        return 0
    ctx = context()
    pix = np.ascontiguousarray(c_pix, dtype=np.complex128)
    Zw = Z if Z.flags.c_contiguous else np.ascontiguousarray(Z)
    t = nat.make_tile(pix=pix, lin_mat=lin_mat, Z=Zw, stop_reason=stop_reason,
                      stop_iter=stop_iter, center=center, dx=dx, i_znorbit=spec.i_znorbit,
                      proj=proj)
    rc = ctx.std_tiles(_shaped_calc(spec, False), [t], nat.HOST)
    if Zw is not Z:
        Z[...] = Zw
    return _check_rc(rc)


def _tile_for(fractal_args, spec, pix=None, xs=None, ys=None, Z=None, U=None, sr=None,
              si=None, pot=None, dem=None):
    ref = fractal_args["ref"]
    kw = dict(lin_mat=fractal_args["lin_mat"], Z=Z, U=U, stop_reason=sr, stop_iter=si,
              ref=ref, dx_m=fractal_args["dx_m"], dx_e=fractal_args["dx_e"],
              i_dzndz=spec.i_dzndz, i_dzndc=spec.i_dzndc, potential=pot, dem=dem,
              dzndc_scale_e=fractal_args.get("dzndc_scale_e", 0), i_znorbit=spec.i_znorbit,
              proj=fractal_args.get("proj"))
    if spec.flavor == 0:
        kw.update(drift_m=fractal_args["drift_m"], drift_e=fractal_args["drift_e"])
    else:
        kw.update(drift_m=fractal_args["driftx_m"], drift_e=fractal_args["driftx_e"],
                  drifty_m=fractal_args["drifty_m"], drifty_e=fractal_args["drifty_e"])
    if pix is not None:
        return nat.make_tile(pix=pix, **kw)
    return nat.make_tile(xs=xs, ys=ys, **kw)


def run_perturb_pixels(cycle_dep_args, cycle_indep_args):
    """numba_cycles_perturb(_BS) replacement (perturbation.py:988-1045,
    1406-1451): one tile of pixels given as the reference's c_pix array."""
    c_pix, Z, U, stop_reason, stop_iter = cycle_dep_args
    args = cycle_indep_args
    if args["interrupted"][0]:
        return 1
    if c_pix.size == 0:
        return 0
    spec = args["spec"]
    ctx = context()
    pix = np.ascontiguousarray(c_pix, dtype=np.complex128)
    Zw = Z if Z.flags.c_contiguous else np.ascontiguousarray(Z)
    Uw = U if U.shape[0] > 0 else None
    t = _tile_for(args, spec, pix=pix, Z=Zw, U=Uw, sr=stop_reason, si=stop_iter)
    rc = ctx.perturb_tiles(_shaped_calc(spec, True), [t], nat.HOST)
    if Zw is not Z:
        Z[...] = Zw
    return _check_rc(rc)


def run_image(fractal, xs, ys, cycle_indep_args, potential=True):
    """Every pixel of the image in one launch (host buffers).  Returns the raw
    arrays (Z [nZ, n], U, stop_reason, stop_iter, potential, dem) with pixels
    in row-major image order."""
    ctx = context()
    n = xs.size * ys.size
    complex_type = fractal.complex_type
    nZ = len(fractal.codes[0])
    nU = len(fractal.codes[1])
    Z = np.zeros((nZ, n), dtype=complex_type)
    U = np.zeros((max(nU, 1), n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    pot = np.zeros(n) if potential else None
    dem = np.zeros(n) if potential else None
    if isinstance(cycle_indep_args, dict):
        spec = cycle_indep_args["spec"]
        if spec.flavor == 0 and not spec.calc_dzndc:
            dem = None
        t = _tile_for(cycle_indep_args, spec, xs=xs, ys=ys, Z=Z,
                      U=U if nU else None, sr=sr, si=si, pot=pot, dem=dem)
        rc = ctx.perturb_tiles(_shaped_calc(spec, True), [t], nat.HOST)
    else:
        (_init, spec, center, proj, lin_mat, dx, interrupted) = cycle_indep_args
        t = nat.make_tile(xs=xs, ys=ys, lin_mat=lin_mat, Z=Z, stop_reason=sr, stop_iter=si,
                          center=center, dx=dx, potential=pot, dem=dem,
                          i_znorbit=spec.i_znorbit, proj=proj)
        rc = ctx.std_tiles(_shaped_calc(spec, False), [t], nat.HOST)
    if rc == nat.FSG_INTERRUPTED:
        return None
    return {"Z": Z, "U": U[:nU], "stop_reason": sr[0], "stop_iter": si[0],
            "potential": pot, "dem": dem, "stats": ctx.stats()}
