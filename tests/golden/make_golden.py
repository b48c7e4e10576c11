"""
Generate golden vectors by running the reference (Fractalshades 1.2.1) itself.

The reference cannot run as shipped here: numba, gmpy2 and PIL are absent.
This script imports it from its source tree with three stand-ins:

* ``numba``: ``njit``/``jit`` become identity decorators, so the reference's
  hot-path functions run as plain Python, statement for statement;
* ``fractalshades.numpy_utils.numba_xr``: the four functions the hot path calls
  (``to_standard``, ``to_Xrange_scalar``, ``extended_abs2``, ``one``) are
  mapped onto the reference's own host ``Xrange_array`` class
  (``numpy_utils/xrange.py``), whose arithmetic the numba extension mirrors;
* ``PIL`` and the Cython module ``mpmath_utils/FP_loop``: unused stubs.  The
  reference orbit is computed here in mpmath with the recurrence of
  ``FP_loop.pyx:274-421`` and stored through the reference's own
  ``save_ref_point`` so that ``get_FP_orbit`` reuses it.

Two lowering rules of numba are applied to the reference modules when they are
loaded (an AST rewrite, nothing else changes): ``x ** 2`` with a literal
integer exponent becomes ``x * x`` (numba's static power), and ``abs`` /
``np.abs`` of a complex scalar becomes the C library's ``hypot(re, im)``
(numba's complex abs).  Plain CPython would call libm ``pow`` and numpy's vectorised complex
abs, which are not always correctly rounded and differ from numba in the last
bit.

Everything else -- pixel grid (``chunk_pixel_pos``), ``get_cycle_indep_args``,
the derivative paths, ``ref_point_kc``, the BLA tree, ``numba_cycles`` /
``numba_cycles_perturb(_BS)`` -- is the reference's code.  Python evaluates each
floating point operation once, in source order, with IEEE rounding, which is
what the oracle restates (the jitted reference may contract some operations
into FMAs under ``fastmath=True``).

Usage: python tests/golden/make_golden.py <reference_src_dir> [case]
(or the source directory in $FRACTALSHADES_SRC: the reference's ``src``
folder, the one holding the ``fractalshades`` package).
Writes tests/golden/*.npz (small fixtures, committed).
"""
import os
import sys
import tempfile
import types

import numpy as np
import mpmath

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FRACTALSHADES_SRC")
if not REF_SRC or not os.path.isdir(os.path.join(REF_SRC, "fractalshades")):
    sys.exit("usage: make_golden.py <reference_src_dir> [case]  (the folder that holds the "
             "reference's fractalshades package; or set FRACTALSHADES_SRC)")


# --------------------------------------------------------------------------
# Stand-ins
# --------------------------------------------------------------------------
class _Any:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return _Any()

    def __getattr__(self, name):
        return _Any()

    def __getitem__(self, k):
        return _Any()

    def __iter__(self):
        return iter(())


def _njit(*a, **k):
    if len(a) == 1 and callable(a[0]) and not k:
        return a[0]
    return lambda f: f


class _NumbaLowering(__import__("ast").NodeTransformer):
    """x ** 2 -> x * x ; abs(z) / np.abs(z) -> _nb_abs(z)."""

    def visit_BinOp(self, node):
        import ast
        self.generic_visit(node)
        if (isinstance(node.op, ast.Pow) and isinstance(node.right, ast.Constant)
                and node.right.value == 2 and isinstance(node.left, (
                    ast.Name, ast.Subscript, ast.Attribute))):
            return ast.copy_location(
                ast.BinOp(left=node.left, op=ast.Mult(), right=node.left), node)
        return node

    def visit_Call(self, node):
        import ast
        self.generic_visit(node)
        f = node.func
        is_abs = isinstance(f, ast.Name) and f.id == "abs"
        is_npabs = (isinstance(f, ast.Attribute) and f.attr == "abs"
                    and isinstance(f.value, ast.Name) and f.value.id == "np")
        if (is_abs or is_npabs) and len(node.args) == 1:
            node.func = ast.copy_location(ast.Name(id="_nb_abs", ctx=ast.Load()), f)
        return node


def _libm_hypot():
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.hypot.argtypes = [ctypes.c_double, ctypes.c_double]
    libm.hypot.restype = ctypes.c_double
    return libm.hypot


_HYPOT = _libm_hypot()


def _nb_abs(x):
    # numba lowers abs(complex) to a call of the C library's hypot
    # (CPython's math.hypot is a different algorithm)
    if isinstance(x, (complex, np.complexfloating)):
        return np.float64(_HYPOT(float(x.real), float(x.imag)))
    if isinstance(x, (float, np.floating, int, np.integer)):
        return abs(x)
    return np.abs(x)


def _install_lowering_loader():
    import ast
    import builtins
    import importlib.abc
    import importlib.machinery
    builtins._nb_abs = _nb_abs

    class Loader(importlib.machinery.SourceFileLoader):
        def source_to_code(self, data, path, *, _optimize=-1):
            tree = ast.parse(data, filename=path)
            tree = ast.fix_missing_locations(_NumbaLowering().visit(tree))
            return compile(tree, path, "exec", dont_inherit=True)

        def get_code(self, fullname):
            # never reuse a cached (unrewritten) bytecode file
            return self.source_to_code(self.get_data(self.path), self.path)

    class Finder(importlib.abc.MetaPathFinder):
        def find_spec(self, name, path, target=None):
            if not name.startswith("fractalshades"):
                return None
            spec = importlib.machinery.PathFinder.find_spec(name, path)
            if spec is None or not str(spec.origin).endswith(".py"):
                return spec
            spec.loader = Loader(name, spec.origin)
            return spec

    sys.meta_path.insert(0, Finder())


def install_shims():
    _install_lowering_loader()
    nb = types.ModuleType("numba")
    nb.njit = nb.jit = nb.vectorize = nb.guvectorize = _njit
    nb.complex128, nb.float64, nb.int32, nb.int64 = (
        np.complex128, np.float64, np.int32, np.int64)
    nb.bool_ = nb.boolean = np.bool_
    nb.intp, nb.uint8, nb.int8 = np.intp, np.uint8, np.int8
    nb.prange = range
    nb.types = nb.core = nb.extending = nb.np = nb.cpython = _Any()
    nb.from_dtype = lambda d: d
    sys.modules["numba"] = nb
    for sub in ["numba.core", "numba.core.types", "numba.core.cgutils",
                "numba.extending", "numba.core.errors", "numba.np",
                "numba.np.numpy_support", "numba.cpython",
                "numba.cpython.unsafe", "numba.cpython.unsafe.numbers",
                "numba.typed"]:
        sys.modules[sub] = _Any()
    pil = types.ModuleType("PIL")
    pil.Image = _Any()
    pil.PngImagePlugin = _Any()
    sys.modules["PIL"] = pil
    sys.modules["PIL.PngImagePlugin"] = pil.PngImagePlugin
    sys.modules["PIL.Image"] = pil.Image

    xrm = types.ModuleType("fractalshades.numpy_utils.numba_xr")

    def _fsx():
        import fractalshades.numpy_utils.xrange as fsx
        return fsx

    def to_standard(item):
        fsx = _fsx()
        if isinstance(item, fsx.Xrange_array):
            return item.to_standard()[()]
        return item

    def to_Xrange_scalar(item):
        fsx = _fsx()
        if isinstance(item, fsx.Xrange_array):
            return item
        dt = np.complex128 if np.iscomplexobj(item) else np.float64
        return fsx.Xrange_array(np.asarray(item, dtype=dt))

    def extended_abs2(item):
        fsx = _fsx()
        if isinstance(item, fsx.Xrange_array):
            return item.abs2()
        return item.real ** 2 + item.imag ** 2

    def one():
        fsx = _fsx()
        return fsx.Xrange_array(np.asarray(1., dtype=np.float64))

    xrm.to_standard = to_standard
    xrm.to_Xrange_scalar = to_Xrange_scalar
    xrm.extended_abs2 = extended_abs2
    xrm.one = one
    sys.modules["fractalshades.numpy_utils.numba_xr"] = xrm

    fp = types.ModuleType("fractalshades.mpmath_utils.FP_loop")
    mu = types.ModuleType("fractalshades.mpmath_utils")
    mu.FP_loop = fp
    mu.__path__ = []
    sys.modules["fractalshades.mpmath_utils"] = mu
    sys.modules["fractalshades.mpmath_utils.FP_loop"] = fp
    sys.path.insert(0, REF_SRC)


install_shims()
import fractalshades as fs                       # noqa: E402
import fractalshades.models as fsm               # noqa: E402
import fractalshades.numpy_utils.xrange as fsx   # noqa: E402


# --------------------------------------------------------------------------
# Helpers
# --------------------------------------------------------------------------
def mp_orbit(c, max_iter, M, need_xr, ref_orbit_len, xr_threshold=None):
    """mpmath restatement of FP_loop.pyx:274-421 (orbit stored as float64).
    ``xr_threshold``: the side-table threshold; FP_loop.pyx:143 reads
    settings.xrange_zoom_level once, when the module is imported."""
    tshold = fs.settings.xrange_zoom_level if xr_threshold is None else xr_threshold
    orbit = np.zeros(ref_orbit_len, dtype=np.complex128)
    z = mpmath.mpc(0)
    xr_dict = {}
    i = 0
    abs_i = 0.
    for i in range(1, ref_orbit_len):
        z = z * z + c
        x, y = float(z.real), float(z.imag)
        orbit[i] = complex(x, y)
        abs_i = np.hypot(x, y)
        if abs_i > M:
            break
        if need_xr and abs_i < tshold:
            xr_dict[i] = fsx.mpc_to_Xrange(z)
    if i == ref_orbit_len - 1 and abs_i <= M:
        i += 1
    return i, orbit, xr_dict


def mp_orbit_n(c, nexp, max_iter, M, need_xr, ref_orbit_len):
    """mp_orbit for z^n + c (FP_loop.pyx:255-421, mpc_pow_ui)."""
    orbit = np.zeros(ref_orbit_len, dtype=np.complex128)
    z = mpmath.mpc(0)
    xr_dict = {}
    i = 0
    abs_i = 0.
    for i in range(1, ref_orbit_len):
        z = z ** nexp + c
        x, y = float(z.real), float(z.imag)
        orbit[i] = complex(x, y)
        abs_i = np.hypot(x, y)
        if abs_i > M:
            break
        if need_xr and abs_i < fs.settings.xrange_zoom_level:
            xr_dict[i] = fsx.mpc_to_Xrange(z)
    if i == ref_orbit_len - 1 and abs_i <= M:
        i += 1
    return i, orbit, xr_dict


def mp_nucleus_n(nexp, p, dps, c0):
    """Newton for f^p(0) = 0 with f = z^n + c, from c0."""
    with mpmath.workdps(dps):
        c = mpmath.mpc(c0)
        for _ in range(200):
            z = mpmath.mpc(0)
            d = mpmath.mpc(0)
            for _k in range(p):
                d = nexp * z ** (nexp - 1) * d + 1
                z = z ** nexp + c
            dc = z / d
            c = c - dc
            if abs(dc) < mpmath.mpf(10) ** (-dps + 5):
                break
        return c


def mp_nucleus(p, dps, seed_frac=0.):
    """Newton for a period-p nucleus from a start outside the 1/p bulb root."""
    with mpmath.workdps(dps):
        th = 2 * mpmath.pi / p
        c = mpmath.expj(th) / 2 - mpmath.expj(2 * th) / 4
        c = c * (1 + mpmath.mpf(1) / (p * p) * (1 + seed_frac))
        for _ in range(200):
            z = mpmath.mpc(0)
            d = mpmath.mpc(0)
            for _k in range(p):
                d = 2 * z * d + 1
                z = z * z + c
            dc = z / d
            c = c - dc
            if abs(dc) < mpmath.mpf(10) ** (-dps + 5):
                break
        return c


def store_orbit(f, ref_point, order, max_iter, M, xr_threshold=None):
    """Store an orbit where the reference looks for it (perturbation.py:256-274)."""
    ref_orbit_len = max_iter + 1
    if order is not None:
        ref_orbit_len = min(order, ref_orbit_len)
    i, orbit, xr_dict = mp_orbit(ref_point, max_iter, 2 * M,
                                 f.xr_detect_activated, ref_orbit_len, xr_threshold)
    init_kwargs = f.init_kwargs
    del init_kwargs["directory"]
    FP_params = {
        "ref_point": ref_point, "dps": mpmath.mp.dps, "order": order,
        "max_iter": max_iter, "FP_code": f.FP_code, "partials": {},
        "xr": xr_dict, "div_iter": i, "init_kwargs": init_kwargs,
        "ref_orbit_len": ref_orbit_len,
    }
    f.save_ref_point(FP_params, orbit)
    return FP_params, orbit


def store_orbit_n(f, nexp, ref_point, order, max_iter, M):
    """store_orbit for z^n + c."""
    ref_orbit_len = max_iter + 1
    if order is not None:
        ref_orbit_len = min(order, ref_orbit_len)
    i, orbit, xr_dict = mp_orbit_n(ref_point, nexp, max_iter, 2 * M,
                                   f.xr_detect_activated, ref_orbit_len)
    init_kwargs = f.init_kwargs
    del init_kwargs["directory"]
    FP_params = {
        "ref_point": ref_point, "dps": mpmath.mp.dps, "order": order,
        "max_iter": max_iter, "FP_code": f.FP_code, "partials": {},
        "xr": xr_dict, "div_iter": i, "init_kwargs": init_kwargs,
        "ref_orbit_len": ref_orbit_len,
    }
    f.save_ref_point(FP_params, orbit)
    return FP_params, orbit


def xr_arrays(path):
    """Split an Xrange_array into (mantissa, exp) numpy arrays."""
    return np.asarray(path._mantissa), np.asarray(path._exp, dtype=np.int32)


def run_tile(f, calc_name):
    chunk = (0, f.nx, 0, f.ny)
    (c_pix, Z, U, stop_reason, stop_iter), _ = f.get_cycling_dep_args(
        calc_name, chunk)
    cia = f._calc_data[calc_name]["cycle_indep_args"]
    ret = f.numba_cycle_call((c_pix, Z, U, stop_reason, stop_iter), cia)
    assert ret == 0
    return c_pix, Z, U, stop_reason, stop_iter, cia


# --------------------------------------------------------------------------
# Cases
# --------------------------------------------------------------------------
def golden_std_m2(out):
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Mandelbrot(d)
        f.zoom(x=-0.5, y=0., dx=3., nx=48, xy_ratio=4. / 3., theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=400,
                       M_divergence=1000., epsilon_stationnary=0.01)
        c_pix, Z, U, sr, si, cia = run_tile(f, "std")
        np.savez_compressed(
            out, pix=c_pix, Z=Z, stop_reason=sr, stop_iter=si,
            center=np.array([-0.5, 0.]), lin_mat=f.lin_mat, dx=3.,
            max_iter=400, M=1000., eps=0.01, nx=f.nx, ny=f.ny)


def golden_std_bs(out):
    res = {}
    for flavor_int, flavor in enumerate(
            ["Burning ship", "Perpendicular burning ship", "Shark fin",
             "Celtic", "Buffalo"], start=1):
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Burning_ship(d, flavor=flavor)
            f.zoom(x=-0.5, y=-0.5, dx=3.5, nx=24, xy_ratio=1., theta_deg=0.)
            f.calc_std_div(calc_name="std", subset=None, max_iter=200,
                           M_divergence=1000.)
            c_pix, Z, U, sr, si, cia = run_tile(f, "std")
            res[f"pix_{flavor_int}"] = c_pix
            res[f"Z_{flavor_int}"] = Z
            res[f"stop_reason_{flavor_int}"] = sr
            res[f"stop_iter_{flavor_int}"] = si
            res["lin_mat"] = f.lin_mat
    np.savez_compressed(out, center=np.array([-0.5, -0.5]), dx=3.5,
                        max_iter=200, M=1000., **res)


def golden_perturb_m2(out, *, x, y, dx, nx, precision, order, max_iter,
                      interior, bla_eps=1e-6, eps_stat=1e-3, M=1000.,
                      ref_shift=0j, x_offset="0", backshift=0, projection=None,
                      xr_zoom_level=None):
    """``xr_zoom_level``: settings.xrange_zoom_level while the view is set up
    and iterated (the Xrange branch then runs at widths below it); the orbit's
    side table keeps the import-time threshold 1e-300 (FP_loop.pyx:143)."""
    saved = fs.settings.xrange_zoom_level
    if xr_zoom_level is not None:
        fs.settings.xrange_zoom_level = xr_zoom_level
    try:
        _golden_perturb_m2(out, x=x, y=y, dx=dx, nx=nx, precision=precision, order=order,
                           max_iter=max_iter, interior=interior, bla_eps=bla_eps,
                           eps_stat=eps_stat, M=M, ref_shift=ref_shift, x_offset=x_offset,
                           backshift=backshift, projection=projection,
                           xr_threshold=None if xr_zoom_level is None else saved)
    finally:
        fs.settings.xrange_zoom_level = saved


def _golden_perturb_m2(out, *, x, y, dx, nx, precision, order, max_iter,
                       interior, bla_eps, eps_stat, M, ref_shift, x_offset, backshift,
                       projection, xr_threshold):
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Perturbation_mandelbrot(d)
        x = str(mpmath.mpf(x) + mpmath.mpf(x_offset))
        f.zoom(precision=precision, x=x, y=y, dx=dx, nx=nx, xy_ratio=1.,
               theta_deg=0., projection=projection or fs.projection.Cartesian())
        ref_point = mpmath.mpc(x, y) + mpmath.mpc(ref_shift) * mpmath.mpf(dx)
        f.max_iter = max_iter
        f.M_divergence = M
        FP_params, orbit = store_orbit(f, ref_point, order, max_iter, M, xr_threshold)
        f.calc_std_div(calc_name="pert", subset=None, max_iter=max_iter,
                       M_divergence=M, epsilon_stationnary=eps_stat,
                       BLA_eps=bla_eps, interior_detect=interior,
                       calc_dzndc=True, calc_orbit=backshift > 0, backshift=backshift)
        c_pix, Z, U, sr, si, cia = run_tile(f, "pert")
        (_, _, _, Zn_path, dZndc_path, dZndz_path, has_xr, ref_index_xr,
         ref_xr, ref_div_iter, ref_order, drift_xr, dx_xr, _proj, lin_mat,
         lin_scale_xr, kc, M_bla, r_bla, bla_len, stages_bla, _m, _i) = cia
        xr = f.xr_detect_activated
        res = dict(
            pix=c_pix, Z=Z, U=U, stop_reason=sr, stop_iter=si, backshift=backshift,
            Zn=Zn_path, ref_div_iter=ref_div_iter, ref_order=ref_order,
            xr_mode=int(xr), lin_mat=lin_mat,
            dx_m=np.asarray(dx_xr._mantissa)[0],
            dx_e=np.asarray(dx_xr._exp)[0],
            drift_m=np.asarray(drift_xr._mantissa)[0],
            drift_e=np.asarray(drift_xr._exp)[0],
            kc_m=np.asarray(kc._mantissa)[0], kc_e=np.asarray(kc._exp)[0],
            max_iter=max_iter, M=M, eps_stat=eps_stat, bla_eps=bla_eps,
            interior=int(interior), codes=np.array(f.codes[0]),
            M_bla=M_bla, r_bla=r_bla, stages_bla=stages_bla,
            xr_idx=ref_index_xr,
        )
        m, e = xr_arrays(ref_xr)
        res["xr_m"], res["xr_e"] = m, e
        if xr:
            res["dZndc_m"], res["dZndc_e"] = xr_arrays(dZndc_path)
            if interior:
                res["dZndz_m"], res["dZndz_e"] = xr_arrays(dZndz_path)
        else:
            res["dZndc"] = dZndc_path
            if interior:
                res["dZndz"] = dZndz_path
        np.savez_compressed(out, **res)


def golden_std_mn(out):
    """Standard power-n Mandelbrot (models/mandelbrot_Mn.py:20-176), n = 3, 4."""
    res = {}
    for nexp in (3, 4):
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Mandelbrot_N(d, exponent=nexp)
            f.zoom(x=0., y=0., dx=3., nx=40, xy_ratio=1., theta_deg=0.)
            f.calc_std_div(calc_name="std", subset=None, max_iter=300,
                           M_divergence=1000., epsilon_stationnary=0.01)
            c_pix, Z, U, sr, si, cia = run_tile(f, "std")
            res[f"pix_{nexp}"] = c_pix
            res[f"Z_{nexp}"] = Z
            res[f"stop_reason_{nexp}"] = sr
            res[f"stop_iter_{nexp}"] = si
            res["lin_mat"] = f.lin_mat
    np.savez_compressed(out, center=np.array([0., 0.]), dx=3., max_iter=300, M=1000.,
                        eps=0.01, **res)


def golden_perturb_mn(out, *, nexp, x, y, dx, nx, precision, order, max_iter,
                      interior, bla_eps=1e-6, eps_stat=1e-3, M=1000., ref_shift=0j,
                      backshift=0):
    """Perturbation power-n Mandelbrot (models/mandelbrot_Mn.py:387-740)."""
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Perturbation_mandelbrot_N(d, exponent=nexp)
        f.zoom(precision=precision, x=x, y=y, dx=dx, nx=nx, xy_ratio=1.,
               theta_deg=0., projection=fs.projection.Cartesian())
        ref_point = mpmath.mpc(x, y) + mpmath.mpc(ref_shift) * mpmath.mpf(dx)
        f.max_iter = max_iter
        f.M_divergence = M
        store_orbit_n(f, nexp, ref_point, order, max_iter, M)
        f.calc_std_div(calc_name="pert", subset=None, max_iter=max_iter,
                       M_divergence=M, epsilon_stationnary=eps_stat,
                       BLA_eps=bla_eps, interior_detect=interior,
                       calc_dzndc=True, calc_orbit=backshift > 0, backshift=backshift)
        c_pix, Z, U, sr, si, cia = run_tile(f, "pert")
        (_, _, _, Zn_path, dZndc_path, dZndz_path, has_xr, ref_index_xr,
         ref_xr, ref_div_iter, ref_order, drift_xr, dx_xr, _proj, lin_mat,
         lin_scale_xr, kc, M_bla, r_bla, bla_len, stages_bla, _m, _i) = cia
        xr = f.xr_detect_activated
        res = dict(
            pix=c_pix, Z=Z, U=U, stop_reason=sr, stop_iter=si, nexp=nexp,
            backshift=backshift,
            Zn=Zn_path, ref_div_iter=ref_div_iter, ref_order=ref_order,
            xr_mode=int(xr), lin_mat=lin_mat,
            dx_m=np.asarray(dx_xr._mantissa)[0],
            dx_e=np.asarray(dx_xr._exp)[0],
            drift_m=np.asarray(drift_xr._mantissa)[0],
            drift_e=np.asarray(drift_xr._exp)[0],
            kc_m=np.asarray(kc._mantissa)[0], kc_e=np.asarray(kc._exp)[0],
            max_iter=max_iter, M=M, eps_stat=eps_stat, bla_eps=bla_eps,
            interior=int(interior), codes=np.array(f.codes[0]),
            M_bla=M_bla, r_bla=r_bla, stages_bla=stages_bla,
            xr_idx=ref_index_xr,
        )
        m, e = xr_arrays(ref_xr)
        res["xr_m"], res["xr_e"] = m, e
        if xr:
            res["dZndc_m"], res["dZndc_e"] = xr_arrays(dZndc_path)
            if interior:
                res["dZndz_m"], res["dZndz_e"] = xr_arrays(dZndz_path)
        else:
            res["dZndc"] = dZndc_path
            if interior:
                res["dZndz"] = dZndz_path
        np.savez_compressed(out, **res)


def golden_perturb_bs(out, *, x, y, dx, nx, precision, max_iter, flavor,
                      bla_eps=1e-6, M=1000., backshift=0, projection=None):
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Perturbation_burning_ship(d, flavor=flavor)
        f.zoom(precision=precision, x=x, y=y, dx=dx, nx=nx, xy_ratio=1.,
               theta_deg=0., projection=projection or fs.projection.Cartesian())
        ref_point = mpmath.mpc(x, y)
        f.max_iter = max_iter
        f.M_divergence = M
        flavor_int = fs.models.burning_ship.get_flavor_int(flavor)
        # BS orbit: perturbation_nonholomorphic_FP_loop (FP_loop.pyx:1828-1979)
        ref_orbit_len = max_iter + 1
        orbit = np.zeros(ref_orbit_len, dtype=np.complex128)
        xn, yn = mpmath.mpf(0), mpmath.mpf(0)
        a, b = ref_point.real, ref_point.imag
        it = f.xnyn_iterate
        i = 0
        # the side table of FP_loop.pyx:1828-1979: iterations where |X| or |Y|
        # is below xrange_zoom_level, when the Xrange branch is active
        xr_dict = {}
        need_xr = f.xr_detect_activated
        for i in range(1, ref_orbit_len):
            xn, yn = it(xn, yn, a, b)
            orbit[i] = complex(float(xn), float(yn))
            if np.hypot(orbit[i].real, orbit[i].imag) > 2 * M:
                break
            if need_xr and (abs(xn) < fs.settings.xrange_zoom_level
                            or abs(yn) < fs.settings.xrange_zoom_level):
                xr_dict[i] = (fsx.mpf_to_Xrange(xn).ravel(), fsx.mpf_to_Xrange(yn).ravel())
        if i == ref_orbit_len - 1 and np.hypot(orbit[i].real, orbit[i].imag) <= 2 * M:
            i += 1
        init_kwargs = f.init_kwargs
        del init_kwargs["directory"]
        FP_params = {"ref_point": ref_point, "dps": mpmath.mp.dps,
                     "order": None, "max_iter": max_iter, "FP_code": f.FP_code,
                     "partials": {}, "xr": xr_dict, "div_iter": i,
                     "init_kwargs": init_kwargs, "ref_orbit_len": ref_orbit_len}
        f.save_ref_point(FP_params, orbit)
        f.calc_std_div(calc_name="pert", subset=None, max_iter=max_iter,
                       M_divergence=M, BLA_eps=bla_eps, calc_hessian=True,
                       calc_orbit=backshift > 0, backshift=backshift)
        c_pix, Z, U, sr, si, cia = run_tile(f, "pert")
        (_, _, _, Zn_path, dXa, dXb, dYa, dYb, has_xr, ref_index_xr, refx_xr,
         refy_xr, ref_div_iter, ref_order, driftx_xr, drifty_xr, dx_xr, _p,
         lin_mat, lin_scale_xr, kc, M_bla, r_bla, bla_len, stages_bla, _m,
         _i) = cia
        xr = bool(f.xr_detect_activated)
        extra = {"xr_mode": int(xr)}
        if xr:
            extra["xr_idx"] = ref_index_xr
            extra["xr_xm"], extra["xr_xe"] = xr_arrays(refx_xr)
            extra["xr_ym"], extra["xr_ye"] = xr_arrays(refy_xr)
            for k, pth in (("dXa", dXa), ("dXb", dXb), ("dYa", dYa), ("dYb", dYb)):
                extra[k + "_m"], extra[k + "_e"] = xr_arrays(pth)
            dXa = dXb = dYa = dYb = np.zeros(1)
        np.savez_compressed(
            out, pix=c_pix, Z=Z, U=U, stop_reason=sr, stop_iter=si,
            Zn=Zn_path, dXa=dXa, dXb=dXb, dYa=dYa, dYb=dYb,
            ref_div_iter=ref_div_iter, ref_order=ref_order,
            lin_mat=lin_mat, flavor=flavor_int,
            dx_m=np.asarray(dx_xr._mantissa)[0], dx_e=np.asarray(dx_xr._exp)[0],
            driftx_m=np.asarray(driftx_xr._mantissa)[0],
            driftx_e=np.asarray(driftx_xr._exp)[0],
            drifty_m=np.asarray(drifty_xr._mantissa)[0],
            drifty_e=np.asarray(drifty_xr._exp)[0],
            kc_m=np.asarray(kc._mantissa)[0], kc_e=np.asarray(kc._exp)[0],
            max_iter=max_iter, M=M, bla_eps=bla_eps, backshift=backshift,
            M_bla=M_bla, r_bla=r_bla, stages_bla=stages_bla, **extra)


def golden_std_opts(out):
    """Standard loops with the optional outputs: d2zndc2 (Milnor) and the
    orbit point n - backshift (calc_orbit) for the power-2 and power-3
    models, the orbit point for Burning Ship flavors 1 and 4."""
    res = {}
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Mandelbrot(d)
        f.zoom(x=-0.5, y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=400, M_divergence=1000.,
                       epsilon_stationnary=0.01, calc_d2zndc2=True, calc_orbit=True,
                       backshift=3)
        c_pix, Z, U, sr, si, cia = run_tile(f, "std")
        res.update(pix_m2=c_pix, Z_m2=Z, stop_reason_m2=sr, stop_iter_m2=si,
                   codes_m2=np.array(f.codes[0]), lin_mat=f.lin_mat)
    for nexp in (2, 3):
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Mandelbrot_N(d, exponent=nexp)
            f.zoom(x=0., y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
            f.calc_std_div(calc_name="std", subset=None, max_iter=300, M_divergence=1000.,
                           epsilon_stationnary=0.01, calc_d2zndc2=True, calc_orbit=True,
                           backshift=4)
            c_pix, Z, U, sr, si, cia = run_tile(f, "std")
            res.update({f"pix_mn{nexp}": c_pix, f"Z_mn{nexp}": Z,
                        f"stop_reason_mn{nexp}": sr, f"stop_iter_mn{nexp}": si})
    for flavor_int, flavor in ((1, "Burning ship"), (4, "Celtic")):
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Burning_ship(d, flavor=flavor)
            f.zoom(x=-0.5, y=-0.5, dx=3.5, nx=24, xy_ratio=1., theta_deg=0.)
            f.calc_std_div(calc_name="std", subset=None, max_iter=200, M_divergence=1000.,
                           calc_orbit=True, backshift=3)
            c_pix, Z, U, sr, si, cia = run_tile(f, "std")
            res.update({f"pix_bs{flavor_int}": c_pix, f"Z_bs{flavor_int}": Z,
                        f"stop_reason_bs{flavor_int}": sr, f"stop_iter_bs{flavor_int}": si})
    np.savez_compressed(out, **res)


def _run_postprocs(f, calc_name, c_pix, Z, U, sr, si, posts):
    """Fractal.postproc (core.py:2736-2778) on one chunk: the reference's
    Postproc_batch evaluated post by post, each updating the shared context;
    returns the float64 values (before the float32 cast of post_array)."""
    batch = fs.postproc.Postproc_batch(f, calc_name)
    for name, pp in posts:
        batch.add_postproc(name, pp)
    chunk = (0, f.nx, 0, f.ny)
    codes = f._calc_data[calc_name]["state"].codes
    complex_dic, int_dic, termination_dic = f.codes_mapping(*codes)
    batch.set_chunk_data(chunk, None, c_pix, Z, U, sr, si, complex_dic, int_dic,
                         termination_dic)
    out = {}
    for name, pp in batch.posts.items():
        val, upd = pp[chunk]
        out[name] = np.asarray(val, dtype=np.float64)
        batch.update_context(chunk, upd)
    return out


def golden_postproc(out):
    """Continuous iteration, field lines (zn_orbit, backshift 3) and DEM
    normals (potential and Milnor) from the reference's postproc classes, for
    the power-2, power-3 and Burning Ship (flavor 1) standard loops."""
    res = {}
    fl_kw = dict(n_iter=5, swirl=0.7, endpoint_k=0.5)
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Mandelbrot(d)
        f.zoom(x=-0.5, y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=400, M_divergence=1000.,
                       epsilon_stationnary=0.01, calc_d2zndc2=True, calc_orbit=True,
                       backshift=3)
        c_pix, Z, U, sr, si, cia = run_tile(f, "std")
        r = _run_postprocs(f, "std", c_pix, Z, U, sr, si, [
            ("cont", fs.postproc.Continuous_iter_pp()),
            ("fl", fs.postproc.Fieldlines_pp(**fl_kw)),
            ("dn", fs.postproc.DEM_normal_pp(kind="potential")),
            ("mil", fs.postproc.DEM_normal_pp(kind="Milnor"))])
        res.update({f"m2_{k}": v for k, v in r.items()})
        res.update(m2_pix=c_pix, m2_Z=Z, m2_si=si, m2_cpt=f.get_std_cpt(c_pix))
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Mandelbrot_N(d, exponent=3)
        f.zoom(x=0., y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=300, M_divergence=1000.,
                       epsilon_stationnary=0.01, calc_orbit=True, backshift=3)
        c_pix, Z, U, sr, si, cia = run_tile(f, "std")
        r = _run_postprocs(f, "std", c_pix, Z, U, sr, si, [
            ("cont", fs.postproc.Continuous_iter_pp()),
            ("fl", fs.postproc.Fieldlines_pp(**fl_kw)),
            ("dn", fs.postproc.DEM_normal_pp(kind="potential"))])
        res.update({f"mn3_{k}": v for k, v in r.items()})
        res.update(mn3_pix=c_pix, mn3_Z=Z, mn3_si=si, mn3_cpt=f.get_std_cpt(c_pix))
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Burning_ship(d, flavor="Burning ship")
        f.zoom(x=-0.5, y=-0.5, dx=3.5, nx=32, xy_ratio=1., theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=300, M_divergence=1000.,
                       calc_orbit=True, backshift=3)
        c_pix, Z, U, sr, si, cia = run_tile(f, "std")
        r = _run_postprocs(f, "std", c_pix, Z, U, sr, si, [
            ("cont", fs.postproc.Continuous_iter_pp()),
            ("fl", fs.postproc.Fieldlines_pp(**fl_kw)),
            ("dn", fs.postproc.DEM_normal_pp(kind="potential"))])
        res.update({f"bs1_{k}": v for k, v in r.items()})
        res.update(bs1_pix=c_pix, bs1_Z=Z, bs1_si=si, bs1_cpt=f.get_std_cpt(c_pix))
    res.update(fl_n_iter=5, fl_swirl=0.7, fl_endpoint_k=0.5, backshift=3)
    np.savez_compressed(out, **res)


def golden_pixel_grids(out):
    """Fractal.chunk_pixel_pos (core.py:1767-1830) with supersampling and
    jitter, whole image and one inner chunk, xy_ratio 1.5."""
    res = {}
    with tempfile.TemporaryDirectory() as d:
        f = fsm.Mandelbrot(d)
        f.zoom(x=-0.5, y=0., dx=3., nx=40, xy_ratio=1.5, theta_deg=0.)
        # float_type follows the calculation's complex_type
        f.calc_std_div(calc_name="std", subset=None, max_iter=10, M_divergence=1000.,
                       epsilon_stationnary=0.01)
        f._calc_data["std"]["state"].complex_type = np.complex128
        f.complex_type = np.complex128
        cases = {"plain": (False, None), "ss3": (False, 3), "jit": (0.7, None),
                 "ss2_jit": (1.0, 2)}
        for chunk_name, cs in (("full", (0, f.nx, 0, f.ny)), ("inner", (8, 24, 4, 20))):
            for name, (jit, ssg) in cases.items():
                res[f"{chunk_name}_{name}"] = f.chunk_pixel_pos(cs, jit, ssg)
        res["nx"], res["ny"] = f.nx, f.ny
    np.savez_compressed(out, **res)


def golden_expmap(out):
    """Standard power-2 loop under an Expmap projection (horizontal and
    vertical orientations): the projected pixel c = center + dx lin
    exp(h_moy + ht pix) (core.py:3161-3194, projection.py:363-373)."""
    res = {}
    for name, orient in (("h", "horizontal"), ("v", "vertical")):
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Mandelbrot(d)
            proj = fs.projection.Expmap(hmin=0., hmax=4., rotates_df=True, orientation=orient)
            f.zoom(x=-0.743643887037151, y=0.13182590420533, dx=1e-4, nx=24, xy_ratio=1.,
                   theta_deg=15., projection=proj)
            f.calc_std_div(calc_name="std", subset=None, max_iter=2000, M_divergence=1000.,
                           epsilon_stationnary=0.01)
            c_pix, Z, U, sr, si, cia = run_tile(f, "std")
            res.update({f"{name}_pix": c_pix, f"{name}_Z": Z, f"{name}_si": si,
                        f"{name}_sr": sr, f"{name}_lin_mat": f.lin_mat,
                        f"{name}_nx": f.nx, f"{name}_ny": f.ny,
                        f"{name}_xy_ratio": f.xy_ratio,
                        f"{name}_c": f.get_std_cpt(c_pix)})
    np.savez_compressed(out, **res)


def expmap_cases():
    # the calculation fingerprint pickles the projection, whose mapping
    # functions are numba dispatchers in the reference and plain closures
    # here; the fixtures need no fingerprint
    fs.core.Fractal.save_fingerprint = lambda self, calc_name, fingerprint: None
    mpmath.mp.dps = 50
    golden_expmap(os.path.join(HERE, "std_expmap.npz"))
    print("std_expmap done", flush=True)
    mpmath.mp.dps = 30
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_expmap.npz"),
        x="-0.743643887037151", y="0.131825904205330", dx="2.e-9", nx=12,
        precision=30, order=None, max_iter=6000, interior=False,
        projection=fs.projection.Expmap(hmin=0., hmax=5., rotates_df=True,
                                        orientation="horizontal"))
    print("pert_m2_expmap done", flush=True)
    golden_perturb_bs(
        os.path.join(HERE, "pert_bs_expmap.npz"),
        x="-1.773934837092732", y="-0.00025062656641604286", dx="4.e-7",
        nx=10, precision=30, max_iter=5000, flavor="Burning ship",
        projection=fs.projection.Expmap(hmin=0., hmax=3., rotates_df=True,
                                        orientation="vertical"))
    print("pert_bs_expmap done", flush=True)


def opts_cases():
    """The calc_orbit / calc_d2zndc2 options of the standard and perturbation
    loops."""
    mpmath.mp.dps = 50
    golden_std_opts(os.path.join(HERE, "std_opts.npz"))
    print("std_opts done", flush=True)
    mpmath.mp.dps = 30
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_orbit.npz"),
        x="-0.743643887037151", y="0.131825904205330", dx="2.e-9", nx=12,
        precision=30, order=None, max_iter=6000, interior=False, backshift=5)
    print("pert_m2_orbit done", flush=True)
    mpmath.mp.dps = 340
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_xr_orbit.npz"),
        x="-0.743643887037158704752191506114774e0",
        y="0.131825904205311970493132056385139", dx="3.e-304", nx=4,
        precision=340, order=None, max_iter=5000, interior=False,
        ref_shift=0.31 - 0.27j, x_offset="1e-14", backshift=7)
    print("pert_m2_xr_orbit done", flush=True)
    mpmath.mp.dps = 60
    c3 = mp_nucleus_n(3, 10, 60, mpmath.mpc("0.64287667998175895118", "0.25145447487965245909"))
    mpmath.mp.dps = 30
    golden_perturb_mn(
        os.path.join(HERE, "pert_mn3_orbit.npz"), nexp=3,
        x=str(c3.real + mpmath.mpf("0.004")), y=str(c3.imag), dx="2.e-3", nx=12,
        precision=30, order=None, max_iter=3000, interior=False, ref_shift=0.21 - 0.13j,
        backshift=4)
    print("pert_mn3_orbit done", flush=True)
    golden_perturb_bs(
        os.path.join(HERE, "pert_bs_orbit.npz"),
        x="-1.773934837092732", y="-0.00025062656641604286", dx="4.e-6",
        nx=10, precision=30, max_iter=5000, flavor="Burning ship", backshift=6)
    print("pert_bs_orbit done", flush=True)


def golden_xrange(out, seed=100, n=400):
    """Xrange arithmetic through the reference's host class (numpy_utils/xrange.py),
    operand generator in the spirit of tests/test_numba_xr.py (seeds 100/800,
    binary exponents up to +-200)."""
    rg = np.random.default_rng(seed)
    am = (rg.random(n) - .5) + 1j * (rg.random(n) - .5)
    bm = (rg.random(n) - .5) + 1j * (rg.random(n) - .5)
    ae = rg.integers(-200, 200, n).astype(np.int32)
    be = rg.integers(-200, 200, n).astype(np.int32)
    # a few exact zeros and equal exponents (edge cases of _coexp_ufunc)
    am[:5] = 0.
    be[5:10] = ae[5:10]
    A = fsx.Xrange_array(am, ae)
    B = fsx.Xrange_array(bm, be)
    S = A + B
    P = A * B
    Q = A.abs2()
    res = dict(am=am, ae=ae, bm=bm, be=be,
               add=S.to_standard() if False else np.zeros(0),
               add_m=np.asarray(S._mantissa), add_e=np.asarray(S._exp),
               mul_m=np.asarray(P._mantissa), mul_e=np.asarray(P._exp),
               abs2_m=np.asarray(Q._mantissa), abs2_e=np.asarray(Q._exp))
    # to_standard on values that stay in the double range
    sm = (rg.random(n) - .5) + 1j * (rg.random(n) - .5)
    se = rg.integers(-1000, 1000, n).astype(np.int32)
    res["std_m"], res["std_e"] = sm, se
    res["std_out"] = fsx.Xrange_array(sm, se).to_standard()
    np.savez_compressed(out, **res)


def golden_flake_orbit(out):
    """The reference's stored FP64 orbit of the 'flake' point
    (tests/REFERENCE_DATA/perturb_REF/flake/dev_pt0.ref), first period."""
    import pickle
    path = os.path.join(os.path.dirname(REF_SRC), "tests", "REFERENCE_DATA",
                        "perturb_REF", "flake", "dev_pt0.ref")
    with open(path, "rb") as f:
        params = pickle.load(f)
        orbit = pickle.load(f)[:, 0]
    rp = params["ref_point"]
    prec = max(rp.real._mpf_[1].bit_length(), rp.imag._mpf_[1].bit_length())
    order = int(params["order"])
    with mpmath.workprec(prec + 64):
        x = mpmath.nstr(rp.real, int(prec / 3.3) + 20)
        y = mpmath.nstr(rp.imag, int(prec / 3.3) + 20)
    np.savez_compressed(out, x=x, y=y, prec=prec, order=order, orbit=orbit[:order + 1])


def golden_newton_kat(out):
    """Newton known answer of the reference's tests/test_FP_loop.py (test_newton):
    the start point and expected nucleus digits, read from the test source."""
    import ast
    path = os.path.join(os.path.dirname(REF_SRC), "tests", "test_FP_loop.py")
    tree = ast.parse(open(path).read())
    found = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and isinstance(node.value, ast.Dict):
            keys = [k.value for k in node.value.keys if isinstance(k, ast.Constant)]
            if "x_nucleus" in keys:
                found = {k.value: v.value for k, v in zip(node.value.keys, node.value.values)
                         if isinstance(v, ast.Constant)}
    np.savez_compressed(out, x_start=found["x_start"], y_start=found["y_start"],
                        order=found["order"], x_nucleus=found["x_nucleus"],
                        y_nucleus=found["y_nucleus"])


def main():
    golden_flake_orbit(os.path.join(HERE, "flake_orbit.npz"))
    golden_newton_kat(os.path.join(HERE, "newton_4252.npz"))
    print("host orbit fixtures done", flush=True)
    mpmath.mp.dps = 50
    golden_xrange(os.path.join(HERE, "xrange_ops.npz"))
    print("xrange done", flush=True)
    golden_std_m2(os.path.join(HERE, "std_m2.npz"))
    print("std_m2 done", flush=True)
    golden_std_bs(os.path.join(HERE, "std_bs.npz"))
    print("std_bs done", flush=True)

    # Perturbation M2, standard (FP64) branch, non-cycle reference at the centre
    mpmath.mp.dps = 30
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_fp64.npz"),
        x="-0.743643887037151", y="0.131825904205330", dx="2.e-9", nx=20,
        precision=30, order=None, max_iter=6000, interior=False)
    print("pert_m2_fp64 done", flush=True)

    # Perturbation M2, cycle reference (period-p nucleus), interior detection
    p = 29
    dps = 60
    mpmath.mp.dps = dps
    c = mp_nucleus(p, dps)
    size = mpmath.mpf(1) / (p ** 2 * 40)
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_cycle.npz"),
        x=str(c.real), y=str(c.imag), dx=str(size * 2), nx=16,
        precision=dps, order=p, max_iter=3000, interior=True)
    print("pert_m2_cycle done", flush=True)

    # Perturbation M2, Xrange branch (dx < 1e-300), cycle reference
    dps = 340
    mpmath.mp.dps = dps
    c = mp_nucleus(p, dps)
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_xr.npz"),
        x=str(c.real), y=str(c.imag), dx="1.e-305", nx=4,
        precision=dps, order=p, max_iter=600, interior=True)
    print("pert_m2_xr done", flush=True)

    # Perturbation M2, Xrange branch, escaping non-cycle reference that is
    # off the image centre (drift), dx < 1e-300
    mpmath.mp.dps = 340
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_xr_div.npz"),
        x="-0.743643887037158704752191506114774e0",
        y="0.131825904205311970493132056385139", dx="3.e-304", nx=5,
        precision=340, order=None, max_iter=5000, interior=False,
        ref_shift=0.31 - 0.27j, x_offset="1e-14")
    print("pert_m2_xr_div done", flush=True)

    # Power-n Mandelbrot, standard loop (n = 3, 4)
    mpmath.mp.dps = 50
    golden_std_mn(os.path.join(HERE, "std_mn.npz"))
    print("std_mn done", flush=True)
    mn_cases()

    # Perturbation Burning Ship (flavors 1 and 4), standard branch, around a
    # point whose orbit escapes after ~2200 iterations
    mpmath.mp.dps = 30
    for fl, flav in ((1, "Burning ship"), (4, "Celtic")):
        golden_perturb_bs(
            os.path.join(HERE, f"pert_bs_{fl}.npz"),
            x="-1.773934837092732", y="-0.00025062656641604286", dx="4.e-6",
            nx=14, precision=30, max_iter=5000, flavor=flav)
        print(f"pert_bs_{fl} done", flush=True)


def mn_cases():
    """Perturbation power-n Mandelbrot: n = 3 around a period-10 nucleus with
    interior detection (standard branch); n = 3 with an off-centre escaping
    reference (rebases); n = 4 in the Xrange branch (dx < 1e-300)."""
    # nuclei found by an order-1 ball (radius 1e-3) around seeded points and
    # Newton on that period (periods 10: the reference's BLA lookup needs an
    # orbit of at least 9 points, perturbation.py:2138-2149)
    dps = 60
    mpmath.mp.dps = dps
    c3 = mp_nucleus_n(3, 10, dps, mpmath.mpc("0.64287667998175895118", "0.25145447487965245909"))
    golden_perturb_mn(
        os.path.join(HERE, "pert_mn3_cycle.npz"), nexp=3,
        x=str(c3.real), y=str(c3.imag), dx="2.5e-4", nx=16,
        precision=dps, order=10, max_iter=3000, interior=True)
    print("pert_mn3_cycle done", flush=True)
    mpmath.mp.dps = 30
    golden_perturb_mn(
        os.path.join(HERE, "pert_mn3_div.npz"), nexp=3,
        x=str(c3.real + mpmath.mpf("0.004")), y=str(c3.imag), dx="2.e-3", nx=16,
        precision=30, order=None, max_iter=3000, interior=False, ref_shift=0.21 - 0.13j)
    print("pert_mn3_div done", flush=True)
    dps = 340
    mpmath.mp.dps = dps
    c4 = mp_nucleus_n(4, 10, dps, mpmath.mpc("-0.51534888699245770184", "0.46481172994907691405"))
    golden_perturb_mn(
        os.path.join(HERE, "pert_mn4_xr.npz"), nexp=4,
        x=str(c4.real), y=str(c4.imag), dx="1.e-305", nx=4,
        precision=dps, order=10, max_iter=600, interior=True)
    print("pert_mn4_xr done", flush=True)


def p2562_cases(nx_edge=16, nx_edge_xr=4):
    """The period-2562 nucleus at 400 digits of the 2048 x 2048, dx = 1e-300
    workload (seed 2), read from fractalshades_gb300/data/nuclei.json where
    the Newton + ball-method search stored it; max_iter 2e5, BLA eps 1e-6,
    escape radius 1e3, dzndc.
      * p2562_1e300: the workload's own width, the Xrange branch, every
        pixel interior (78 periods, BLA stages up to 11);
      * p2562_edge: width 1.6e-9, about four times the nucleus size estimate
        (3.9e-10): the minibrot and its surroundings, about half the pixels
        escaping after 2.6e3 .. 2e5 iterations; FP64 branch;
      * p2562_edge_xr: the same view on the Xrange branch
        (settings.xrange_zoom_level raised to 1e-5), on a coarser grid (the
        Xrange branch runs ~50x slower as plain Python).
    About an hour of CPU in all (16 + 256 + 16 pixels)."""
    import json
    dps = 400
    mpmath.mp.dps = dps
    nuc = os.path.join(os.path.dirname(os.path.dirname(HERE)), "fractalshades_gb300", "data",
                       "nuclei.json")
    with open(nuc) as fh:
        rec = json.load(fh)["2562:400"]
    x, y = rec[0], rec[1]
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_p2562_1e300.npz"), x=x, y=y, dx="1.e-300", nx=4,
        precision=dps, order=2562, max_iter=200000, interior=False)
    print("pert_m2_p2562_1e300 done", flush=True)
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_p2562_edge.npz"), x=x, y=y, dx="1.6e-9", nx=nx_edge,
        precision=dps, order=2562, max_iter=200000, interior=False)
    print("pert_m2_p2562_edge done", flush=True)
    golden_perturb_m2(
        os.path.join(HERE, "pert_m2_p2562_edge_xr.npz"), x=x, y=y, dx="1.6e-9", nx=nx_edge_xr,
        precision=dps, order=2562, max_iter=200000, interior=False, xr_zoom_level=1e-5)
    print("pert_m2_p2562_edge_xr done", flush=True)


def bs_flavor_cases():
    """Perturbation Burning Ship flavors 2, 3 and 5 (Perpendicular burning
    ship, Shark fin, Buffalo; burning_ship.py:535-859), and flavor 4 (Celtic)
    on a second view, FP64 branch: each centred on a point of its own set's
    boundary whose orbit escapes after ~3000 iterations (found with the
    standard loop on a grid), width 1e-5, so that the reference diverges and
    escaping and non-escaping pixels mix."""
    mpmath.mp.dps = 30
    for fl, flav, x, y, name in (
            (2, "Perpendicular burning ship", "-0.5710063401785717", "-0.6660741479166669",
             "pert_bs_2"),
            (3, "Shark fin", "-0.6922635670582709", "-0.3510271929824563", "pert_bs_3"),
            (4, "Celtic", "-0.7584971274906015", "-0.8352377380482457", "pert_bs_4e"),
            (5, "Buffalo", "-1.5394062147086462", "0.2671241854166664", "pert_bs_5")):
        golden_perturb_bs(
            os.path.join(HERE, name + ".npz"), x=x, y=y, dx="1.e-5",
            nx=14, precision=30, max_iter=5000, flavor=flav)
        print(name + " done", flush=True)


def bs_xr_cases():
    """Perturbation Burning Ship on the Xrange branch (dx = 1e-305 <
    xrange_zoom_level): flavor 1 at the centre of pert_bs_1 and flavor 5 at
    that of pert_bs_5, whose references diverge after ~2200 and ~2900
    iterations; the deltas start below the double range."""
    mpmath.mp.dps = 340
    for fl, flav, x, y, name in (
            (1, "Burning ship", "-1.773934837092732", "-0.00025062656641604286", "pert_bs_xr_1"),
            (5, "Buffalo", "-1.5394062147086462", "0.2671241854166664", "pert_bs_xr_5")):
        golden_perturb_bs(
            os.path.join(HERE, name + ".npz"), x=x, y=y, dx="1.e-305",
            nx=5, precision=340, max_iter=5000, flavor=flav)
        print(name + " done", flush=True)


def bs_xr_flavor_cases():
    """The Xrange branch (dx = 1e-305) for flavors 2, 3 and 4 (Perpendicular
    burning ship, Shark fin, Celtic) at the centres of their FP64-branch
    cases, whose references diverge after ~3000 iterations."""
    mpmath.mp.dps = 340
    for flav, x, y, name in (
            ("Perpendicular burning ship", "-0.5710063401785717", "-0.6660741479166669",
             "pert_bs_xr_2"),
            ("Shark fin", "-0.6922635670582709", "-0.3510271929824563", "pert_bs_xr_3"),
            ("Celtic", "-0.7584971274906015", "-0.8352377380482457", "pert_bs_xr_4")):
        golden_perturb_bs(
            os.path.join(HERE, name + ".npz"), x=x, y=y, dx="1.e-305",
            nx=4, precision=340, max_iter=5000, flavor=flav)
        print(name + " done", flush=True)


def bs_xr_axis_case():
    """Burning Ship on the Xrange branch around a point of the real axis
    (-1.7548776662466927, the real map's superstable period 3): Y_n = 0 on
    the whole orbit, so every iteration enters the side table of
    FP_loop.pyx:1828-1979 and the loop reads its Xrange values; no BLA step is
    valid there (r = eps min(|X|, |Y|) = 0)."""
    mpmath.mp.dps = 340
    golden_perturb_bs(
        os.path.join(HERE, "pert_bs_xr_axis.npz"), x="-1.7548776662466927", y="0",
        dx="1.e-305", nx=4, precision=340, max_iter=1500, flavor="Burning ship")
    print("pert_bs_xr_axis done", flush=True)


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "bs_xr":
        bs_xr_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "bs_xr_axis":
        bs_xr_axis_case()
    elif len(sys.argv) > 2 and sys.argv[2] == "bs_xr_flavors":
        bs_xr_flavor_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "p2562":
        p2562_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "bs_flavors":
        bs_flavor_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "opts":
        opts_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "expmap":
        expmap_cases()
    elif len(sys.argv) > 2 and sys.argv[2] == "postproc":
        mpmath.mp.dps = 50
        golden_postproc(os.path.join(HERE, "postproc.npz"))
        golden_pixel_grids(os.path.join(HERE, "pixel_grids.npz"))
    elif len(sys.argv) > 2 and sys.argv[2] == "mn":
        mpmath.mp.dps = 50
        golden_std_mn(os.path.join(HERE, "std_mn.npz"))
        mn_cases()
    else:
        main()
