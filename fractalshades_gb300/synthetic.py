"""
Seeded synthetic deep-zoom workloads.

The deep-zoom configurations are centred on nuclei of period-p hyperbolic
components: p is drawn from a seeded generator, the start point sits on the
root of the 1/p bulb of the main cardioid, c0 = e^{i t}/2 - e^{2 i t}/4 with
t = 2 pi / p, moved outward along the cardioid normal by pi / p^3 (the
asymptotic distance between the root and the nucleus of that bulb), and is
refined by the Newton search of mpmath_utils.FP_loop (division by the
divisor periods); the ball method confirms the period.

``prepare_m2`` returns everything a perturbation launch needs: the FP64
orbit with its Xrange side table, kc, and the pixel axes of the image.
"""
import dataclasses

import mpmath
import numpy as np

from .mpmath_utils import FP_loop as fsFP
from .numpy_utils import xrange as fsx
from . import settings


def nucleus_start(p, dps):
    with mpmath.workdps(dps):
        th = 2 * mpmath.pi / p
        c0 = mpmath.expj(th) / 2 - mpmath.expj(2 * th) / 4
        tangent = 1j * mpmath.expj(th) / 2 - 1j * mpmath.expj(2 * th) / 2
        normal = -1j * tangent / abs(tangent)
        return c0 + normal * (mpmath.pi / mpmath.mpf(p) ** 3)


def find_nucleus(p, dps):
    """Nucleus of period p near the root of the 1/p bulb, at dps digits."""
    with mpmath.workdps(dps):
        prec = mpmath.mp.prec
        c0 = nucleus_start(p, dps)
        ok, c = fsFP.perturbation_mandelbrot_find_nucleus(
            str(c0.real), str(c0.imag), prec, p, 80, str(mpmath.mpf(2) ** (-prec)),
            str(mpmath.mpf(10) ** (-(dps // 2))))
        if not ok:
            raise RuntimeError(f"Newton did not converge for period {p}")
        order = fsFP.perturbation_mandelbrot_ball_method(
            str(c.real), str(c.imag), prec, str(mpmath.mpf(10) ** (-(dps // 2))), 10 * p, 1e5)
        if order != p:
            raise RuntimeError(f"ball method found period {order}, expected {p}")
        return c


@dataclasses.dataclass
class M2Workload:
    p: int
    dps: int
    center: object          # mpmath mpc
    dx: object              # mpmath mpf
    nx: int
    ny: int
    max_iter: int
    M: float
    Zn: np.ndarray          # complex128 [len]
    div_iter: int
    order: int
    xr_idx: np.ndarray
    xr_m: np.ndarray
    xr_e: np.ndarray
    xr_mode: bool
    dx_m: float
    dx_e: int
    drift_m: complex
    drift_e: int
    kc: float
    xs: np.ndarray
    ys: np.ndarray


def image_axes(nx, ny, xy_ratio=1.0, chunk=None):
    """Per-column / per-row screen coordinates of the reference's tiling
    (core.py:1767-1830), tile by tile."""
    chunk = chunk or settings.chunk_size

    def ax(n):
        out = np.empty(n)
        k = 0.5 / (n - 1)
        for i0 in range(0, n, chunk):
            i1 = min(i0 + chunk, n)
            out[i0:i1] = np.linspace(k * (2 * i0 - n + 1), k * (2 * i1 - n - 1), num=i1 - i0)
        return out

    xs = ax(nx)
    ys = (-ax(ny)) / xy_ratio
    return np.ascontiguousarray(xs), np.ascontiguousarray(ys)


def prepare_m2(*, p, dps, dx, nx, ny=None, max_iter, M=1000., center=None, offset=(0, 0)):
    """Orbit and view for a power-2 Mandelbrot perturbation render centred on
    the period-p nucleus (or ``center``), shifted by ``offset`` (in units of
    dx).  The reference point is the nucleus; the orbit wraps at p."""
    ny = ny or nx
    with mpmath.workdps(dps):
        c = center if center is not None else find_nucleus(p, dps)
        dxm = mpmath.mpf(dx)
        view = c + mpmath.mpc(offset[0], offset[1]) * dxm
        prec = mpmath.mp.prec
        xr_mode = dxm < settings.xrange_zoom_level
        ref_len = min(p, max_iter + 1)
        Zn = np.empty(ref_len, dtype=np.complex128)
        if ref_len == max_iter + 1:
            i, _, xr = fsFP.perturbation_mandelbrot_FP_loop(
                Zn, xr_mode, max_iter, 2 * M, str(c.real), str(c.imag), prec)
        else:
            full = np.empty(ref_len, dtype=np.complex128)
            i, _, xr = fsFP.perturbation_mandelbrot_FP_loop(
                full, xr_mode, ref_len - 1, 2 * M, str(c.real), str(c.imag), prec)
            Zn[:] = full
        idx, m, e = fsx.xr_table(xr)
        dx_xr = fsx.mpf_to_Xrange(dxm)
        drift = fsx.mpc_to_Xrange(view - c)
        # kc (perturbation.py:166-194), Cartesian, no rotation
        half = mpmath.mpf(0.5) * dxm
        shift = c - view
        corners = [mpmath.mpc(sx * half, sy * half / (nx / ny)) for sx in (1, -1) for sy in (1, -1)]
        kc = max(abs(shift - cc) for cc in corners) * mpmath.mpf(1.1)
        kc_xr = fsx.mpf_to_Xrange(kc)
    xs, ys = image_axes(nx, ny, nx / ny)
    return M2Workload(
        p=p, dps=dps, center=view, dx=dxm, nx=nx, ny=ny, max_iter=max_iter, M=M, Zn=Zn,
        div_iter=max_iter + 1, order=p, xr_idx=idx, xr_m=m, xr_e=e, xr_mode=bool(xr_mode),
        dx_m=dx_xr.m, dx_e=dx_xr.e, drift_m=drift.m, drift_e=drift.e,
        kc=kc_xr.to_standard(), xs=xs, ys=ys)


def config2_workload(seed=2, nx=2048, max_iter=200000):
    """2048 x 2048 at dx = 1e-300 on a period-p nucleus, p ~ U[300, 3000],
    400 digits, max_iter 2e5, escape radius 1e3."""
    rng = np.random.default_rng(seed)
    p = int(rng.integers(300, 3001))
    return prepare_m2(p=p, dps=400, dx="1e-300", nx=nx, max_iter=max_iter, M=1000.)
