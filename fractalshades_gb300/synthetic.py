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
import json
import os

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


NUCLEI_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "nuclei.json")
_nuclei = None


def nucleus(p, dps):
    """``find_nucleus(p, dps)``, read from data/nuclei.json when that file
    holds it (written by data/make_nuclei.py with the same search)."""
    global _nuclei
    if _nuclei is None:
        try:
            with open(NUCLEI_FILE) as f:
                _nuclei = json.load(f)
        except (OSError, ValueError):
            _nuclei = {}
    rec = _nuclei.get(f"{p}:{dps}")
    if rec is None:
        return find_nucleus(p, dps)
    with mpmath.workdps(dps):
        return mpmath.mpc(mpmath.mpf(rec[0]), mpmath.mpf(rec[1]))


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


def prepare_m2(*, p, dps, dx, nx, ny=None, max_iter, M=1000., center=None, offset=(0, 0),
               xr_mode=None):
    """Orbit and view for a power-2 Mandelbrot perturbation render centred on
    the period-p nucleus (or ``center``), shifted by ``offset`` (in units of
    dx).  The reference point is the nucleus; the orbit wraps at p.  With
    ``p=None`` the reference is ``center`` itself, without period: its orbit
    has max_iter + 1 points, diverges at its exit index and has no order
    (2^62, perturbation.py:455-456).
    ``xr_mode``: the Xrange branch on or off whatever the width (None: the
    reference's switch, dx < settings.xrange_zoom_level)."""
    ny = ny or nx
    with mpmath.workdps(dps):
        c = center if center is not None else nucleus(p, dps)
        dxm = mpmath.mpf(dx)
        view = c + mpmath.mpc(offset[0], offset[1]) * dxm
        prec = mpmath.mp.prec
        if xr_mode is None:
            xr_mode = dxm < settings.xrange_zoom_level
        ref_len = min(p, max_iter + 1) if p else max_iter + 1
        Zn = np.zeros(ref_len, dtype=np.complex128)
        div_iter = max_iter + 1
        if ref_len == max_iter + 1:
            i, _, xr = fsFP.perturbation_mandelbrot_FP_loop(
                Zn, xr_mode, max_iter, 2 * M, str(c.real), str(c.imag), prec)
            if not p:
                div_iter = int(i)
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
        div_iter=div_iter, order=p if p else (1 << 62), xr_idx=idx, xr_m=m, xr_e=e,
        xr_mode=bool(xr_mode),
        dx_m=dx_xr.m, dx_e=dx_xr.e, drift_m=drift.m, drift_e=drift.e,
        kc=kc_xr.to_standard(), xs=xs, ys=ys)


def config2_workload(seed=2, nx=2048, max_iter=200000):
    """2048 x 2048 at dx = 1e-300 on a period-p nucleus, p ~ U[300, 3000],
    400 digits, max_iter 2e5, escape radius 1e3."""
    rng = np.random.default_rng(seed)
    p = int(rng.integers(300, 3001))
    return prepare_m2(p=p, dps=400, dx="1e-300", nx=nx, max_iter=max_iter, M=1000.)


# ---------------------------------------------------------------------------
# the other measured configurations
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class StdWorkload:
    nx: int
    ny: int
    center: complex
    dx: float
    max_iter: int
    M: float
    eps: float
    xs: np.ndarray
    ys: np.ndarray


def config1_workload():
    """Standard power-2 Mandelbrot: 800 x 600 (xy_ratio 4/3) centred on
    -0.5, width 3, max_iter 1000, escape radius 1e3, stationarity eps 0.01."""
    nx, ny = 800, 600
    xs, ys = image_axes(nx, ny, nx / ny)
    return StdWorkload(nx=nx, ny=ny, center=-0.5 + 0j, dx=3.0, max_iter=1000, M=1000.,
                       eps=0.01, xs=xs, ys=ys)


def edge_workload(nx=1024, max_iter=200000, xr_mode=None, seed=2):
    """The period-2562 nucleus of ``config2_workload`` at width 1.6e-9, about
    four times its nucleus size estimate (3.9e-10, FP_loop.pyx:457-604): the
    minibrot and its surroundings, where about half the pixels escape after
    2.6e3 .. 2e5 iterations.  A boundary-straddling correctness view (the
    1e-300 image is interior everywhere)."""
    p = int(np.random.default_rng(seed).integers(300, 3001))
    return prepare_m2(p=p, dps=400, dx="1.6e-9", nx=nx, max_iter=max_iter, M=1000.,
                      xr_mode=xr_mode)


def seahorse_workload(nx=1024, max_iter=6000):
    """An escape-dominated view: the seahorse valley at
    -0.743643887037151 + 0.131825904205330 i, width 2e-9, 30 digits,
    max_iter 6000, the reference at the centre (no period; it diverges)."""
    with mpmath.workdps(30):
        c = mpmath.mpc("-0.743643887037151", "0.131825904205330")
    return prepare_m2(p=None, dps=30, dx="2.e-9", nx=nx, max_iter=max_iter, M=1000., center=c)


def config3_workload(seed=3, nx=4096, max_iter=1000000):
    """4096 x 4096 at dx = 1e-1000 on a period-p nucleus, p ~ U[2000, 20000],
    1100 digits, max_iter 1e6, interior detection (eps 1e-3)."""
    rng = np.random.default_rng(seed)
    p = int(rng.integers(2000, 20001))
    return prepare_m2(p=p, dps=1100, dx="1e-1000", nx=nx, max_iter=max_iter, M=1000.)


@dataclasses.dataclass
class BSTile:
    side: int
    dx: object              # mpmath mpf
    seed_point: tuple       # (x0, y0) floats drawn
    order: object           # period found by the ball method + Newton, or None
    Zn: np.ndarray          # complex128 (x + i y) [len]
    div_iter: int
    ref_order: int
    dx_m: float
    dx_e: int
    driftx_m: float
    driftx_e: int
    drifty_m: float
    drifty_e: int
    kc: float
    xs: np.ndarray
    ys: np.ndarray


def bs_center(rng, dps, kind=1, radius="1e-3", tries=64, max_iter=50000):
    """A Burning Ship view centre: seeded points x ~ U[-1.8, -1.7],
    y ~ U[-0.1, 0], the first whose order-1 ball of ``radius`` finds a period
    (FP_loop.pyx:2357-2440), refined by Newton (FP_loop.pyx:2564-2720); the
    last raw point when no draw finds one (the reference's fallback,
    perturbation.py:747-751)."""
    with mpmath.workdps(dps):
        prec = mpmath.mp.prec
        for _ in range(tries):
            x0, y0 = -1.8 + 0.1 * rng.random(), -0.1 * rng.random()
            order = fsFP.perturbation_nonholomorphic_ball_method(
                repr(x0), repr(y0), prec, radius, max_iter, 1e5, kind)
            if order <= 0:
                continue
            ok, c = fsFP.perturbation_nonholomorphic_find_any_nucleus(
                repr(x0), repr(y0), prec, order, 80, str(mpmath.mpf(val=(2, -prec))),
                str(mpmath.mpf(10) ** (-(dps // 2))), kind)
            if ok:
                return (x0, y0), c, order
        return (x0, y0), mpmath.mpc(x0, y0), None


def config4_workload(seed=4, n_tiles=64, max_iter=50000, M=1000., kind=1, dps=250,
                     newton=True, edge=False):
    """64 Burning Ship tiles, side round(exp(U[ln 256, ln 2048])), width
    10^U[-200, -30], each on its own centre (``bs_center``) with its own
    250-digit reference orbit; max_iter 5e4, escape radius 1e3.
    newton=False: the raw seeded points are the centres (the reference's
    fallback when no nucleus is found, perturbation.py:747-757) -- points off
    the real axis; the widths are drawn the same way.
    edge=True: each tile whose centre is a nucleus takes as width four times
    that nucleus' size estimate (FP_loop.pyx:2100-2356), so that it straddles
    the minibrot's boundary and pixels escape (the seeded width where there is
    no nucleus or the estimate is not a finite size below 1)."""
    rng = np.random.default_rng(seed)
    tiles = []
    for _ in range(n_tiles):
        side = int(round(np.exp(rng.uniform(np.log(256), np.log(2048)))))
        width_exp = rng.uniform(-200, -30)
        if newton:
            seed_pt, c, order = bs_center(rng, dps, kind)
        else:
            x0, y0 = -1.8 + 0.1 * rng.random(), -0.1 * rng.random()
            with mpmath.workdps(dps):
                seed_pt, c, order = (x0, y0), mpmath.mpc(x0, y0), None
        with mpmath.workdps(dps):
            dxm = mpmath.mpf(10) ** mpmath.mpf(width_exp)
            prec = mpmath.mp.prec
            if edge and order:
                size, _ = fsFP.perturbation_nonholomorphic_nucleus_size_estimate(
                    str(c.real), str(c.imag), prec, order, kind)
                size = abs(mpmath.mpf(size))
                if mpmath.isfinite(size) and 0 < size < 1:
                    dxm = 4 * size
            ref_len = min(order, max_iter + 1) if order else max_iter + 1
            orb = np.empty(max_iter + 1 if not order else ref_len, dtype=np.complex128)
            i, _, _ = fsFP.perturbation_nonholomorphic_FP_loop(
                orb.view(np.float64), False, orb.size - 1, 2 * M, str(c.real), str(c.imag),
                prec, kind)
            div_iter = max_iter + 1 if order else i
            Zn = orb[:ref_len] if order else orb[:min(i + 1, orb.size)]
            dx_xr = fsx.mpf_to_Xrange(dxm)
            half = mpmath.mpf(0.5) * dxm
            kc = mpmath.sqrt(2) * half * mpmath.mpf(1.1)
            kc_xr = fsx.mpf_to_Xrange(kc)
        xs, ys = image_axes(side, side)
        tiles.append(BSTile(
            side=side, dx=dxm, seed_point=seed_pt, order=order, Zn=np.ascontiguousarray(Zn),
            div_iter=int(div_iter), ref_order=int(order) if order else (1 << 62),
            dx_m=dx_xr.m, dx_e=dx_xr.e, driftx_m=0., driftx_e=0, drifty_m=0., drifty_e=0,
            kc=kc_xr.to_standard(), xs=xs, ys=ys))
    return tiles
