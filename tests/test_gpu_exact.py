"""
The perturbation kernels against exact arithmetic (z -> z^2 + c iterated
directly at 400 digits by the host library's MPFR orbit): views of width
1e-300 one to three nucleus sizes away from the period-2562 nucleus that
serves as the reference (tests/test_direct_iteration.py pins the oracle on
the same views).  Every pixel of a 16 x 16 view escapes at the exact count in
the XR64 form (the reference's Xrange branch) and in the FP32 + exponent form,
and at 1e-30 in the FP64 form; the fused potential (postproc.py:352-406) is
within 1e-5 of the exact one and the distance estimate (postproc.py:684-731)
within 1e-2 (the reference's own algorithm, BLA eps 1e-6, is off by up to
0.4 % there).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from test_direct_iteration import OFFSETS, offset_view  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from fractalshades_gb300 import _native as nat
    c = nat.Context(0)
    yield c
    c.close()


def run_view(ctx, w, mode):
    from fractalshades_gb300 import _native as nat
    n = w.nx * w.ny
    ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, xr_idx=w.xr_idx,
                        xr_m=w.xr_m, xr_e=w.xr_e, xr_paths=bool(w.xr_mode), calc_dzndc=True,
                        scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
    Z = np.zeros((2, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    pot = np.zeros(n)
    dem = np.zeros(n)
    t = nat.make_tile(xs=w.xs, ys=w.ys, lin_mat=bench.LIN, Z=Z, stop_reason=sr, stop_iter=si,
                      ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
                      i_dzndc=1, potential=pot, dem=dem)
    calc = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=mode, calc_dzndc=True,
                         bla=True, xr_semantics=bool(w.xr_mode))
    ctx.perturb_tiles(calc, [t])
    ref.free()
    return si[0], sr[0], pot, dem


@pytest.mark.parametrize("fac,quarter", OFFSETS)
@pytest.mark.parametrize("mode,dx", [("xr64", "1e-300"), ("fe32", "1e-300"), ("fp64", "1e-30")])
def test_kernels_vs_exact_counts(ctx, fac, quarter, mode, dx):
    w = offset_view(fac, quarter, dx=dx)
    assert w.xr_mode == (dx == "1e-300")
    idx = bench.sample_indices(w.nx * w.ny, 8, 5)
    exact = bench.direct_pixels(w, idx)
    assert len(np.unique(exact["si"])) == 1 and (exact["sr"] == 1).all()
    si, sr, pot, dem = run_view(ctx, w, mode)
    assert (sr == 1).all()
    assert (si == exact["si"][0]).all(), np.unique(si)
    pe, de = bench.potential_dem(exact["zn"], exact["dzndc"], exact["si"], w.M)
    err_p = np.max(np.abs(pot[idx] - pe) / pe)
    err_d = np.max(np.abs(dem[idx] - de) / de)
    print(f"{mode} {dx} offset {fac}/{quarter}: count {exact['si'][0]}, potential "
          f"{err_p:.2e}, DEM {err_d:.2e}")
    assert err_p < 1e-5
    assert err_d < 1e-2
