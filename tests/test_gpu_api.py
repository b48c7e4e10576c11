"""
The model API end to end on the GPU: zoom -> calc_std_div -> calc_raw ->
get_raw, against the oracle, with the reference's on-disk storage (results
found again by a second instance without a launch).
"""
import mpmath
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_standard_calc_raw_vs_oracle_and_storage(tmp_path):
    import fractalshades_gb300.models as fsm

    def make():
        f = fsm.Mandelbrot(str(tmp_path))
        f.zoom(x=-0.5, y=0., dx=3., nx=450, xy_ratio=1.5, theta_deg=0.)
        f.calc_std_div(calc_name="std", subset=None, max_iter=300, M_divergence=1000.,
                       epsilon_stationnary=0.01)
        return f

    f = make()
    f.calc_raw("std")
    xs, ys = f.image_axes()
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    Zo, sio, sro = orc.std_m2(pix, -0.5 + 0j, f.lin_mat, 3.0, 300, 1000., 0.01)
    si = f.get_raw("std", "stop_iter")
    assert np.array_equal(si.ravel(), sio.ravel())
    assert np.array_equal(f.get_raw("std", "stop_reason").ravel(), sro.ravel())
    zn = f.get_raw("std", "zn").ravel()
    assert np.array_equal(zn.view(np.uint64), Zo[f.codes[0].index("zn")].view(np.uint64))
    assert (tmp_path / "data" / "std_Z.arr").exists()

    g = make()
    assert g.calc_raw("std") is None          # stored: nothing launched
    assert np.array_equal(g.get_raw("std", "stop_iter"), si)
    assert np.array_equal(g.get_raw("std", "zn").ravel().view(np.uint64), zn.view(np.uint64))


@pytest.mark.parametrize("mode", ["auto", "fe32"])
def test_perturbation_calc_raw_vs_oracle(tmp_path, mode):
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import settings
    from fractalshades_gb300 import synthetic as syn
    c = syn.find_nucleus(40, 80)
    with mpmath.workdps(80):
        x, y = str(c.real + mpmath.mpf("3e-40")), str(c.imag)
    old = settings.precision_mode
    settings.precision_mode = mode
    try:
        f = fsm.Perturbation_mandelbrot(str(tmp_path / mode))
        f.zoom(precision=80, x=x, y=y, dx="1e-38", nx=64, xy_ratio=1., theta_deg=0.)
        f.calc_std_div(calc_name="deep", subset=None, max_iter=3000, M_divergence=1000.,
                       epsilon_stationnary=1e-3, BLA_eps=1e-6, interior_detect=False,
                       calc_dzndc=True)
        f.calc_raw("deep")
        si = f.get_raw("deep", "stop_iter").ravel()
    finally:
        settings.precision_mode = old
    (Zn, has_xr, idx, xr, div_iter, order, drift, dx) = f.get_path_data()
    kc = f.ref_point_kc().to_standard()
    Mb, rb, _, st = orc.make_bla_m2(Zn, kc, 1e-6)
    dz = orc.dzndc_path_m2(Zn, div_iter, order, False, dx.m, dx.e, None, None, None)
    xs, ys = f.image_axes()
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    Zo, Uo, sro, sio = orc.perturb_m2(
        pix, Zn=Zn, ref_div_iter=div_iter, ref_order=order, lin_mat=f.lin_mat, dx_m=dx.m,
        dx_e=dx.e, drift_m=complex(drift.m), drift_e=drift.e, max_iter=3000, M=1000.,
        eps_stat=1e-3, xr_mode=False, bla=(Mb, rb, st), dZndc=dz)
    agree = float(np.mean(si == sio.ravel()))
    assert agree >= (0.9999 if mode == "auto" else 0.99), agree


@pytest.mark.parametrize("mode", ["auto", "fe32"])
def test_burning_ship_below_double_range(tmp_path, mode):
    """Burning Ship below dx = 1e-300 (the reference's Xrange branch): the
    XR64 loop ("auto") or the FP32 + exponent loop, with unit-scale Jacobian
    paths and the tile's scale 2^e.  Every pixel of the view escapes at the
    iteration a direct 340-digit iteration of the map gives, at 1e-310 as at
    1e-250 (the FP64 path), and the Hessian per unit of c agrees between the
    two depths."""
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import settings
    from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
    with mpmath.workdps(340):
        ok, nuc = fsFP.perturbation_nonholomorphic_find_any_nucleus(
            b"0.88410156557344", b"1.5218981991448", mpmath.mp.prec, 3, 60,
            str(mpmath.mpf(2) ** (-mpmath.mp.prec)).encode(), b"1e-300", 1)
        assert ok
        c0 = nuc + mpmath.mpf("0.015")
        x, y = mpmath.nstr(c0.real, 340), mpmath.nstr(c0.imag, 340)
        zx = zy = mpmath.mpf(0)
        for n0 in range(1, 5000):
            zx, zy = zx * zx - zy * zy + c0.real, 2 * abs(zx * zy) - c0.imag
            if zx * zx + zy * zy > 1e6:
                break
    out = {}
    old = settings.precision_mode
    settings.precision_mode = mode
    try:
        for dx in ("1e-250", "1e-310"):
            f = fsm.Perturbation_burning_ship(str(tmp_path / dx))
            f.zoom(precision=340, x=x, y=y, dx=dx, nx=24, xy_ratio=1., theta_deg=0.)
            f.calc_std_div(calc_name="bs", subset=None, max_iter=2000, M_divergence=1000.,
                           BLA_eps=1e-6, calc_hessian=True)
            f.calc_raw("bs")
            out[dx] = {k: f.get_raw("bs", k) for k in ("stop_iter", "dxnda", "dyndb")}
            assert f.xr_detect_activated == (dx == "1e-310")
    finally:
        settings.precision_mode = old
    for dx, o in out.items():
        assert np.all(o["stop_iter"] == n0), (dx, np.unique(o["stop_iter"]), n0)
    for k in ("dxnda", "dyndb"):
        a = out["1e-310"][k] / 1e-310 * 1e-250       # per unit of c, both
        b = out["1e-250"][k]
        np.testing.assert_allclose(a, b, rtol=1e-3)


@pytest.mark.parametrize("nexp,x,y,dx", [
    # z^3 + c: the edge of the period-10 component, where the ball method
    # finds a period-70 nucleus; the view holds escaping, stationary and
    # max_iter pixels
    (3, "0.64289167998175895118", "0.25147047487965245909", "8e-6"),
    # z^4 + c: the period-10 nucleus at 1e-305 (Xrange branch, interior)
    (4, "-0.51534888699245770184", "0.46481172994907691405", "1e-305"),
])
def test_power_n_calc_raw_vs_oracle(tmp_path, nexp, x, y, dx):
    """Perturbation_mandelbrot_N end to end: ball method and Newton on the
    host, reference tables and the power-n loop on the GPU (FP64 at 8e-6,
    the Xrange branch at 1e-305), against the oracle run on the same orbit;
    Mandelbrot_N's standard loop bit-exact against the oracle."""
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
    if float(dx) < 1e-300:
        # centre on the nucleus to 340 digits (Newton from the 20-digit seed)
        with mpmath.workdps(340):
            ok, nuc = fsFP.perturbation_mandelbrotN_find_any_nucleus(
                x.encode(), y.encode(), mpmath.mp.prec, nexp, 10, 80,
                str(mpmath.mpf(2) ** -mpmath.mp.prec).encode(), b"1e-300")
            assert ok
            x, y = mpmath.nstr(nuc.real, 340), mpmath.nstr(nuc.imag, 340)
    f = fsm.Perturbation_mandelbrot_N(str(tmp_path / "pert"), nexp)
    f.zoom(precision=340, x=x, y=y, dx=dx, nx=48, xy_ratio=1., theta_deg=0.)
    f.calc_std_div(calc_name="mn", subset=None, max_iter=5000, M_divergence=1000.,
                   epsilon_stationnary=1e-3, BLA_eps=1e-6, interior_detect=True,
                   calc_dzndc=True)
    f.calc_raw("mn")
    assert f.FP_params["order"] == (70 if nexp == 3 else 10)
    xr = f.xr_detect_activated
    assert xr == (dx == "1e-305")
    si = f.get_raw("mn", "stop_iter").ravel()
    (Zn, has_xr, idx, xrt, div_iter, order, drift, dxx) = f.get_path_data()
    kc = f.ref_point_kc().to_standard()
    Mb, rb, _, st = orc.make_bla_m2(Zn, kc, 1e-6, nexp)
    xi, xm, xe = (idx, xrt[0], xrt[1]) if has_xr else (None, None, None)
    dz = orc.dzndc_path_m2(Zn, div_iter, order, xr, dxx.m, dxx.e, xi, xm, xe, nexp=nexp)
    dzz = orc.dzndz_path_m2(Zn, div_iter, xr, xi, xm, xe, nexp=nexp)
    xs, ys = f.image_axes()
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    Zo, Uo, sro, sio = orc.perturb_m2(
        pix, Zn=Zn, ref_div_iter=div_iter, ref_order=order, lin_mat=f.lin_mat, dx_m=dxx.m,
        dx_e=dxx.e, drift_m=complex(drift.m), drift_e=drift.e, max_iter=5000, M=1000.,
        eps_stat=1e-3, xr_mode=xr, interior=True, bla=(Mb, rb, st), dZndc=dz, dZndz=dzz,
        xr_idx=xi, xr_m=xm, xr_e=xe, nexp=nexp)
    agree = float(np.mean(si == sio.ravel()))
    assert agree >= 0.9999, agree
    assert np.mean(f.get_raw("mn", "stop_reason").ravel() == sro.ravel()) >= 0.9999

    g = fsm.Mandelbrot_N(str(tmp_path / "std"), nexp)
    g.zoom(x=0., y=0., dx=3., nx=200, xy_ratio=1., theta_deg=0.)
    g.calc_std_div(calc_name="s", subset=None, max_iter=300, M_divergence=1000.,
                   epsilon_stationnary=0.01)
    g.calc_raw("s")
    xs, ys = g.image_axes()
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    Zs, sis, srs = orc.std_mn(pix, 0j, g.lin_mat, 3.0, 300, 1000., 0.01, nexp)
    assert np.array_equal(g.get_raw("s", "stop_iter").ravel(), sis.ravel())
    zn = g.get_raw("s", "zn").ravel()
    assert np.array_equal(zn.view(np.uint64), Zs[0].view(np.uint64))


def test_postproc_batch_fieldlines_and_normals(tmp_path):
    """Mandelbrot with calc_d2zndc2 and calc_orbit (backshift 3), then a
    Postproc_batch of continuous iteration, field lines and DEM normals
    (potential, Milnor), against the reference's outputs for the same view."""
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import postproc as fspp
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "postproc.npz"))
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.5, y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
    f.calc_std_div(calc_name="std", subset=None, max_iter=400, M_divergence=1000.,
                   epsilon_stationnary=0.01, calc_d2zndc2=True, calc_orbit=True, backshift=3)
    f.calc_raw("std")
    f.float_postproc_type = np.float64
    b = fspp.Postproc_batch(f, "std")
    b.add_postproc("cont", fspp.Continuous_iter_pp())
    b.add_postproc("fl", fspp.Fieldlines_pp(n_iter=5, swirl=0.7, endpoint_k=0.5))
    b.add_postproc("dn", fspp.DEM_normal_pp(kind="potential"))
    b.add_postproc("mil", fspp.DEM_normal_pp(kind="Milnor"))
    out = b.evaluate()
    cont = out["cont"].ravel()
    esc = np.isfinite(cont)
    np.testing.assert_array_equal(cont, d["m2_cont"])
    np.testing.assert_allclose(out["fl"].ravel()[esc], d["m2_fl"][esc], rtol=0, atol=1e-9)
    for k in ("dn_x", "dn_y", "mil_x", "mil_y"):
        np.testing.assert_allclose(out[k].ravel(), d[f"m2_{k}"], rtol=0, atol=1e-12)


def test_final_render_supersampling_and_jitter(tmp_path):
    """Postproc_batch in final-render mode: the raw arrays are computed on the
    fly on the 2x2-supersampled, jittered grid (core.py:2572-2593) -- the
    continuous iteration count equals the oracle's on the same points."""
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import postproc as fspp
    from oracle import postproc_ref as ppr
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.5, y=0., dx=3., nx=60, xy_ratio=1.5, theta_deg=0.)
    f.calc_std_div(calc_name="std", subset=None, max_iter=300, M_divergence=1000.,
                   epsilon_stationnary=0.01)
    f.float_postproc_type = np.float64
    b = fspp.Postproc_batch(f, "std")
    b.add_postproc("cont", fspp.Continuous_iter_pp())
    out = b.evaluate({"final_render": True, "supersampling": "2x2", "jitter": 0.5})
    assert out["cont"].shape == (2 * f.ny, 2 * f.nx)
    pix = np.ravel(f.chunk_pixel_pos((0, f.nx, 0, f.ny), 0.5, 2))
    Zo, sio, sro = orc.std_m2(pix, -0.5 + 0j, f.lin_mat, 3.0, 300, 1000., 0.01)
    nu, n = ppr.continuous_context(Zo[0], sio.ravel(), 2, 1000.)
    np.testing.assert_array_equal(out["cont"].ravel(), n + nu)


def test_std_expmap_calc_raw_vs_reference(tmp_path):
    """Mandelbrot under Expmap through the model API (zoom adjusts nx and
    xy_ratio, the kernels project each pixel) against the reference."""
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import projection as fsproj
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "std_expmap.npz"))
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.743643887037151, y=0.13182590420533, dx=1e-4, nx=24, xy_ratio=1.,
           theta_deg=15., projection=fsproj.Expmap(hmin=0., hmax=4.))
    f.calc_std_div(calc_name="s", subset=None, max_iter=2000, M_divergence=1000.,
                   epsilon_stationnary=0.01)
    f.calc_raw("s")
    si = f.get_raw("s", "stop_iter").ravel()
    assert np.mean(si == d["h_si"].ravel()) >= 0.995
