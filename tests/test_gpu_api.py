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
