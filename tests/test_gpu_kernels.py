"""
GPU kernels against the CPU oracle, through the C-ABI (include/fsgpu.h).

Inputs are the golden fixtures (reference orbits, pixel grids) of
tests/golden/.  The FP64 and Xrange (XR64) kernels reproduce the oracle's
operation order (-fmad=false): integer outputs must agree on >= 99.99 % of the
pixels with the rest within 1 iteration, floating outputs within 1e-6
relative.  The FE32 kernel is held to the same iteration-count criterion.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(G, name + ".npz"), allow_pickle=False)


@pytest.fixture(scope="module")
def ctx():
    from fractalshades_gb300 import _native as nat
    c = nat.Context(0)
    yield c
    c.close()


def axes(pix, nx):
    pix = np.asarray(pix)
    xs = np.ascontiguousarray(pix[:nx].real)
    ys = np.ascontiguousarray(pix[::nx].imag)
    ny = ys.size
    assert np.array_equal(pix, (xs[None, :] + 1j * ys[:, None]).ravel()) or \
        np.array_equal(pix.real, np.tile(xs, ny))
    return xs, ys


def iter_agree(a, b, frac=0.9999, tol=1):
    a = np.asarray(a).ravel().astype(np.int64)
    b = np.asarray(b).ravel().astype(np.int64)
    same = np.mean(a == b)
    assert same >= frac, f"only {same:.6f} of the iteration counts agree"
    assert np.max(np.abs(a - b)) <= tol or same == 1.0 or np.mean(np.abs(a - b) <= tol) >= frac


def rel_close(a, b, rtol=1e-6, mask=None):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    if mask is not None:
        a, b = a[mask.ravel()], b[mask.ravel()]
    ok = np.isfinite(a) & np.isfinite(b)
    assert np.array_equal(np.isfinite(a), np.isfinite(b))
    err = np.abs(a[ok] - b[ok]) / np.maximum(np.abs(b[ok]), 1e-300)
    assert err.size == 0 or np.max(err) <= rtol, f"max rel err {np.max(err)}"


# ---------------------------------------------------------------------------
def test_std_m2_bit_exact_vs_oracle(ctx):
    from fractalshades_gb300 import _native as nat
    d = load("std_m2")
    nx = int(d["nx"])
    xs, ys = axes(d["pix"], nx)
    n = xs.size * ys.size
    Z = np.zeros((3, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    pot = np.zeros(n)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr, stop_iter=si,
                      center=complex(*d["center"]), dx=float(d["dx"]), potential=pot)
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                         epsilon_stationnary=float(d["eps"]), flavor=0)
    ctx.std_tiles(calc, [t])
    assert np.array_equal(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    assert np.array_equal(Z.view(np.uint64), d["Z"].view(np.uint64))
    st = ctx.stats()
    assert st["pixel_iters"] == int(d["stop_iter"].sum())


def test_std_m2_full_config_vs_oracle(ctx):
    """800 x 600, x=-0.5, dx=3, max_iter 1000, M 1000 (the standard-loop
    configuration), bit-exact against the oracle."""
    from fractalshades_gb300 import _native as nat
    nx, ny = 800, 600
    kx, ky = 0.5 / (nx - 1), 0.5 / (ny - 1)
    xs = np.linspace(kx * (-nx + 1), kx * (nx - 1), nx)
    ys = -np.linspace(ky * (-ny + 1), ky * (ny - 1), ny) / (4. / 3.)
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    lin = np.array([[1., -0.], [0., 1.]])
    Zo, sio, sro = orc.std_m2(pix, -0.5 + 0j, lin, 3.0, 1000, 1000., 0.01)
    n = nx * ny
    Z = np.zeros((3, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=lin, Z=Z, stop_reason=sr, stop_iter=si,
                      center=-0.5 + 0j, dx=3.0)
    ctx.std_tiles(nat.make_calc(max_iter=1000, M_divergence=1000., epsilon_stationnary=0.01), [t])
    assert np.array_equal(si, sio)
    assert np.array_equal(sr, sro)
    assert np.array_equal(Z.view(np.uint64), Zo.view(np.uint64))


@pytest.mark.parametrize("flavor", [1, 2, 3, 4, 5])
def test_std_bs_vs_oracle(ctx, flavor):
    from fractalshades_gb300 import _native as nat
    d = load("std_bs")
    pix = d[f"pix_{flavor}"]
    nx = int(round(np.sqrt(pix.size)))
    xs, ys = axes(pix, nx)
    n = pix.size
    Z = np.zeros((6, n))
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr, stop_iter=si,
                      center=complex(*d["center"]), dx=float(d["dx"]))
    ctx.std_tiles(nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                                flavor=flavor), [t])
    assert np.array_equal(si, d[f"stop_iter_{flavor}"])
    assert np.array_equal(sr, d[f"stop_reason_{flavor}"])
    assert np.array_equal(Z.view(np.uint64), d[f"Z_{flavor}"].view(np.uint64))


def _std_opts(ctx, pix, center, dx, max_iter, eps, nZ, i_orb, **calc_kw):
    from fractalshades_gb300 import _native as nat
    nx = int(round(np.sqrt(pix.size)))
    xs, ys = axes(pix, nx)
    n = pix.size
    dt = np.complex128 if calc_kw.get("flavor", 0) == 0 else np.float64
    Z = np.zeros((nZ, n), dtype=dt)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    d = load("std_opts")
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr, stop_iter=si,
                      center=center, dx=dx, i_znorbit=i_orb)
    ctx.std_tiles(nat.make_calc(max_iter=max_iter, M_divergence=1000.,
                                epsilon_stationnary=eps, **calc_kw), [t])
    return Z, si, sr


def test_std_options_bit_exact_vs_golden(ctx):
    """d2zndc2 and the orbit point n - backshift of the standard loops
    (mandelbrot_M2.py:316-317, mandelbrot_Mn.py:325-333, core.py:2965-3056)
    against the reference's own outputs."""
    d = load("std_opts")
    Z, si, sr = _std_opts(ctx, d["pix_m2"], -0.5 + 0j, 3., 400, 0.01, 5, 4,
                          calc_d2zndc2=True, backshift=3)
    assert np.array_equal(si, d["stop_iter_m2"]) and np.array_equal(sr, d["stop_reason_m2"])
    assert np.array_equal(Z.view(np.uint64), d["Z_m2"].view(np.uint64))
    for nexp in (2, 3):
        Z, si, sr = _std_opts(ctx, d[f"pix_mn{nexp}"], 0j, 3., 300, 0.01, 5, 4,
                              calc_d2zndc2=True, backshift=4, nexp=nexp)
        assert np.array_equal(si, d[f"stop_iter_mn{nexp}"])
        assert np.array_equal(Z.view(np.uint64), d[f"Z_mn{nexp}"].view(np.uint64)), nexp
    for fl in (1, 4):
        Z, si, sr = _std_opts(ctx, d[f"pix_bs{fl}"], -0.5 - 0.5j, 3.5, 200, 0., 8, 6,
                              flavor=fl, backshift=3)
        assert np.array_equal(si, d[f"stop_iter_bs{fl}"])
        assert np.array_equal(Z.view(np.uint64), d[f"Z_bs{fl}"].view(np.uint64)), fl


def test_orbit_options_are_validated(ctx):
    """calc_orbit in the FP32 + exponent form, a row index that collides with
    the other outputs, a negative backshift and d2zndc2 outside the standard
    Mandelbrot loop are refused."""
    from fractalshades_gb300 import _native as nat
    d = load("std_opts")
    for kw, nZ, i_orb in (({"backshift": -1}, 3, 0), ({"backshift": 3}, 4, 2),
                          ({"calc_d2zndc2": True, "flavor": 1}, 6, 0)):
        with pytest.raises(RuntimeError):
            _std_opts(ctx, d["pix_m2"], -0.5 + 0j, 3., 10, 0.01, nZ, i_orb, **kw)
    dd = load("pert_m2_orbit")
    ref = _ref_from_golden(ctx, dd, False)
    with pytest.raises(RuntimeError):
        _run_m2(ctx, dd, ref, "fe32", False)


@pytest.mark.parametrize("nexp", [3, 4])
def test_std_mn_bit_exact_vs_golden(ctx, nexp):
    """Power-n standard loop against the reference's own outputs."""
    from fractalshades_gb300 import _native as nat
    d = load("std_mn")
    pix = d[f"pix_{nexp}"]
    nx = int(round(np.sqrt(pix.size)))
    xs, ys = axes(pix, nx)
    n = pix.size
    Z = np.zeros((3, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    pot = np.zeros(n)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr, stop_iter=si,
                      center=complex(*d["center"]), dx=float(d["dx"]), potential=pot)
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                         epsilon_stationnary=float(d["eps"]), flavor=0, nexp=nexp)
    ctx.std_tiles(calc, [t])
    assert np.array_equal(si, d[f"stop_iter_{nexp}"])
    assert np.array_equal(sr, d[f"stop_reason_{nexp}"])
    assert np.array_equal(Z.view(np.uint64), d[f"Z_{nexp}"].view(np.uint64))
    # potential with d = n (postproc.py:1001-1009)
    esc = (sr[0] == 1)
    az = np.abs(Z[0][esc])
    nu = -(np.log(np.log(az) / np.log(float(d["M"]))) / np.log(nexp))
    q = np.floor(-nu)
    np.testing.assert_allclose(pot[esc], (si[0][esc] - q) - (-nu - q), rtol=1e-12)


# ---------------------------------------------------------------------------
def _nexp(d):
    return int(d["nexp"]) if "nexp" in d.files else 0


def _ref_from_golden(ctx, d, xr_paths):
    from fractalshades_gb300 import _native as nat
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    return nat.Reference(
        ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
        xr_idx=d["xr_idx"], xr_m=d["xr_m"], xr_e=d["xr_e"], xr_paths=xr_paths,
        calc_dzndc=True, calc_dzndz=bool(d["interior"]), scale_m=float(d["dx_m"]),
        scale_e=int(d["dx_e"]), bla=True, kc=kc, bla_eps=float(d["bla_eps"]),
        nexp=_nexp(d))


def _backshift(d):
    return int(d["backshift"]) if "backshift" in d.files else 0


def _run_m2(ctx, d, ref, mode, xr_sem):
    from fractalshades_gb300 import _native as nat
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    interior = bool(d["interior"])
    bs = _backshift(d)
    nZ = 2 + int(interior) + int(bs > 0)
    Z = np.zeros((nZ, n), dtype=np.complex128)
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, U=U, stop_reason=sr,
                      stop_iter=si, ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]),
                      i_dzndz=1 if interior else -1, i_dzndc=1 + int(interior),
                      i_znorbit=nZ - 1 if bs > 0 else 0)
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                         epsilon_stationnary=float(d["eps_stat"]), mode=mode,
                         calc_dzndc=True, interior=interior, bla=True,
                         xr_semantics=xr_sem, nexp=_nexp(d), backshift=bs)
    ctx.perturb_tiles(calc, [t])
    return Z, U, sr, si


M2_CASES = ["pert_m2_fp64", "pert_m2_cycle", "pert_m2_xr", "pert_m2_xr_div",
            # the period-2562 nucleus of the 2048^2 / 1e-300 workload, max_iter
            # 2e5: at 1e-300 (Xrange branch) and at the boundary-straddling
            # width 1.6e-9 (FP64 branch, and the Xrange branch forced)
            "pert_m2_p2562_1e300", "pert_m2_p2562_edge", "pert_m2_p2562_edge_xr"]
# power-n model: period-10 nuclei of z^3 + c (interior and escaping views)
# and of z^4 + c at dx = 1e-305 (Xrange branch)
MN_CASES = ["pert_mn3_cycle", "pert_mn3_div", "pert_mn4_xr"]
# calc_orbit (backshift 5, 7, 4): FP64 and Xrange branches, power 2 and 3
ORBIT_CASES = ["pert_m2_orbit", "pert_m2_xr_orbit", "pert_mn3_orbit"]


def _xr_rel(m, e, eref):
    return m * np.exp2((np.asarray(e, dtype=np.int64) - eref).astype(float))


@pytest.mark.parametrize("case", M2_CASES + MN_CASES)
def test_ref_tables_vs_oracle(ctx, case):
    """BLA tree and derivative paths built on the GPU against the oracle's
    (same operation order; CUDA's hypot may differ from the C library's by an
    ulp in the BLA radii, and the combine's r2 - |B1| kc can amplify that ulp
    by a few tens: 1.5e-14 relative on one radius of the period-2562 tree)."""
    d = load(case)
    xr = bool(d["xr_mode"])
    ref = _ref_from_golden(ctx, d, xr)
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mo, ro, _, st = orc.make_bla_m2(d["Zn"], kc, float(d["bla_eps"]), _nexp(d))
    M, r = ref.download("bla")
    assert ref.stages == st
    np.testing.assert_allclose(r, ro, rtol=1e-13, atol=0)
    np.testing.assert_allclose(M, Mo, rtol=1e-14, atol=0)
    dzo = orc.dzndc_path_m2(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), xr,
                            float(d["dx_m"]), int(d["dx_e"]), d["xr_idx"], d["xr_m"], d["xr_e"],
                            nexp=_nexp(d))
    dz = ref.download("dzndc")
    if xr:
        eref = int(dzo[1].max())
        np.testing.assert_allclose(_xr_rel(dz[0], dz[1], eref),
                                   _xr_rel(dzo[0], dzo[1], eref), rtol=1e-15, atol=0)
    else:
        assert np.array_equal(dz.view(np.uint64), dzo.view(np.uint64))
    if bool(d["interior"]):
        dzzo = orc.dzndz_path_m2(d["Zn"], int(d["ref_div_iter"]), xr, d["xr_idx"],
                                 d["xr_m"], d["xr_e"], nexp=_nexp(d))
        dzz = ref.download("dzndz")
        if xr:
            eref = int(dzzo[1].max())
            np.testing.assert_allclose(_xr_rel(dzz[0], dzz[1], eref),
                                       _xr_rel(dzzo[0], dzzo[1], eref), rtol=1e-15, atol=0)
        else:
            assert np.array_equal(dzz.view(np.uint64), dzzo.view(np.uint64))


@pytest.mark.parametrize("case", M2_CASES + MN_CASES + ORBIT_CASES)
def test_perturb_m2_reference_branch_vs_oracle(ctx, case):
    """FP64 kernel on the standard-branch cases, XR64 on the Xrange cases."""
    d = load(case)
    xr = bool(d["xr_mode"])
    ref = _ref_from_golden(ctx, d, xr)
    Z, U, sr, si = _run_m2(ctx, d, ref, "xr64" if xr else "fp64", xr)
    iter_agree(si, d["stop_iter"])
    assert np.mean(sr == d["stop_reason"]) >= 0.9999
    same = (si == d["stop_iter"]).ravel()
    for k in range(Z.shape[0]):
        if k == 1 and bool(d["interior"]):
            continue          # the Xrange branch never writes dzndz back
        rel_close(Z[k], d["Z"][k], 1e-6, same)


def _oracle_fp32_sensitivity(d):
    """Fraction of pixels whose iteration count changes when every pixel's
    c offset is moved by a relative 2^-24 (one FP32 rounding), in the oracle:
    the scale of count differences any FP32-mantissa form meets on a case."""
    kw = dict(_oracle_kw(d))
    a = orc.perturb_m2(d["pix"], **kw)[3]
    kw["lin_mat"] = np.asarray(d["lin_mat"]) * (1. + 2. ** -24)
    b = orc.perturb_m2(d["pix"], **kw)[3]
    return float(np.mean(a != b))


# The bar of the FP32+exponent form: its iteration counts may differ from the
# oracle's on at most 2.5 x the case's FP32 sensitivity plus 0.5 % of the
# pixels (measured on escape-dominated views: 1.7 x), its stop reasons on at
# most the same fraction.
FE32_SENSITIVITY_FACTOR = 2.5
FE32_ALLOWANCE = 0.005


def _oracle_kw(d):
    xr = bool(d["xr_mode"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, _, st = orc.make_bla_m2(d["Zn"], kc, float(d["bla_eps"]))
    dz = orc.dzndc_path_m2(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), xr,
                           float(d["dx_m"]), int(d["dx_e"]), d["xr_idx"], d["xr_m"], d["xr_e"])
    kw = dict(Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]), ref_order=int(d["ref_order"]),
              lin_mat=d["lin_mat"], dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
              drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]),
              max_iter=int(d["max_iter"]), M=float(d["M"]), eps_stat=float(d["eps_stat"]),
              xr_mode=xr, interior=bool(d["interior"]), bla=(Mb, rb, st), dZndc=dz,
              xr_idx=d["xr_idx"], xr_m=d["xr_m"], xr_e=d["xr_e"])
    if bool(d["interior"]):
        kw["dZndz"] = orc.dzndz_path_m2(d["Zn"], int(d["ref_div_iter"]), xr, d["xr_idx"],
                                        d["xr_m"], d["xr_e"])
    return kw


@pytest.mark.parametrize("case", M2_CASES)
def test_perturb_m2_fe32_vs_oracle(ctx, case):
    """FP32-mantissa deltas against the reference's counts: differences on at
    most FE32_SENSITIVITY_FACTOR x the case's FP32 sensitivity (the oracle
    against itself with c moved by 2^-24) + FE32_ALLOWANCE of the pixels."""
    d = load(case)
    xr = bool(d["xr_mode"])
    ref = _ref_from_golden(ctx, d, xr)
    Z, U, sr, si = _run_m2(ctx, d, ref, "fe32", xr)
    bar = FE32_SENSITIVITY_FACTOR * _oracle_fp32_sensitivity(d) + FE32_ALLOWANCE
    differ = float(np.mean(si != d["stop_iter"]))
    assert differ <= bar, f"FE32 counts differ on {differ:.4f} of the pixels, bar {bar:.4f}"
    assert np.mean(sr != d["stop_reason"]) <= bar


def _run_bs(ctx, d, mode):
    from fractalshades_gb300 import _native as nat
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    ref = nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
                        flavor=fl, calc_dzndc=True, scale_m=float(d["dx_m"]),
                        scale_e=int(d["dx_e"]), bla=True, kc=kc, bla_eps=float(d["bla_eps"]))
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    Z = np.zeros((6, n))
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, U=U, stop_reason=sr,
                      stop_iter=si, ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=float(d["driftx_m"]), drift_e=int(d["driftx_e"]),
                      drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]))
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]), flavor=fl,
                         calc_dzndc=True, bla=True, mode=mode)
    ctx.perturb_tiles(calc, [t])
    return Z, sr, si


def _oracle_bs(d, lin_scale=1.):
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, _, st = orc.make_bla_bs(d["Zn"], fl, kc, float(d["bla_eps"]))
    paths = orc.dzndc_path_bs(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), fl,
                              float(np.ldexp(d["dx_m"], d["dx_e"])))
    return orc.perturb_bs(
        d["pix"], Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]),
        ref_order=int(d["ref_order"]), lin_mat=np.asarray(d["lin_mat"]) * lin_scale,
        dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
        driftx_m=float(d["driftx_m"]), driftx_e=int(d["driftx_e"]),
        drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
        max_iter=int(d["max_iter"]), M=float(d["M"]), flavor=fl, bla=(Mb, rb, st),
        dpaths=paths)


BS_CASES = ["pert_bs_1", "pert_bs_4",
            # flavors 2, 3, 5 and a second Celtic view, each around a point of
            # its set's boundary (reference diverging, pixels escaping or not)
            "pert_bs_2", "pert_bs_3", "pert_bs_4e", "pert_bs_5"]


def _z_rel_err(Z, Zo, si, sio):
    same = (si == sio).ravel()
    z = Z[0].ravel()[same] + 1j * Z[1].ravel()[same]
    zo = Zo[0].ravel()[same] + 1j * Zo[1].ravel()[same]
    return np.abs(z - zo) / np.abs(zo)              # relative to |z|


@pytest.mark.parametrize("case", BS_CASES)
def test_perturb_bs_fe32_vs_oracle(ctx, case):
    """Burning Ship with FP32-mantissa + int32-exponent deltas against the
    reference's results, on the bar of the power-2 form: counts and stop
    reasons differ on at most FE32_SENSITIVITY_FACTOR x the case's FP32
    sensitivity (the oracle against itself with c moved by 2^-24) +
    FE32_ALLOWANCE of the pixels; z at exit (pixels with equal counts),
    relative to |z|, within 100 x the oracle's own shift in median and 90th
    percentile (the FP32 rounding of dz is amplified by the orbit's derivative
    on the way out, as a 2^-24 change of c is)."""
    d = load(case)
    Z, sr, si = _run_bs(ctx, d, "fe32")
    Zs, _, srs, sis = _oracle_bs(d, 1. + 2. ** -24)
    sens = float(np.mean(sis != d["stop_iter"]))
    bar = FE32_SENSITIVITY_FACTOR * sens + FE32_ALLOWANCE
    differ = float(np.mean(si != d["stop_iter"]))
    assert differ <= bar, f"counts differ on {differ:.4f}, bar {bar:.4f}"
    assert np.mean(sr != d["stop_reason"]) <= bar
    err = _z_rel_err(Z, d["Z"], si, d["stop_iter"])
    err_s = _z_rel_err(Zs, d["Z"], sis, d["stop_iter"])
    for q in (50, 90):
        a, b = np.percentile(err, q), np.percentile(err_s, q)
        assert a <= 100. * b + 1e-6, (q, a, b)


def _bs_nucleus(kind, real_axis):
    """A period-p nucleus of the flavor (ball method + Newton at 300 bits on
    the native host side) and its orbit over one period."""
    import mpmath
    from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
    rng = np.random.default_rng(10 + kind + (100 if real_axis else 0))
    prec = 300
    with mpmath.workprec(prec):
        for _ in range(60):
            if real_axis:
                c0 = mpmath.mpc(-1.8 + 0.1 * rng.random(), -0.1 * rng.random())
            else:
                c0 = mpmath.mpc(-2 + 2.5 * rng.random(), -1.5 + 2 * rng.random())
            sx, sy = str(c0.real).encode(), str(c0.imag).encode()
            order = fsFP.perturbation_nonholomorphic_ball_method(sx, sy, prec, b"0.01", 400,
                                                                 1e5, kind)
            if order < 3 or order > 200:
                continue
            ok, c = fsFP.perturbation_nonholomorphic_find_any_nucleus(
                sx, sy, prec, order, 80, str(mpmath.mpf(val=(2, -prec))).encode(), b"1e-60",
                kind)
            if not ok:
                continue
            orb = np.zeros(order + 1, dtype=np.complex128)
            fsFP.perturbation_nonholomorphic_FP_loop(orb.view(np.float64), False, order, 2e3,
                                                     str(c.real).encode(), str(c.imag).encode(),
                                                     prec, kind)
            return orb[:order], order
    pytest.skip("no nucleus found")


@pytest.mark.parametrize("dx", [1e-9, 1e-45])
@pytest.mark.parametrize("kind,real_axis", [(k, r) for k in (1, 2, 3, 4, 5) for r in (True, False)])
def test_perturb_bs_fe32_vs_fp64_every_flavor(ctx, kind, real_axis, dx):
    """The FP32 + exponent Burning Ship loop (fr values and their frame form)
    against the FP64 kernel on the same reference and tile, every flavor,
    around nuclei on and off the real axis: iteration counts on >= 99 % of the
    pixels, z and the Hessian to FP32 accuracy amplified by the orbit.  The
    Hessian is compared normwise (against the pixel's largest entry) and
    entry by entry above 1e-6 of it: the frame form holds the four entries on
    one exponent, so an entry far below the others (the cross terms around a
    real-axis reference, ~1e-112 of the diagonal) is resolved only to that
    absolute level."""
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300.synthetic import image_axes
    Zn, order = _bs_nucleus(kind, real_axis)
    max_iter, side = 3000, 96
    m, e = np.frexp(dx)
    kc = float(np.sqrt(2) * 0.5 * dx * 1.1)
    ref = nat.Reference(ctx, Zn, div_iter=max_iter + 1, order=order, flavor=kind,
                        calc_dzndc=True, scale_m=float(m), scale_e=int(e), bla=True, kc=kc,
                        bla_eps=1e-6)
    xs, ys = image_axes(side, side)
    out = {}
    for mode in ("fp64", "fe32"):
        n = side * side
        Z = np.zeros((6, n))
        U = np.zeros((1, n), dtype=np.int32)
        sr = -np.ones((1, n), dtype=np.int8)
        si = np.zeros((1, n), dtype=np.int32)
        t = nat.make_tile(xs=xs, ys=ys, lin_mat=np.eye(2), Z=Z, U=U, stop_reason=sr,
                          stop_iter=si, ref=ref, dx_m=float(m), dx_e=int(e), drift_m=0.,
                          drift_e=0, drifty_m=0., drifty_e=0)
        calc = nat.make_calc(max_iter=max_iter, M_divergence=1e3, flavor=kind, calc_dzndc=True,
                             bla=True, mode=mode)
        ctx.perturb_tiles(calc, [t])
        out[mode] = (Z, sr, si)
    Z64, sr64, si64 = out["fp64"]
    Z32, sr32, si32 = out["fe32"]
    assert np.mean(si32 == si64) >= 0.99, np.mean(si32 == si64)
    assert np.mean(sr32 == sr64) >= 0.99
    same = (si32 == si64).ravel()
    z64 = np.hypot(Z64[0], Z64[1])[same]
    dz = np.hypot(Z32[0] - Z64[0], Z32[1] - Z64[1])[same]
    err = dz / np.maximum(z64, 1e-300)
    assert np.median(err) <= 1e-3, np.median(err)
    # the Hessian, relative to its largest entry per pixel, and entry by entry
    H64, H32 = Z64[2:6][:, same], Z32[2:6][:, same]
    hmax = np.max(np.abs(H64), axis=0)
    herr = np.max(np.abs(H32 - H64), axis=0) / np.maximum(hmax, 1e-300)
    assert np.median(herr) <= 1e-2, np.median(herr)
    for k in range(4):
        big = np.abs(H64[k]) > 1e-6 * hmax
        if np.any(big):
            ek = np.abs(H32[k] - H64[k])[big] / np.abs(H64[k])[big]
            assert np.median(ek) <= 1e-2, (k, np.median(ek))


@pytest.mark.parametrize("case", BS_CASES + ["pert_bs_orbit"])
def test_perturb_bs_vs_oracle(ctx, case):
    from fractalshades_gb300 import _native as nat
    d = load(case)
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    ref = nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
                        flavor=fl, calc_dzndc=True, scale_m=float(d["dx_m"]),
                        scale_e=int(d["dx_e"]), bla=True, kc=kc, bla_eps=float(d["bla_eps"]))
    paths = ref.download("bs_paths")
    for k, name in enumerate(["dXa", "dXb", "dYa", "dYb"]):
        assert np.array_equal(paths[k].view(np.uint64), d[name].view(np.uint64))
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    bs = _backshift(d)
    nZ = 8 if bs > 0 else 6
    Z = np.zeros((nZ, n))
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, U=U, stop_reason=sr,
                      stop_iter=si, ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=float(d["driftx_m"]), drift_e=int(d["driftx_e"]),
                      drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
                      i_znorbit=6 if bs > 0 else 0)
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]), flavor=fl,
                         calc_dzndc=True, bla=True, backshift=bs)
    ctx.perturb_tiles(calc, [t])
    iter_agree(si, d["stop_iter"])
    same = (si == d["stop_iter"]).ravel()
    for k in range(nZ):
        rel_close(Z[k], d["Z"][k], 1e-6, same)


@pytest.mark.parametrize("mode", ["fp64", "fe32"])
def test_dzndc_scale_and_derived_bla(ctx, mode):
    """fsg_tile.dzndc_scale_e = k on a reference of derivative scale 2^s gives
    the outputs of a reference of scale 2^(s+k) (the derivative recurrence is
    linear in its scale; power-of-two scaling is exact), and a BLA tree
    derived with fsg_ref_derive_bla equals the one of a fresh reference."""
    from fractalshades_gb300 import _native as nat
    d = load("pert_m2_fp64")
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))

    def ref(scale_e, kc_=kc, bla=True):
        return nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]),
                             order=int(d["ref_order"]), calc_dzndc=True,
                             scale_m=float(d["dx_m"]), scale_e=int(d["dx_e"]) + scale_e,
                             bla=bla, kc=kc_, bla_eps=float(d["bla_eps"]))

    def run(r, k):
        nx = int(round(np.sqrt(d["pix"].size)))
        xs, ys = axes(d["pix"], nx)
        n = d["pix"].size
        Z = np.zeros((2, n), dtype=np.complex128)
        sr = -np.ones((1, n), dtype=np.int8)
        si = np.zeros((1, n), dtype=np.int32)
        dem = np.zeros(n)
        pot = np.zeros(n)
        t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr,
                          stop_iter=si, ref=r, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                          drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]),
                          i_dzndc=1, potential=pot, dem=dem, dzndc_scale_e=k)
        ctx.perturb_tiles(nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                                        mode=mode, calc_dzndc=True, bla=True), [t])
        return Z, si, dem

    Za, sia, dema = run(ref(7), 0)
    Zb, sib, demb = run(ref(0), 7)
    assert np.array_equal(sia, sib)
    assert np.array_equal(Za.view(np.uint64), Zb.view(np.uint64))
    assert np.array_equal(dema.view(np.uint64), demb.view(np.uint64))
    base = ref(0, bla=False)
    kc2 = kc * 4.
    derived = base.derive_bla(kc2, float(d["bla_eps"]))
    Zc, sic, _ = run(derived, 7)
    Zd, sid, _ = run(ref(0, kc_=kc2), 7)
    assert np.array_equal(sic, sid)
    assert np.array_equal(Zc.view(np.uint64), Zd.view(np.uint64))
    with pytest.raises(nat.GPUError):
        base.free()                 # a base outlives the references derived from it
    derived.free()
    base.free()


def test_power_n_rejects_fe32_and_mismatched_exponent(ctx):
    """The power-n model runs in FP64 / XR64; a reference built for one
    exponent serves no calculation of another."""
    from fractalshades_gb300 import _native as nat
    d = load("pert_mn3_div")
    ref = _ref_from_golden(ctx, d, False)
    with pytest.raises(RuntimeError):
        _run_m2(ctx, d, ref, "fe32", False)
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    Z = np.zeros((2, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, stop_reason=sr, stop_iter=si,
                      ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]), i_dzndc=1)
    for k in (0, 4):
        with pytest.raises(RuntimeError):
            ctx.perturb_tiles(nat.make_calc(max_iter=100, M_divergence=1e3, nexp=k), [t])


# ---------------------------------------------------------------------------
# post-processing kernels (csrc/fsg_postproc.cu) against the reference's
# Postproc_batch outputs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("pre,model,i_orb", [("m2", 0, 4), ("mn3", 3, 3), ("bs1", -1, 6)])
def test_postproc_kernels_vs_reference(ctx, pre, model, i_orb):
    """Field lines within 1e-9 (CUDA's sin / atan2 against glibc's), the
    normals within 1e-12 of the reference's values."""
    from oracle import postproc_ref as ppr
    d = load("postproc")
    Z = d[f"{pre}_Z"]
    si = d[f"{pre}_si"].ravel()
    zn = Z[0] if model >= 0 else Z[0] + 1j * Z[1]
    nu, n = ppr.continuous_context(zn, si, 3 if model == 3 else 2, 1000.)
    k, phi = ppr.fieldlines_params(int(d["fl_n_iter"]), float(d["fl_swirl"]),
                                   float(d["fl_endpoint_k"]))
    z = Z[i_orb] if model >= 0 else Z[i_orb] + 1j * Z[i_orb + 1]
    fl = ctx.fieldlines(model=model, c=d[f"{pre}_cpt"], z=z, nu_frac=nu, n=n, k=k, phi=phi,
                        is_backward=True, backshift=int(d["backshift"]))
    esc = np.isfinite(nu)
    np.testing.assert_allclose(fl[esc], d[f"{pre}_fl"][esc], rtol=0, atol=1e-9)
    if model >= 0:
        nv = ctx.normal(kind=0, zn=zn, dzndc=Z[2])
    else:
        nv = ctx.normal(kind=2, zn=zn, dzndc=Z[2:6])
    np.testing.assert_allclose(nv.real, d[f"{pre}_dn_x"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(nv.imag, d[f"{pre}_dn_y"], rtol=0, atol=1e-12)
    if pre == "m2":
        mil = ctx.normal(kind=1, zn=zn, dzndc=Z[2], d2zndc2=Z[3])
        np.testing.assert_allclose(mil.real, d["m2_mil_x"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(mil.imag, d["m2_mil_y"], rtol=0, atol=1e-12)
        # the skew is undone on the normal (core.py:3147-3158)
        skew = np.array([[1.1, 0.2], [-0.3, 0.9]])
        nvs = ctx.normal(kind=0, zn=zn, dzndc=Z[2], skew=skew)
        np.testing.assert_allclose(nvs, ppr.normal(0, zn, dzndc=Z[2], skew=skew), atol=1e-12)


# ---------------------------------------------------------------------------
# Expmap projection in the kernels (fsg_tile.proj): CUDA's exp / sin / cos
# place a pixel's c within an ulp or two of numpy's, so chaotic pixels may
# take another count; the rest agree to 1e-6
# ---------------------------------------------------------------------------
def _expmap(hmax, orient, xy_ratio):
    from fractalshades_gb300 import projection as fsproj
    p = fsproj.Expmap(hmin=0., hmax=hmax, orientation=orient)
    p.xy_ratio = xy_ratio
    p.make_impl()
    return p


@pytest.mark.parametrize("key", ["h", "v"])
def test_std_expmap_vs_reference(ctx, key):
    from fractalshades_gb300 import _native as nat
    d = load("std_expmap")
    p = _expmap(4., {"h": "horizontal", "v": "vertical"}[key], float(d[f"{key}_xy_ratio"]))
    nx = int(d[f"{key}_nx"])
    xs, ys = axes(d[f"{key}_pix"], nx)
    n = xs.size * ys.size
    Z = np.zeros((3, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d[f"{key}_lin_mat"], Z=Z, stop_reason=sr,
                      stop_iter=si, center=-0.743643887037151 + 0.13182590420533j, dx=1e-4,
                      proj=p.kernel_params())
    ctx.std_tiles(nat.make_calc(max_iter=2000, M_divergence=1000., epsilon_stationnary=0.01),
                  [t])
    iter_agree(si, d[f"{key}_si"], frac=0.995, tol=2000)
    same = (si == d[f"{key}_si"]).ravel()
    rel_close(Z[0], d[f"{key}_Z"][0], 1e-6, same)


def _expmap_scale(d, hmoy):
    """dx * exp(h_moy) as the reference's Xrange product (perturbation.py:459-468)"""
    import mpmath
    m, e = mpmath.frexp(mpmath.exp(hmoy))
    return float(d["dx_m"]) * float(m), int(d["dx_e"]) + int(e)


def test_perturb_expmap_vs_reference(ctx):
    """Power-2 perturbation (FP64) under Expmap: derivative paths at the
    scale dx exp(h_moy), projected pixels, dzndc times the exit modifier."""
    from fractalshades_gb300 import _native as nat
    d = load("pert_m2_expmap")
    p = _expmap(5., "horizontal", 5. / (2. * np.pi))
    sm, se = _expmap_scale(d, 2.5)
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    ref = nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
                        calc_dzndc=True, scale_m=sm, scale_e=se, bla=True, kc=kc,
                        bla_eps=float(d["bla_eps"]))
    dz = ref.download("dzndc")
    assert np.array_equal(dz.view(np.uint64), d["dZndc"].view(np.uint64))
    xs = np.unique(d["pix"].real)
    ys = np.unique(d["pix"].imag)[::-1]
    assert np.array_equal((xs[None, :] + 1j * ys[:, None]).ravel(), d["pix"])
    n = d["pix"].size
    Z = np.zeros((2, n), dtype=np.complex128)
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, U=U, stop_reason=sr,
                      stop_iter=si, ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]), i_dzndc=1,
                      proj=p.kernel_params())
    ctx.perturb_tiles(nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                                    calc_dzndc=True, bla=True), [t])
    iter_agree(si, d["stop_iter"], frac=0.99, tol=6000)
    same = (si == d["stop_iter"]).ravel()
    rel_close(Z[0], d["Z"][0], 1e-6, same)
    rel_close(Z[1], d["Z"][1], 1e-6, same)


def test_perturb_bs_expmap_vs_reference(ctx):
    from fractalshades_gb300 import _native as nat
    d = load("pert_bs_expmap")
    fl = int(d["flavor"])
    xs = np.unique(d["pix"].real)
    ys = np.unique(d["pix"].imag)[::-1]
    assert np.array_equal((xs[None, :] + 1j * ys[:, None]).ravel(), d["pix"])
    p = _expmap(3., "vertical", 2. * np.pi / 3.)     # adjust_to_zoom, vertical h axis
    sm, se = _expmap_scale(d, 1.5)
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    ref = nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
                        flavor=fl, calc_dzndc=True, scale_m=sm, scale_e=se, bla=True, kc=kc,
                        bla_eps=float(d["bla_eps"]))
    n = d["pix"].size
    Z = np.zeros((6, n))
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], Z=Z, U=U, stop_reason=sr,
                      stop_iter=si, ref=ref, dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
                      drift_m=float(d["driftx_m"]), drift_e=int(d["driftx_e"]),
                      drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
                      proj=p.kernel_params())
    ctx.perturb_tiles(nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                                    flavor=fl, calc_dzndc=True, bla=True), [t])
    iter_agree(si, d["stop_iter"], frac=0.99, tol=5000)
    same = (si == d["stop_iter"]).ravel()
    for k in range(6):
        rel_close(Z[k], d["Z"][k], 1e-5, same)


@pytest.mark.parametrize("xr", [False, True])
def test_long_orbit_paths_scan_vs_oracle(ctx, xr):
    """Orbits above 8,192 points: the derivative paths come from the chunked
    scan (chunk composites, their prefix, then each chunk replayed in the
    reference's order); they agree with the oracle's sequential paths to
    1e-11 relative."""
    from fractalshades_gb300 import _native as nat
    rng = np.random.default_rng(7)
    n = 150_000
    r = 0.6 * np.sqrt(rng.random(n))
    Zn = r * np.exp(2j * np.pi * rng.random(n))
    Zn[0] = 0.
    ref = nat.Reference(ctx, Zn, div_iter=n, order=None, xr_paths=xr, calc_dzndc=True,
                        calc_dzndz=True, scale_m=0.5, scale_e=-30, bla=False)
    dzo = orc.dzndc_path_m2(Zn, n, 1 << 62, xr, 0.5, -30, None, None, None)
    dzzo = orc.dzndz_path_m2(Zn, n, xr, None, None, None)
    dz = ref.download("dzndc")
    dzz = ref.download("dzndz")
    if xr:
        for got, exp in ((dz, dzo), (dzz, dzzo)):
            a = got[0] * np.exp2(got[1].astype(np.float64) - exp[1])
            ok = np.abs(exp[0]) > 0
            np.testing.assert_allclose(a[ok], exp[0][ok], rtol=1e-11, atol=0)
            assert np.all(got[0][~ok] == 0)
    else:
        np.testing.assert_allclose(dz, dzo, rtol=1e-11, atol=1e-300)
        big = np.abs(dzzo) > 1e-250
        np.testing.assert_allclose(dzz[big], dzzo[big], rtol=1e-11, atol=0)
        assert np.all(np.abs(dzz[~big]) < 1e-240)


# ---------------------------------------------------------------------------
# Burning Ship on the Xrange branch (dx = 1e-305, reference-generated): the
# XR64 kernel against the reference's results, its Xrange Jacobian paths
# against the oracle's; the FP32 + exponent form on the same cases
BS_XR_CASES = ["pert_bs_xr_1", "pert_bs_xr_2", "pert_bs_xr_3", "pert_bs_xr_4", "pert_bs_xr_5",
               "pert_bs_xr_axis"]


def _bs_xr_ref(ctx, d):
    from fractalshades_gb300 import _native as nat
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    n_xr = int(d["xr_idx"].size)
    xr_m = np.concatenate([d["xr_xm"], d["xr_ym"]]) if n_xr else None
    xr_e = np.concatenate([d["xr_xe"], d["xr_ye"]]) if n_xr else None
    return nat.Reference(ctx, d["Zn"], div_iter=int(d["ref_div_iter"]), order=int(d["ref_order"]),
                         flavor=fl, xr_idx=d["xr_idx"] if n_xr else None, xr_m=xr_m, xr_e=xr_e,
                         xr_paths=True, calc_dzndc=True, scale_m=float(d["dx_m"]),
                         scale_e=int(d["dx_e"]), bla=True, kc=kc, bla_eps=float(d["bla_eps"]))


def _run_bs_ref(ctx, d, ref, mode, lin_scale=1.):
    from fractalshades_gb300 import _native as nat
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    Z = np.zeros((6, n))
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=np.asarray(d["lin_mat"]) * lin_scale, Z=Z, U=U,
                      stop_reason=sr, stop_iter=si, ref=ref, dx_m=float(d["dx_m"]),
                      dx_e=int(d["dx_e"]), drift_m=float(d["driftx_m"]),
                      drift_e=int(d["driftx_e"]), drifty_m=float(d["drifty_m"]),
                      drifty_e=int(d["drifty_e"]))
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                         flavor=int(d["flavor"]), calc_dzndc=True, bla=True, mode=mode)
    ctx.perturb_tiles(calc, [t])
    return Z, U, sr, si


def _xr_pairs(m, e):
    f, k = np.frexp(np.asarray(m, dtype=np.float64))
    return np.stack([f, np.where(f == 0., 0, np.asarray(e, dtype=np.int64) + k).astype(float)])


@pytest.mark.parametrize("case", BS_XR_CASES)
def test_perturb_bs_xr64_vs_reference(ctx, case):
    """The XR64 Burning Ship kernel (the reference's Xrange branch, -fmad=false,
    numba_xr operations in the reference's order): Jacobian paths equal to the
    oracle's, iteration counts, stop reasons and U equal to the reference's,
    Z within 1e-6 relative (bit for bit where it runs like the oracle)."""
    d = load(case)
    fl = int(d["flavor"])
    ref = _bs_xr_ref(ctx, d)
    m, e = ref.download("bs_xpaths")
    xr = (d["xr_idx"], d["xr_xm"], d["xr_xe"], d["xr_ym"], d["xr_ye"])
    pm, pe = orc.dzndc_path_bs_xr(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), fl,
                                  float(d["dx_m"]), int(d["dx_e"]), xr)
    for j in range(4):
        assert np.array_equal(_xr_pairs(m[j], e[j]), _xr_pairs(pm[j], pe[j])), j
    Z, U, sr, si = _run_bs_ref(ctx, d, ref, "xr64")
    ref.free()
    iter_agree(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    same = (si == d["stop_iter"]).ravel()
    for k in range(6):
        rel_close(Z[k], d["Z"][k], 1e-6, same)


@pytest.mark.parametrize("case", BS_XR_CASES)
def test_perturb_bs_fe32_vs_xrange_reference(ctx, case):
    """The FP32 + exponent Burning Ship form below the double range against
    the reference's Xrange branch: counts differ on at most
    FE32_SENSITIVITY_FACTOR x the case's FP32 sensitivity (the oracle's
    Xrange branch against itself with c moved by 2^-24) + FE32_ALLOWANCE."""
    d = load(case)
    fl = int(d["flavor"])
    ref = _bs_xr_ref(ctx, d)
    Z, U, sr, si = _run_bs_ref(ctx, d, ref, "fe32")
    ref.free()
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, _, st = orc.make_bla_bs(d["Zn"], fl, kc, float(d["bla_eps"]))
    xr = (d["xr_idx"], d["xr_xm"], d["xr_xe"], d["xr_ym"], d["xr_ye"])
    paths = orc.dzndc_path_bs_xr(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), fl,
                                 float(d["dx_m"]), int(d["dx_e"]), xr)
    _, _, _, sis = orc.perturb_bs_xr(
        d["pix"], Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]),
        ref_order=int(d["ref_order"]), lin_mat=np.asarray(d["lin_mat"]) * (1. + 2. ** -24),
        dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]), driftx_m=float(d["driftx_m"]),
        driftx_e=int(d["driftx_e"]), drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
        max_iter=int(d["max_iter"]), M=float(d["M"]), flavor=fl, bla=(Mb, rb, st),
        xpaths=paths, xr=xr)
    bar = FE32_SENSITIVITY_FACTOR * float(np.mean(sis != d["stop_iter"])) + FE32_ALLOWANCE
    assert float(np.mean(si != d["stop_iter"])) <= bar
    assert float(np.mean(sr != d["stop_reason"])) <= bar
