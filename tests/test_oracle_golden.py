"""
Pin the CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py runs Fractalshades' hot-path functions as plain
Python).  Integer outputs (stop_iter, stop_reason, U) must match exactly;
floating point outputs are compared bit-for-bit where both sides evaluate the
same IEEE operations in the same order, else to the stated tolerance.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(G, name + ".npz"), allow_pickle=False)


# ---------------------------------------------------------------------------
def test_xrange_ops_vs_reference_host_class():
    d = load("xrange_ops")
    am, ae, bm, be = d["am"], d["ae"], d["bm"], d["be"]
    sm, se = orc.xr_binop("add", am, ae, bm, be)
    ref = d["add_m"] * np.exp2(d["add_e"].astype(float))
    got = sm * np.exp2(se.astype(float))
    np.testing.assert_allclose(got, ref, rtol=2e-16, atol=0)
    pm, pe = orc.xr_binop("mul", am, ae, bm, be)
    np.testing.assert_allclose(pm * np.exp2(pe.astype(float)),
                               d["mul_m"] * np.exp2(d["mul_e"].astype(float)),
                               rtol=4e-16, atol=0)
    qm, qe = orc.xr_binop("abs2", am, ae)
    np.testing.assert_allclose(qm.real * np.exp2(qe.astype(float)),
                               d["abs2_m"] * np.exp2(d["abs2_e"].astype(float)),
                               rtol=4e-16, atol=0)
    tm, _ = orc.xr_binop("to_standard", d["std_m"], d["std_e"])
    ok = np.isfinite(d["std_out"])
    assert np.array_equal(tm[ok], d["std_out"][ok])


def test_xrange_to_standard_edges():
    # underflow to 0, overflow to inf, exact powers of two
    m = np.array([1 + 1j, 0.75 - 0.5j, 1j, 0.5, 0j])
    e = np.array([-1080, 1030, -1022, 3, 17], dtype=np.int32)
    out, _ = orc.xr_binop("to_standard", m, e)
    assert out[0] == 0
    assert np.isinf(out[1].real)
    assert out[2] == 1j * 2.0 ** -1022
    assert out[3] == 4.0
    assert out[4] == 0


# ---------------------------------------------------------------------------
def test_std_m2_matches_reference_bit_exact():
    d = load("std_m2")
    Z, si, sr = orc.std_m2(d["pix"], complex(*d["center"]), d["lin_mat"],
                           float(d["dx"]), int(d["max_iter"]), float(d["M"]),
                           float(d["eps"]))
    assert np.array_equal(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    assert np.array_equal(Z.view(np.uint64), d["Z"].view(np.uint64))


def test_std_options_match_reference_bit_exact():
    """calc_d2zndc2 and calc_orbit (backshift 3 / 4) of the standard loops:
    power 2 (mandelbrot_M2.py:316-317, core.py:2965-3004), power 2 and 3 of
    Mandelbrot_N (mandelbrot_Mn.py:325-333, whose d2zndc2 recurrence uses
    dzndz) and Burning Ship flavors 1, 4 (core.py:3007-3056)."""
    d = load("std_opts")
    lin = d["lin_mat"]
    Z, si, sr = orc.std_m2(d["pix_m2"], -0.5 + 0j, lin, 3., 400, 1000., 0.01,
                           calc_d2zndc2=True, backshift=3)
    assert list(d["codes_m2"]) == ["zn", "dzndz", "dzndc", "d2zndc2", "zn_orbit"]
    assert np.array_equal(si, d["stop_iter_m2"]) and np.array_equal(sr, d["stop_reason_m2"])
    assert np.array_equal(Z.view(np.uint64), d["Z_m2"].view(np.uint64))
    for nexp in (2, 3):
        Z, si, sr = orc.std_mn(d[f"pix_mn{nexp}"], 0j, lin, 3., 300, 1000., 0.01, nexp,
                               calc_d2zndc2=True, backshift=4)
        assert np.array_equal(si, d[f"stop_iter_mn{nexp}"])
        assert np.array_equal(Z.view(np.uint64), d[f"Z_mn{nexp}"].view(np.uint64)), nexp
    for fl in (1, 4):
        Z, si, sr = orc.std_bs(d[f"pix_bs{fl}"], -0.5 - 0.5j, lin, 3.5, fl, 200, 1000.,
                               backshift=3)
        assert np.array_equal(si, d[f"stop_iter_bs{fl}"])
        assert np.array_equal(Z.view(np.uint64), d[f"Z_bs{fl}"].view(np.uint64)), fl


@pytest.mark.parametrize("nexp", [3, 4])
def test_std_mn_matches_reference_bit_exact(nexp):
    """Standard power-n loop (models/mandelbrot_Mn.py:317-355); the fixture's
    `zn ** (n - 1)` ran as numpy's complex integer power."""
    d = load("std_mn")
    Z, si, sr = orc.std_mn(d[f"pix_{nexp}"], complex(*d["center"]), d["lin_mat"],
                           float(d["dx"]), int(d["max_iter"]), float(d["M"]),
                           float(d["eps"]), nexp)
    assert np.array_equal(si, d[f"stop_iter_{nexp}"])
    assert np.array_equal(sr, d[f"stop_reason_{nexp}"])
    assert np.array_equal(Z.view(np.uint64), d[f"Z_{nexp}"].view(np.uint64))


@pytest.mark.parametrize("flavor", [1, 2, 3, 4, 5])
def test_std_bs_matches_reference_bit_exact(flavor):
    d = load("std_bs")
    Z, si, sr = orc.std_bs(d[f"pix_{flavor}"], complex(*d["center"]), d["lin_mat"],
                           float(d["dx"]), flavor, int(d["max_iter"]), float(d["M"]))
    assert np.array_equal(si, d[f"stop_iter_{flavor}"])
    assert np.array_equal(sr, d[f"stop_reason_{flavor}"])
    assert np.array_equal(Z.view(np.uint64), d[f"Z_{flavor}"].view(np.uint64))


# ---------------------------------------------------------------------------
def _nexp(d):
    """0 for the power-2 model, n for the power-n model's fixtures."""
    return int(d["nexp"]) if "nexp" in d.files else 0


def _backshift(d):
    """calc_orbit fixtures store the backshift (0: no orbit output)."""
    return int(d["backshift"]) if "backshift" in d.files else 0


def _pm2_inputs(d, recompute_tables):
    xr = bool(d["xr_mode"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    kw = dict(Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]),
              ref_order=int(d["ref_order"]), lin_mat=d["lin_mat"],
              dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
              drift_m=complex(d["drift_m"]), drift_e=int(d["drift_e"]),
              max_iter=int(d["max_iter"]), M=float(d["M"]),
              eps_stat=float(d["eps_stat"]), xr_mode=xr,
              interior=bool(d["interior"]), calc_dzndc=True,
              xr_idx=d["xr_idx"], xr_m=d["xr_m"], xr_e=d["xr_e"], nexp=_nexp(d),
              backshift=_backshift(d))
    if recompute_tables:
        Mb, rb, _, st = orc.make_bla_m2(d["Zn"], kc, float(d["bla_eps"]), _nexp(d))
        kw["bla"] = (Mb, rb, st)
        kw["dZndc"] = orc.dzndc_path_m2(
            d["Zn"], kw["ref_div_iter"], kw["ref_order"], xr, kw["dx_m"], kw["dx_e"],
            d["xr_idx"], d["xr_m"], d["xr_e"], nexp=_nexp(d))
        if kw["interior"]:
            kw["dZndz"] = orc.dzndz_path_m2(d["Zn"], kw["ref_div_iter"], xr,
                                            d["xr_idx"], d["xr_m"], d["xr_e"], nexp=_nexp(d))
    else:
        kw["bla"] = (d["M_bla"], d["r_bla"], int(d["stages_bla"]))
        if xr:
            kw["dZndc"] = (d["dZndc_m"], d["dZndc_e"])
            if kw["interior"]:
                kw["dZndz"] = (d["dZndz_m"], d["dZndz_e"])
        else:
            kw["dZndc"] = d["dZndc"]
            if kw["interior"]:
                kw["dZndz"] = d["dZndz"]
    return kw


def _xr_val(m, e, e_ref=None):
    """m * 2**(e - e_ref) with e_ref the largest exponent: values O(1), no
    underflow of the comparison."""
    e = np.asarray(e).astype(np.int64)
    if e_ref is None:
        e_ref = int(e.max()) if e.size else 0
    return m * np.exp2((e - e_ref).astype(float))


PERT_CASES = ["pert_m2_fp64", "pert_m2_cycle", "pert_m2_xr", "pert_m2_xr_div",
              "pert_mn3_cycle", "pert_mn3_div", "pert_mn4_xr",
              "pert_m2_orbit", "pert_m2_xr_orbit", "pert_mn3_orbit",
              # the period-2562 nucleus of the 2048^2 / 1e-300 workload at
              # max_iter 2e5 (12 BLA stages): the workload's own width
              # (Xrange branch, interior) and the boundary-straddling width
              # 1.6e-9 (FP64 branch, half the pixels escaping; and on the
              # Xrange branch, forced by settings.xrange_zoom_level)
              "pert_m2_p2562_1e300", "pert_m2_p2562_edge", "pert_m2_p2562_edge_xr"]


@pytest.mark.parametrize("case", PERT_CASES)
def test_orbit_tables_match_reference(case):
    d = load(case)
    xr = bool(d["xr_mode"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, bl, st = orc.make_bla_m2(d["Zn"], kc, float(d["bla_eps"]), _nexp(d))
    assert st == int(d["stages_bla"])
    assert np.array_equal(Mb.view(np.uint64), d["M_bla"].view(np.uint64))
    assert np.array_equal(rb.view(np.uint64), d["r_bla"].view(np.uint64))
    dz = orc.dzndc_path_m2(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), xr,
                           float(d["dx_m"]), int(d["dx_e"]), d["xr_idx"], d["xr_m"], d["xr_e"],
                           nexp=_nexp(d))
    if xr:
        # the golden Xrange paths come from the reference's numpy Xrange_array
        # class, whose rounding differs from numba_xr in the last bits
        eref = int(d["dZndc_e"].max())
        np.testing.assert_allclose(_xr_val(dz[0], dz[1], eref),
                                   _xr_val(d["dZndc_m"], d["dZndc_e"], eref),
                                   rtol=1e-13, atol=0)
    else:
        assert np.array_equal(dz.view(np.uint64), d["dZndc"].view(np.uint64))
    if bool(d["interior"]):
        dzz = orc.dzndz_path_m2(d["Zn"], int(d["ref_div_iter"]), xr,
                                d["xr_idx"], d["xr_m"], d["xr_e"], nexp=_nexp(d))
        if xr:
            eref = int(d["dZndz_e"].max())
            np.testing.assert_allclose(_xr_val(dzz[0], dzz[1], eref),
                                       _xr_val(d["dZndz_m"], d["dZndz_e"], eref),
                                       rtol=1e-13, atol=0)
        else:
            assert np.array_equal(dzz.view(np.uint64), d["dZndz"].view(np.uint64))


@pytest.mark.parametrize("case", PERT_CASES)
@pytest.mark.parametrize("recompute", [False, True])
def test_perturb_m2_matches_reference(case, recompute):
    d = load(case)
    kw = _pm2_inputs(d, recompute)
    Z, U, sr, si = orc.perturb_m2(d["pix"], **kw)
    assert np.array_equal(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    assert np.array_equal(U, d["U"])
    if not kw["xr_mode"]:
        assert np.array_equal(Z.view(np.uint64), d["Z"].view(np.uint64))
    elif case == "pert_m2_p2562_edge_xr":
        # the golden's Xrange values come from the reference's numpy host
        # class, whose last-bit rounding differs from numba_xr's; over the
        # 2.6e3 .. 3.3e4 chaotic iterations of the escaping pixels the
        # difference grows to ~2e-9 (counts and stop reasons stay equal)
        np.testing.assert_allclose(Z, d["Z"], rtol=1e-6, atol=0)
    else:
        np.testing.assert_allclose(Z, d["Z"], rtol=1e-13, atol=0)


def test_dzndz_carryover_is_erased_by_first_step():
    """The reference keeps the Xrange dzndz of the previous pixel in a tile
    (perturbation.py:1015, 1055-1060); the first full step multiplies it by
    (Z_0 + dz_0) = 0, so results do not depend on it."""
    d = load("pert_m2_xr")
    kw = _pm2_inputs(d, False)
    a = orc.perturb_m2(d["pix"], carryover=True, **kw)
    b = orc.perturb_m2(d["pix"], carryover=False, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("case", ["pert_bs_1", "pert_bs_4", "pert_bs_orbit", "pert_bs_2",
                                  "pert_bs_3", "pert_bs_4e", "pert_bs_5"])
def test_perturb_bs_matches_reference(case):
    d = load(case)
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, bl, st = orc.make_bla_bs(d["Zn"], fl, kc, float(d["bla_eps"]))
    assert st == int(d["stages_bla"])
    assert np.array_equal(Mb.view(np.uint64), d["M_bla"].view(np.uint64))
    assert np.array_equal(rb.view(np.uint64), d["r_bla"].view(np.uint64))
    scale = float(np.ldexp(d["dx_m"], d["dx_e"]))
    paths = orc.dzndc_path_bs(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), fl, scale)
    for got, k in zip(paths, ["dXa", "dXb", "dYa", "dYb"]):
        assert np.array_equal(got.view(np.uint64), d[k].view(np.uint64))
    Z, U, sr, si = orc.perturb_bs(
        d["pix"], Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]),
        ref_order=int(d["ref_order"]), lin_mat=d["lin_mat"],
        dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
        driftx_m=float(d["driftx_m"]), driftx_e=int(d["driftx_e"]),
        drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
        max_iter=int(d["max_iter"]), M=float(d["M"]), flavor=fl,
        bla=(Mb, rb, st), dpaths=paths, backshift=_backshift(d))
    assert np.array_equal(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    assert np.array_equal(U, d["U"])
    # bit for bit, NaN for NaN (a Hessian that overflows on the way out gives
    # inf - inf: NaN in both, with another sign bit in numpy than in C)
    nan = np.isnan(Z)
    assert np.array_equal(nan, np.isnan(d["Z"]))
    assert np.array_equal(Z[~nan].view(np.uint64), d["Z"][~nan].view(np.uint64))


# ---------------------------------------------------------------------------
# field lines and DEM normals (postproc.py:409-628), golden vectors from the
# reference's Postproc_batch
# ---------------------------------------------------------------------------
def _pp_inputs(d, pre):
    from oracle import postproc_ref as ppr
    Z = d[f"{pre}_Z"]
    si = d[f"{pre}_si"].ravel()
    zn = Z[0] if pre != "bs1" else Z[0] + 1j * Z[1]
    deg = 3 if pre == "mn3" else 2
    nu, n = ppr.continuous_context(zn, si, deg, 1000.)
    return Z, zn, nu, n


@pytest.mark.parametrize("pre,model,i_orb", [("m2", 0, 4), ("mn3", 3, 3), ("bs1", -1, 6)])
def test_postproc_oracle_matches_reference(pre, model, i_orb):
    from oracle import postproc_ref as ppr
    d = load("postproc")
    Z, zn, nu, n = _pp_inputs(d, pre)
    np.testing.assert_array_equal(n + nu, d[f"{pre}_cont"])     # Continuous_iter_pp
    k, phi = ppr.fieldlines_params(int(d["fl_n_iter"]), float(d["fl_swirl"]),
                                   float(d["fl_endpoint_k"]))
    z = Z[i_orb] if model >= 0 else Z[i_orb] + 1j * Z[i_orb + 1]
    fl = ppr.fieldlines(model, d[f"{pre}_cpt"], z, nu, n, k, phi, True, int(d["backshift"]))
    # escaped pixels: elsewhere the reference casts a NaN to int32, which
    # depends on the platform (INT_MIN on x86-64, 0 on aarch64)
    esc = np.isfinite(nu)
    assert esc.sum() > 500
    np.testing.assert_allclose(fl[esc], d[f"{pre}_fl"][esc], rtol=0, atol=1e-12)
    if model >= 0:
        nv = ppr.normal(0, zn, dzndc=Z[2])
    else:
        nv = ppr.normal(2, zn, jac=Z[2:6])
    np.testing.assert_array_equal(nv.real, d[f"{pre}_dn_x"])
    np.testing.assert_array_equal(nv.imag, d[f"{pre}_dn_y"])
    if pre == "m2":
        mil = ppr.normal(1, zn, dzndc=Z[2], d2zndc2=Z[3])
        np.testing.assert_allclose(mil.real, d["m2_mil_x"], rtol=0, atol=1e-15)
        np.testing.assert_allclose(mil.imag, d["m2_mil_y"], rtol=0, atol=1e-15)


# ---------------------------------------------------------------------------
# Expmap projection (projection.py:226-503): the oracle iterates the
# projected pixels; the perturbation loop's derivative modifier at exit
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("key", ["h", "v"])
def test_std_expmap_oracle_matches_reference(key):
    from fractalshades_gb300 import projection as fsproj
    d = load("std_expmap")
    proj = fsproj.Expmap(hmin=0., hmax=4., orientation={"h": "horizontal", "v": "vertical"}[key])
    proj.xy_ratio = float(d[f"{key}_xy_ratio"])
    proj.make_impl()
    fp = proj.f(d[f"{key}_pix"])
    Z, si, sr = orc.std_m2(fp, -0.743643887037151 + 0.13182590420533j, d[f"{key}_lin_mat"],
                           1e-4, 2000, 1000., 0.01)
    assert np.array_equal(si, d[f"{key}_si"]) and np.array_equal(sr, d[f"{key}_sr"])
    assert np.array_equal(Z.view(np.uint64), d[f"{key}_Z"].view(np.uint64))


def test_perturb_expmap_oracle_matches_reference():
    from fractalshades_gb300 import projection as fsproj
    d = load("pert_m2_expmap")
    proj = fsproj.Expmap(hmin=0., hmax=5.)
    proj.xy_ratio = 5. / (2. * np.pi)
    proj.make_impl()
    kw = _pm2_inputs(d, False)
    Z, U, sr, si = orc.perturb_m2(proj.f(d["pix"]), **kw)
    assert np.array_equal(si, d["stop_iter"]) and np.array_equal(U, d["U"])
    Z[-1] = Z[-1] * proj.dzndc_modifier(d["pix"])
    assert np.array_equal(Z.view(np.uint64), d["Z"].view(np.uint64))


# ---------------------------------------------------------------------------
# Burning Ship on the Xrange branch (dx = 1e-305): flavor 1 and 5 around
# diverging references, flavor 1 on the real axis (every orbit point in the
# side table)
BS_XR_CASES = ["pert_bs_xr_1", "pert_bs_xr_2", "pert_bs_xr_3", "pert_bs_xr_4", "pert_bs_xr_5",
               "pert_bs_xr_axis"]


def _xr_normal(m, e):
    """Records (m, e) as normalised (mantissa in [0.5, 1), exponent) pairs,
    zero as (0, 0): equal values give equal pairs."""
    f, k = np.frexp(np.asarray(m, dtype=np.float64))
    ex = np.where(f == 0., 0, np.asarray(e, dtype=np.int64) + k)
    return np.stack([f, ex.astype(np.float64)])


def bs_xr_inputs(d):
    fl = int(d["flavor"])
    kc = float(np.ldexp(d["kc_m"], d["kc_e"]))
    Mb, rb, _, st = orc.make_bla_bs(d["Zn"], fl, kc, float(d["bla_eps"]))
    xr = (d["xr_idx"], d["xr_xm"], d["xr_xe"], d["xr_ym"], d["xr_ye"])
    paths = orc.dzndc_path_bs_xr(d["Zn"], int(d["ref_div_iter"]), int(d["ref_order"]), fl,
                                 float(d["dx_m"]), int(d["dx_e"]), xr)
    return (Mb, rb, st), xr, paths


@pytest.mark.parametrize("case", BS_XR_CASES)
def test_perturb_bs_xr_matches_reference(case):
    d = load(case)
    assert int(d["xr_mode"]) == 1
    fl = int(d["flavor"])
    bla, xr, paths = bs_xr_inputs(d)
    assert bla[2] == int(d["stages_bla"])
    assert np.array_equal(bla[0].view(np.uint64), d["M_bla"].view(np.uint64))
    assert np.array_equal(bla[1].view(np.uint64), d["r_bla"].view(np.uint64))
    # the Xrange Jacobian paths: equal values (the reference's host class
    # normalises its records where numba_xr does not)
    for j, k in enumerate(["dXa", "dXb", "dYa", "dYb"]):
        assert np.array_equal(_xr_normal(paths[0][j], paths[1][j]),
                              _xr_normal(d[k + "_m"], d[k + "_e"])), k
    Z, U, sr, si = orc.perturb_bs_xr(
        d["pix"], Zn=d["Zn"], ref_div_iter=int(d["ref_div_iter"]),
        ref_order=int(d["ref_order"]), lin_mat=d["lin_mat"],
        dx_m=float(d["dx_m"]), dx_e=int(d["dx_e"]),
        driftx_m=float(d["driftx_m"]), driftx_e=int(d["driftx_e"]),
        drifty_m=float(d["drifty_m"]), drifty_e=int(d["drifty_e"]),
        max_iter=int(d["max_iter"]), M=float(d["M"]), flavor=fl, bla=bla, xpaths=paths, xr=xr)
    assert np.array_equal(si, d["stop_iter"])
    assert np.array_equal(sr, d["stop_reason"])
    assert np.array_equal(U, d["U"])
    nan = np.isnan(Z)
    assert np.array_equal(nan, np.isnan(d["Z"]))
    assert np.array_equal(Z[~nan].view(np.uint64), d["Z"][~nan].view(np.uint64))
