"""
The host-side mirror of the reference API, without a GPU: decorators, pixel
grid, codes of the calc_std_div variants, reference-point preparation.
Same checks as the reference's tests/test_core.py (chunk indexing) and the
plug-in contract of tests/test_postproc.py (codes, keyword-only options).
"""
import mpmath
import numpy as np
import pytest

import fractalshades_gb300 as fs
import fractalshades_gb300.models as fsm
from fractalshades_gb300 import settings


def test_zoom_options_keyword_only_and_stored(tmp_path):
    f = fsm.Mandelbrot(str(tmp_path))
    with pytest.raises(TypeError):
        f.zoom(0.)
    f.zoom(x=-0.5, y=0.1, dx=3., nx=800, xy_ratio=4. / 3., theta_deg=0.)
    assert f.zoom_kwargs["nx"] == 800 and f.zoom_kwargs["has_skew"] is False
    assert f.x == -0.5 and f.ny == 600
    assert np.array_equal(f.lin_mat, np.array([[1., -0.], [0., 1.]]))


def test_calc_options_hook_receives_defaults(tmp_path):
    seen = {}

    class Probe(fsm.Mandelbrot):
        def calc_hook(self, calc_callable, calc_kwargs, return_dic):
            seen["name"] = calc_callable
            seen["kwargs"] = calc_kwargs
            seen["ret"] = return_dic

    f = Probe(str(tmp_path))
    f.zoom(x=-0.5, y=0., dx=3., nx=80, xy_ratio=1., theta_deg=0.)
    f.calc_std_div(calc_name="c", subset=None, max_iter=100, M_divergence=1000.)
    assert seen["name"] == "calc_std_div"
    assert seen["kwargs"]["epsilon_stationnary"] == 0.01
    assert set(seen["ret"]) == {"set_state", "initialize", "iterate"}
    with pytest.raises(TypeError):
        f.calc_std_div("c")


@pytest.mark.parametrize("nx,ratio", [(800, 4. / 3.), (451, 1.), (203, 0.7)])
def test_chunks_and_pixel_grid(tmp_path, nx, ratio):
    """tests/test_core.py chunk indexing; image_axes reproduces every tile's
    chunk_pixel_pos (core.py:1767-1830)."""
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=0., y=0., dx=1., nx=nx, xy_ratio=ratio, theta_deg=0.)
    xs, ys = f.image_axes()
    for rank, cs in enumerate(f.chunk_slices()):
        assert f.chunk_rank(cs) == rank
        assert f.chunk_from_rank(rank) == cs
        ix, ixx, iy, iyy = cs
        pix = f.chunk_pixel_pos(cs)
        assert np.array_equal(pix.real, np.broadcast_to(xs[ix:ixx], pix.shape))
        assert np.array_equal(pix.imag, np.broadcast_to(ys[iy:iyy, None], pix.shape))
    assert f.chunks_count == rank + 1


def _codes(f, **kw):
    ret = type(f).calc_std_div.__wrapped__(f, **kw)
    ns = type("S", (), {})()
    ret["set_state"]()(ns)
    return ns.codes, ret["iterate"]()


def test_perturbation_codes(tmp_path):
    f = fsm.Perturbation_mandelbrot(str(tmp_path))
    f.zoom(precision=30, x="-0.75", y="0.1", dx="1e-10", nx=64, xy_ratio=1., theta_deg=0.)
    base = dict(calc_name="c", subset=None, max_iter=1000, M_divergence=1000.,
                epsilon_stationnary=1e-3)
    codes, spec = _codes(f, **base)
    assert codes == (["zn", "dzndc"], ["ref_cycle_iter"], ["max_iter", "divergence", "stationnary"])
    assert spec.i_dzndc == 1 and spec.i_dzndz == -1 and spec.bla
    codes, spec = _codes(f, interior_detect=True, **base)
    assert codes[0] == ["zn", "dzndz", "dzndc"] and spec.i_dzndz == 1 and spec.i_dzndc == 2
    codes, spec = _codes(f, calc_dzndc=False, BLA_eps=None, **base)
    assert codes[0] == ["zn"] and not spec.bla
    # precision mode follows the reference's Xrange switch (H1)
    settings.precision_mode = "auto"
    assert spec.mode == "fp64"
    f.zoom(precision=400, x="-0.75", y="0.1", dx="1e-300", nx=64, xy_ratio=1., theta_deg=0.)
    assert f.xr_detect_activated          # mpf('1e-300') < 1e-300 (float)
    _, spec = _codes(f, **base)
    assert spec.mode == "xr64"


def test_bs_codes(tmp_path):
    f = fsm.Perturbation_burning_ship(str(tmp_path), flavor="Celtic")
    f.zoom(precision=30, x="-1.75", y="-0.03", dx="1e-8", nx=64, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(f, calc_name="c", subset=None, max_iter=1000, M_divergence=1000.)
    assert codes == (["xn", "yn", "dxnda", "dxndb", "dynda", "dyndb"], ["ref_cycle_iter"],
                     ["max_iter", "divergence"])
    assert spec.flavor == 4


def test_reference_point_search_and_path_data(tmp_path):
    """get_FP_orbit: ball method -> Newton -> orbit wrapped at the period;
    get_path_data and ref_point_kc (perturbation.py:166-194, 317-375, 651-854)."""
    from fractalshades_gb300 import synthetic as syn
    c = syn.find_nucleus(40, 80)
    f = fsm.Perturbation_mandelbrot(str(tmp_path))
    with mpmath.workdps(80):
        x, y = str(c.real + mpmath.mpf("3e-40")), str(c.imag)
    # zoom sets mpmath's working precision for the calculations that follow
    f.zoom(precision=80, x=x, y=y, dx="1e-38", nx=100, xy_ratio=1., theta_deg=0.)
    f.max_iter = 5000
    f.M_divergence = 1000.
    f.get_FP_orbit()
    assert f.FP_params["order"] == 40
    assert abs(f.FP_params["ref_point"] - c) < mpmath.mpf("1e-60")
    (Zn, has_xr, idx, xr, div_iter, order, drift, dx) = f.get_path_data()
    assert Zn.size == 40 and order == 40 and div_iter == 5001 and not has_xr
    z = mpmath.mpc(0)
    for k in range(1, 40):
        z = z * z + c
        assert Zn[k] == complex(float(z.real), float(z.imag))
    kc = f.ref_point_kc().to_standard()
    assert 1.1 * 0.5 * np.sqrt(2) * 1e-38 < kc < 1.1 * (0.5 * np.sqrt(2) + 0.4) * 1e-38
    # a second call reuses the stored orbit (ref_point_matching)
    assert f.ref_point_matching()


def _std_fractal(path, max_iter=100):
    f = fsm.Mandelbrot(str(path))
    f.zoom(x=-0.5, y=0.1, dx=3., nx=450, xy_ratio=1.5, theta_deg=0.)
    f.calc_std_div(calc_name="c", subset=None, max_iter=max_iter, M_divergence=1000.)
    return f


def test_raw_storage_layout_and_reuse(tmp_path):
    """The reference's on-disk layout (core.py:2125-2510): npy memory maps
    data/<calc>_<key>.arr in chunk-compressed order (chunks by rank, pixels of
    a chunk row-major, x fastest), the .report chunk table and the
    .fingerprint pickle; a second instance with the same parameters finds the
    stored results, another max_iter does not."""
    f = _std_fractal(tmp_path)
    data = f._calc_data["c"]
    assert data["need_new_mmap"]
    f.init_report_mmap("c")
    f.init_data_mmaps("c")
    data["need_new_mmap"] = False
    ny, nx = f.ny, f.nx
    n = nx * ny
    rng = np.random.default_rng(0)
    nZ, nU = len(f.codes[0]), len(f.codes[1])
    Z = rng.random((nZ, n)) + 1j * rng.random((nZ, n))
    U = rng.integers(0, 50, (nU, n)).astype(np.int32)
    sr = rng.integers(-1, 3, n).astype(np.int8)
    si = rng.integers(0, 100, n).astype(np.int32)
    f._store_image("c", {"Z": Z, "U": U, "stop_reason": sr, "stop_iter": si})
    for cs in f.chunk_slices():
        subset, c_pix, Zc, Uc, src, sic = f.reload_data(cs, "c")
        ix, ixx, iy, iyy = cs
        m = (ixx - ix) * (iyy - iy)
        assert subset is None
        assert np.array_equal(Zc, Z.reshape(nZ, ny, nx)[:, iy:iyy, ix:ixx].reshape(nZ, m))
        assert np.array_equal(sic[0], si.reshape(ny, nx)[iy:iyy, ix:ixx].ravel())
        assert np.array_equal(src[0], sr.reshape(ny, nx)[iy:iyy, ix:ixx].ravel())
        assert np.array_equal(c_pix, np.ravel(f.chunk_pixel_pos(cs)))
    arr = np.load(str(tmp_path / "data" / "c_Z.arr"), mmap_mode="r")
    assert arr.shape == (nZ, n) and arr.dtype == np.complex128
    items, report = f.reload_report("c", None)
    assert items == ["chunk1d_begin", "chunk1d_end", "chunk_pts", "done"]
    assert report[-1, 1] == n and np.all(report[:, 3] == 1)

    g = _std_fractal(tmp_path)
    assert not g._calc_data["c"]["need_new_mmap"]
    assert all(g.res_available("c", cs) for cs in g.chunk_slices())
    assert g.calc_raw("c") is None            # every tile done: nothing launched
    assert np.array_equal(g.get_raw("c", "stop_iter"), si.reshape(ny, nx))
    assert np.array_equal(g.get_raw("c", "zn"), Z[f.codes[0].index("zn")].reshape(ny, nx))

    h = _std_fractal(tmp_path, max_iter=200)
    assert h._calc_data["c"]["need_new_mmap"]         # calc_raw starts a new set
    assert h.reload_fingerprint("c")["calc_kwargs"]["max_iter"] == 200
    h.init_report_mmap("c")
    assert not h.res_available("c", next(h.chunk_slices()))


def test_reads_reference_written_ref_pt(tmp_path, monkeypatch):
    """data/ref_pt.dat as the reference writes it (perturbation.py:256-274:
    FP_params then Zn_path, Xrange values pickled as its Xrange_array record
    arrays) is read back, and its Xrange side table feeds get_path_data."""
    import pickle
    import sys
    import types
    from fractalshades_gb300.numpy_utils import xrange as fsx

    class Xrange_array(np.ndarray):
        pass
    Xrange_array.__module__ = "fractalshades.numpy_utils.xrange"
    Xrange_array.__qualname__ = "Xrange_array"
    for name in ("fractalshades", "fractalshades.numpy_utils", "fractalshades.numpy_utils.xrange"):
        monkeypatch.setitem(sys.modules, name, types.ModuleType(name))
    sys.modules["fractalshades.numpy_utils.xrange"].Xrange_array = Xrange_array
    rec = np.zeros((1,), dtype=fsx.get_xr_dtype(np.complex128))
    rec["mantissa"], rec["exp"] = 0.75 - 0.5j, -1200
    xr_val = rec.view(Xrange_array)
    with mpmath.workdps(30):
        FP_params = {"ref_point": mpmath.mpc("-1.75", "0.01"), "dps": 30, "order": 7,
                     "max_iter": 100, "FP_code": ["zn"], "partials": {}, "xr": {3: xr_val},
                     "div_iter": 101, "ref_orbit_len": 7, "init_kwargs": {}}
    Zn = (np.arange(7) * (0.1 + 0.2j)).astype(np.complex128)
    (tmp_path / "data").mkdir()
    with open(tmp_path / "data" / "ref_pt.dat", "wb") as fh:
        pickle.dump(FP_params, fh, pickle.HIGHEST_PROTOCOL)
        pickle.dump(Zn, fh, pickle.HIGHEST_PROTOCOL)
    for name in ("fractalshades", "fractalshades.numpy_utils", "fractalshades.numpy_utils.xrange"):
        monkeypatch.delitem(sys.modules, name)

    f = fsm.Perturbation_mandelbrot(str(tmp_path))
    params, path = f.reload_ref_point()
    assert params["order"] == 7 and np.array_equal(path, Zn)
    idx, m, e = fsx.xr_table(params["xr"])
    assert idx.tolist() == [3] and m[0] == 0.75 - 0.5j and e[0] == -1200


def test_power_n_models(tmp_path):
    """Mandelbrot_N / Perturbation_mandelbrot_N (models/mandelbrot_Mn.py):
    codes, the exponent carried to the GPU options, FP32 refused, the
    reference's find_nucleus refusal and the Julia size exponent."""
    f = fsm.Mandelbrot_N(str(tmp_path / "std"), 5)
    f.zoom(x=0., y=0., dx=3., nx=64, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(f, calc_name="c", subset=None, max_iter=100, M_divergence=1000.,
                         epsilon_stationnary=1e-3)
    assert codes[0] == ["zn", "dzndz", "dzndc"] and spec.nexp == 5
    assert spec.calc().nexp == 5
    g = fsm.Perturbation_mandelbrot_N(str(tmp_path / "pert"), 3)
    assert g.init_kwargs == {"directory": str(tmp_path / "pert"), "exponent": 3}
    g.zoom(precision=30, x="0.6428766799817589", y="0.2514544748796524", dx="1e-10", nx=64,
           xy_ratio=1., theta_deg=0.)
    base = dict(calc_name="c", subset=None, max_iter=1000, M_divergence=1000.,
                epsilon_stationnary=1e-3)
    codes, spec = _codes(g, interior_detect=True, **base)
    assert codes[0] == ["zn", "dzndz", "dzndc"] and spec.nexp == 3
    settings.precision_mode = "auto"
    assert spec.mode == "fp64" and spec.calc().nexp == 3
    settings.precision_mode = "fe32"
    try:
        with pytest.raises(ValueError):
            spec.mode
    finally:
        settings.precision_mode = "auto"
    with pytest.raises(NotImplementedError):
        g.find_nucleus(g.x + 1j * g.y, 10, 1e-12)
    c0 = mpmath.mpc("0.64287667998175895118", "0.25145447487965245909")
    size, julia = g._nucleus_size_estimate(c0, 10)
    assert abs(julia - size ** (8. / 9.)) < 1e-12 * julia
    with pytest.raises(ValueError):
        fsm.Perturbation_mandelbrot_N(str(tmp_path / "bad"), 1)


def test_orbit_and_d2_options_codes(tmp_path):
    """calc_orbit / backshift / calc_d2zndc2: the reference's code lists
    (mandelbrot_M2.py:107-124, 482-506, burning_ship.py:264-280, 1015-1035)
    and the rows the kernels write."""
    f = fsm.Mandelbrot(str(tmp_path / "a"))
    f.zoom(x=-0.5, y=0., dx=3., nx=64, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(f, calc_name="c", subset=None, max_iter=100, M_divergence=1000.,
                         epsilon_stationnary=1e-3, calc_d2zndc2=True, calc_orbit=True,
                         backshift=3)
    assert codes[0] == ["zn", "dzndz", "dzndc", "d2zndc2", "zn_orbit"]
    assert spec.nZ == 5 and spec.i_znorbit == 4 and spec.calc().backshift == 3
    assert spec.calc().calc_d2zndc2 == 1
    with pytest.raises(ValueError):
        _codes(f, calc_name="c", subset=None, max_iter=100, M_divergence=1000.,
               epsilon_stationnary=1e-3, calc_orbit=True, backshift=0)
    g = fsm.Perturbation_mandelbrot(str(tmp_path / "b"))
    g.zoom(precision=30, x="-0.75", y="0.1", dx="1e-10", nx=64, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(g, calc_name="c", subset=None, max_iter=1000, M_divergence=1000.,
                         epsilon_stationnary=1e-3, interior_detect=True, calc_orbit=True,
                         backshift=7)
    assert codes[0] == ["zn", "dzndz", "dzndc", "zn_orbit"] and spec.i_znorbit == 3
    assert spec.calc().backshift == 7
    settings.precision_mode = "fe32"
    try:
        with pytest.raises(ValueError):
            spec.mode
    finally:
        settings.precision_mode = "auto"
    h = fsm.Perturbation_burning_ship(str(tmp_path / "c"), flavor="Burning ship")
    h.zoom(precision=30, x="-1.75", y="-0.03", dx="1e-8", nx=64, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(h, calc_name="c", subset=None, max_iter=1000, M_divergence=1000.,
                         calc_orbit=True, backshift=2)
    assert codes[0][-2:] == ["xn_orbit", "yn_orbit"] and spec.i_znorbit == 6
    s = fsm.Burning_ship(str(tmp_path / "d"), flavor="Celtic")
    s.zoom(x=-0.5, y=-0.5, dx=3.5, nx=24, xy_ratio=1., theta_deg=0.)
    codes, spec = _codes(s, calc_name="c", subset=None, max_iter=100, M_divergence=1000.,
                         calc_orbit=True, backshift=2)
    assert spec.nZ == 8 and spec.i_znorbit == 6 and codes[0][6:] == ["xn_orbit", "yn_orbit"]


def test_std_cpt_matches_reference(tmp_path):
    """get_std_cpt (core.py:2781-2791): the pixel's c, bit for bit."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "postproc.npz"))
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.5, y=0., dx=3., nx=32, xy_ratio=1., theta_deg=0.)
    assert np.array_equal(f.get_std_cpt(d["m2_pix"]), d["m2_cpt"])
    xs, ys = f.image_axes()
    assert np.array_equal((xs[None, :] + 1j * ys[:, None]).ravel(), d["m2_pix"])


@pytest.mark.parametrize("chunk", ["full", "inner"])
@pytest.mark.parametrize("case,jitter,ssg", [("plain", False, None), ("ss3", False, 3),
                                             ("jit", 0.7, None), ("ss2_jit", 1.0, 2)])
def test_chunk_pixel_pos_matches_reference(tmp_path, chunk, case, jitter, ssg):
    """Supersampled and jittered grids (core.py:1767-1830), bit for bit."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "pixel_grids.npz"))
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.5, y=0., dx=3., nx=40, xy_ratio=1.5, theta_deg=0.)
    cs = (0, f.nx, 0, f.ny) if chunk == "full" else (8, 24, 4, 20)
    assert (f.nx, f.ny) == (int(d["nx"]), int(d["ny"]))
    got = f.chunk_pixel_pos(cs, jitter, ssg)
    assert np.array_equal(got, d[f"{chunk}_{case}"])


@pytest.mark.parametrize("orient,key", [("horizontal", "h"), ("vertical", "v")])
def test_expmap_zoom_and_pixel_c_match_reference(tmp_path, orient, key):
    """Expmap (projection.py:226-503): the zoom's adjusted nx / xy_ratio, the
    pixel grid and each pixel's c (core.py:2781-2791) as the reference's."""
    import os
    from fractalshades_gb300 import projection as fsproj
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "std_expmap.npz"))
    f = fsm.Mandelbrot(str(tmp_path))
    f.zoom(x=-0.743643887037151, y=0.13182590420533, dx=1e-4, nx=24, xy_ratio=1.,
           theta_deg=15., projection=fsproj.Expmap(hmin=0., hmax=4., orientation=orient))
    assert (f.nx, f.ny, f.xy_ratio) == (int(d[f"{key}_nx"]), int(d[f"{key}_ny"]),
                                        float(d[f"{key}_xy_ratio"]))
    assert np.array_equal(f.lin_mat, d[f"{key}_lin_mat"])
    xs, ys = f.image_axes()
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    assert np.array_equal(pix, d[f"{key}_pix"])
    np.testing.assert_allclose(f.get_std_cpt(pix), d[f"{key}_c"], rtol=1e-15, atol=0)
