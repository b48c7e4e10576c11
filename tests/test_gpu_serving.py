"""
Serving loop (fractalshades_gb300/serving.py) on the GPU: continuous
batching over several slots, HBM-budget admission, reference cache, and the
determinism contract -- each request's result is the same alone and in a mix.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def centers():
    from fractalshades_gb300 import serving as srv
    return [srv.make_center(p, 120, 4000) for p in (37, 53)]


def _requests(centers):
    from fractalshades_gb300 import serving as srv
    reqs = [
        srv.Request(rid=0, center=0, side=64, dx="3e-20", offset=(0.02, -0.03), max_iter=4000),
        srv.Request(rid=1, center=1, side=96, dx="1e-45", offset=(-0.05, 0.01), max_iter=4000),
        srv.Request(rid=2, center=0, side=48, dx="2e-8", offset=(0.3, 0.2), max_iter=4000),
        srv.Request(rid=3, center=1, side=80, dx="5e-30", offset=(0.0, 0.07), max_iter=4000),
    ]
    return reqs


def _run(centers, reqs, **kw):
    from fractalshades_gb300 import serving as srv
    server = srv.TileServer(centers, **kw)
    try:
        done = server.run(reqs, realtime=False, timeout=120)
    finally:
        server.close()
    return {r.rid: r for r in done}


def test_alone_and_mixed_results_are_identical(centers):
    alone = {}
    for r in _requests(centers):
        alone.update(_run(centers, [r], n_slots=1))
    mixed = _run(centers, _requests(centers), n_slots=2, max_batch_pixels=1 << 20)
    assert set(mixed) == set(alone)
    for rid in alone:
        a, m = alone[rid].result, mixed[rid].result
        for k in a:
            assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(m[k]).view(np.uint8)), (rid, k)


def test_results_match_a_single_tile_launch(centers):
    """A served request equals, bit for bit, the same tile launched directly
    with a reference built the way the server builds its own: BLA radii from
    kc rounded up to its bucket (TileServer.kc_bucket) and the derivative
    paths at the bucketed scale 2^(e - 1), the tile's dzndc unit set with
    fsg_tile.dzndc_scale_e."""
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import serving as srv
    from fractalshades_gb300 import synthetic as syn
    from fractalshades_gb300.numpy_utils import xrange as fsx
    import mpmath
    req = _requests(centers)[1]
    got = _run(centers, [req], n_slots=1)[req.rid].result
    cen = centers[req.center]
    w = syn.prepare_m2(p=cen.p, dps=cen.dps, dx=req.dx, nx=req.side, max_iter=req.max_iter,
                       center=cen.c, offset=req.offset)
    with mpmath.workdps(cen.dps):
        dx = mpmath.mpf(req.dx)
        half = dx / 2
        shift = -mpmath.mpc(*req.offset) * dx
        kc = max(abs(shift - mpmath.mpc(sx * half, sy * half))
                 for sx in (1, -1) for sy in (1, -1)) * mpmath.mpf(1.1)
    kc_b = srv.TileServer.kc_bucket(fsx.mpf_to_Xrange(kc))
    ctx = nat.Context(0)
    has_xr = cen.xr_idx.size > 0
    ref = nat.Reference(ctx, cen.Zn, div_iter=req.max_iter + 1, order=cen.p,
                        xr_idx=cen.xr_idx if has_xr else None,
                        xr_m=cen.xr_m if has_xr else None, xr_e=cen.xr_e if has_xr else None,
                        xr_paths=w.xr_mode, calc_dzndc=True, scale_m=0.5, scale_e=1, bla=True,
                        kc=kc_b)
    n = req.side ** 2
    Z = np.zeros((2, n), dtype=np.complex128)
    U = np.zeros(n, dtype=np.int32)
    sr = np.zeros(n, dtype=np.int8)
    si = np.zeros(n, dtype=np.int32)
    t = nat.make_tile(xs=w.xs, ys=w.ys, lin_mat=np.array([[1., -0.], [0., 1.]]), Z=Z, U=U,
                      stop_reason=sr, stop_iter=si, ref=ref, dx_m=w.dx_m, dx_e=w.dx_e,
                      drift_m=w.drift_m, drift_e=w.drift_e, i_dzndc=1,
                      dzndc_scale_e=w.dx_e - 1)
    ctx.perturb_tiles(nat.make_calc(max_iter=req.max_iter, M_divergence=1000., mode="fe32",
                                    calc_dzndc=True, bla=True, xr_semantics=w.xr_mode), [t])
    ref.free()
    ctx.close()
    # the server's rescale of dzndc from the bucket scale to dx
    Z.view(np.float64).reshape(2, n, 2)[1] *= 2.0 * w.dx_m
    np.testing.assert_array_equal(got["stop_iter"], si)
    np.testing.assert_array_equal(got["stop_reason"], sr)
    assert np.array_equal(got["Z"].view(np.uint8), Z.view(np.uint8))


def test_hbm_budget_admission(centers):
    """With a budget that fits one request at a time, requests still all
    complete, and the reserved memory never exceeds the budget."""
    from fractalshades_gb300 import serving as srv
    reqs = _requests(centers)
    budget = max(r.side ** 2 for r in reqs) * srv.BYTES_PER_PIXEL + 8 * 2 ** 20
    from fractalshades_gb300 import serving
    server = serving.TileServer(centers, hbm_budget=budget, n_slots=3)
    try:
        done = server.run(reqs, realtime=False, timeout=120)
        assert len(done) == len(reqs)
        assert server.max_reserved <= budget
    finally:
        server.close()
