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
    """A served request equals the same tile launched directly with its own
    reference (the bucketed derivative scale only rescales dzndc)."""
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    import mpmath
    req = _requests(centers)[1]
    got = _run(centers, [req], n_slots=1)[req.rid].result
    cen = centers[req.center]
    with mpmath.workdps(cen.dps):
        dx = mpmath.mpf(req.dx)
        view = cen.c + mpmath.mpc(*req.offset) * dx
    w = syn.prepare_m2(p=cen.p, dps=cen.dps, dx=req.dx, nx=req.side, max_iter=req.max_iter,
                       center=cen.c, offset=req.offset)
    ctx = nat.Context(0)
    ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, xr_paths=w.xr_mode,
                        calc_dzndc=True, scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc)
    n = req.side ** 2
    Z = np.zeros((2, n), dtype=np.complex128)
    U = np.zeros(n, dtype=np.int32)
    sr = np.zeros(n, dtype=np.int8)
    si = np.zeros(n, dtype=np.int32)
    t = nat.make_tile(xs=w.xs, ys=w.ys, lin_mat=np.array([[1., -0.], [0., 1.]]), Z=Z, U=U,
                      stop_reason=sr, stop_iter=si, ref=ref, dx_m=w.dx_m, dx_e=w.dx_e,
                      drift_m=w.drift_m, drift_e=w.drift_e, i_dzndc=1)
    ctx.perturb_tiles(nat.make_calc(max_iter=req.max_iter, M_divergence=1000., mode="fe32",
                                    calc_dzndc=True, bla=True, xr_semantics=w.xr_mode), [t])
    ref.free()
    ctx.close()
    # the BLA radii of the served request use kc rounded up to a power of two
    assert np.mean(got["stop_iter"] == si) >= 0.99
    same = got["stop_iter"] == si
    np.testing.assert_allclose(got["Z"][0][same], Z[0][same], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(np.abs(got["Z"][1][same]), np.abs(Z[1][same]), rtol=1e-4)


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
