"""
Edge cases of the C-ABI and the kernels on the GPU: ragged and degenerate
tiles, more tiles than one launch takes, max_iter at its smallest,
first-iteration escapes, a period-1 reference, interruption, and the
refusals of malformed input (which never reach a kernel).
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

LIN = np.array([[1., -0.], [0., 1.]])


@pytest.fixture(scope="module")
def ctx():
    from fractalshades_gb300 import _native as nat
    c = nat.Context(0)
    yield c
    c.close()


def _std_tile(nat, xs, ys, center=-0.5 + 0j, dx=3.0, nZ=3):
    n = len(xs) * len(ys)
    Z = np.zeros((nZ, n), dtype=np.complex128)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=LIN, Z=Z, stop_reason=sr, stop_iter=si,
                      center=center, dx=dx)
    return t, (Z, sr, si)


def _check_std(xs, ys, out, max_iter, center=-0.5 + 0j, dx=3.0):
    pix = (np.asarray(xs)[None, :] + 1j * np.asarray(ys)[:, None]).ravel()
    Zo, sio, sro = orc.std_m2(pix, center, LIN, dx, max_iter, 1000., 0.01)
    Z, sr, si = out
    assert np.array_equal(si, sio) and np.array_equal(sr, sro)
    assert np.array_equal(Z.view(np.uint64), Zo.view(np.uint64))


def test_ragged_and_many_tiles(ctx):
    """1x1, 1xn, nx1, 3x7 and a 64x48 tile mixed, then 1500 tiles in one
    call (split into launches of at most 1024 tiles): bit-exact against the
    oracle."""
    from fractalshades_gb300 import _native as nat
    rng = np.random.default_rng(0)
    shapes = [(1, 1), (1, 17), (13, 1), (3, 7), (64, 48)] + [(1 + rng.integers(4), 1 + rng.integers(4))
                                                            for _ in range(1495)]
    tiles, outs, axes = [], [], []
    for nx, ny in shapes:
        xs = rng.random(nx) - 0.5
        ys = rng.random(ny) - 0.5
        t, out = _std_tile(nat, xs, ys)
        tiles.append(t); outs.append(out); axes.append((xs, ys))
    calc = nat.make_calc(max_iter=300, M_divergence=1000., epsilon_stationnary=0.01)
    ctx.std_tiles(calc, tiles)
    for (xs, ys), out in zip(axes, outs):
        _check_std(xs, ys, out, 300)


@pytest.mark.parametrize("max_iter", [1, 2, 3])
def test_smallest_max_iter(ctx, max_iter):
    """The standard loop never updates at n = max_iter (mandelbrot_M2.py:
    312-314): max_iter 1 leaves Z at 0 with stop_iter 1."""
    from fractalshades_gb300 import _native as nat
    xs = np.linspace(-0.5, 0.5, 9)
    ys = np.linspace(-0.5, 0.5, 7)
    t, out = _std_tile(nat, xs, ys)
    ctx.std_tiles(nat.make_calc(max_iter=max_iter, M_divergence=1000.,
                                epsilon_stationnary=0.01), [t])
    _check_std(xs, ys, out, max_iter)
    if max_iter == 1:
        assert np.all(out[2] == 1) and np.all(out[0] == 0)


def test_first_iteration_escape(ctx):
    """|c| beyond M escapes at n = 1."""
    from fractalshades_gb300 import _native as nat
    xs = np.linspace(-0.5, 0.5, 5)
    ys = np.linspace(-0.5, 0.5, 5)
    t, out = _std_tile(nat, xs, ys, center=5000. + 0j, dx=10.)
    ctx.std_tiles(nat.make_calc(max_iter=100, M_divergence=1000., epsilon_stationnary=0.01), [t])
    _check_std(xs, ys, out, 100, center=5000. + 0j, dx=10.)
    assert np.all(out[2] == 1) and np.all(out[1] == 1)


@pytest.mark.parametrize("mode", ["fp64", "xr64", "fe32"])
def test_period_one_reference(ctx, mode):
    """The reference orbit of c = 0 is 0 forever (order 1): every step is a
    wrap and a rebase; counts as the oracle's."""
    from fractalshades_gb300 import _native as nat
    Zn = np.zeros(2, dtype=np.complex128)
    xr = mode == "xr64"
    ref = nat.Reference(ctx, Zn, div_iter=1001, order=1, xr_paths=xr, calc_dzndc=True,
                        scale_m=0.5, scale_e=-6, bla=False)
    nx = 16
    xs = np.linspace(-0.5, 0.5, nx)
    ys = np.linspace(-0.5, 0.5, nx)
    n = nx * nx
    Z = np.zeros((2, n), dtype=np.complex128)
    U = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    si = np.zeros((1, n), dtype=np.int32)
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=LIN, Z=Z, U=U, stop_reason=sr, stop_iter=si,
                      ref=ref, dx_m=0.5, dx_e=3, drift_m=0j, drift_e=0, i_dzndc=1)
    ctx.perturb_tiles(nat.make_calc(max_iter=1000, M_divergence=1000., mode=mode,
                                    calc_dzndc=True, bla=False, xr_semantics=xr), [t])
    pix = (xs[None, :] + 1j * ys[:, None]).ravel()
    dz = orc.dzndc_path_m2(Zn, 1001, 1, xr, 0.5, -6)
    Zo, Uo, sro, sio = orc.perturb_m2(pix, Zn=Zn, ref_div_iter=1001, ref_order=1, lin_mat=LIN,
                                      dx_m=0.5, dx_e=3, drift_m=0j, drift_e=0, max_iter=1000,
                                      M=1000., eps_stat=0., xr_mode=xr, dZndc=dz)
    assert np.mean(si == sio) >= (1.0 if mode != "fe32" else 0.99)
    assert np.array_equal(sr, sro) or mode == "fe32"


def test_cancel_interrupts_every_loop(ctx):
    """fsg_cancel before a launch: the kernels claim no pixel and the call
    returns FSG_INTERRUPTED (core.py:2959-2960, perturbation.py:1042); after
    fsg_clear_cancel the same call completes."""
    from fractalshades_gb300 import _native as nat
    xs = np.linspace(-0.5, 0.5, 32)
    ys = np.linspace(-0.5, 0.5, 32)
    t, out = _std_tile(nat, xs, ys)
    calc = nat.make_calc(max_iter=300, M_divergence=1000., epsilon_stationnary=0.01)
    ctx.cancel()
    try:
        assert ctx.std_tiles(calc, [t]) == nat.FSG_INTERRUPTED
        # host buffers are left as they were (the reference stores nothing)
        assert np.all(out[2] == 0) and np.all(out[1] == -1)
    finally:
        ctx.clear_cancel()
    assert ctx.std_tiles(calc, [t]) == nat.FSG_OK
    _check_std(xs, ys, out, 300)


def test_malformed_input_is_refused(ctx):
    """Errors, not launches: zero-sized or pointer-less tiles, nZ too small,
    a perturbation tile without reference, max_iter out of range."""
    from fractalshades_gb300 import _native as nat
    xs = np.linspace(-0.5, 0.5, 4)
    ys = np.linspace(-0.5, 0.5, 4)
    calc = nat.make_calc(max_iter=10, M_divergence=1000.)
    t, out = _std_tile(nat, xs, ys, nZ=2)
    with pytest.raises(RuntimeError):
        ctx.std_tiles(calc, [t])                       # nZ < 3
    t, out = _std_tile(nat, xs, ys)
    t.nx = 0
    with pytest.raises(RuntimeError):
        ctx.std_tiles(calc, [t])                       # empty tile
    t, out = _std_tile(nat, xs, ys)
    t.Z = None
    with pytest.raises(RuntimeError):
        ctx.std_tiles(calc, [t])                       # no output
    t, out = _std_tile(nat, xs, ys)
    with pytest.raises(RuntimeError):
        ctx.perturb_tiles(calc, [t])                   # no reference
    with pytest.raises(RuntimeError):
        ctx.std_tiles(nat.make_calc(max_iter=0, M_divergence=1000.), [t])
    with pytest.raises(RuntimeError):
        ctx.std_tiles(nat.make_calc(max_iter=2 ** 31 - 1, M_divergence=1000.), [t])
    with pytest.raises(RuntimeError):
        ctx.std_tiles(calc, [])                        # no tiles


@pytest.mark.parametrize("kind", ["std", "fe32", "fp64"])
def test_iteration_budget_and_resubmission(ctx, kind):
    """fsg_calc.iter_budget: a launch stops claiming pixels once the pixels it
    finished have used the budget and returns FSG_BUDGET; the pixels it did
    not run keep stop_reason -1 (host buffers); submitting those again
    completes the image, bit for bit equal to one unbudgeted launch.  (The
    images hold more pixels than one wave of the persistent grid claims.)"""
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    if kind == "std":
        xs, ys = syn.image_axes(800, 600, 4. / 3.)
        ref, mk_calc = None, lambda b: nat.make_calc(max_iter=1000, M_divergence=1000.,
                                                     epsilon_stationnary=0.01, iter_budget=b)
        nZ, tile_kw, run = 3, dict(center=-0.5 + 0j, dx=3.0), ctx.std_tiles
    else:
        w = syn.seahorse_workload(nx=512)
        xs, ys = w.xs, w.ys
        ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, calc_dzndc=True,
                            scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
        mk_calc = lambda b: nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=kind,
                                          calc_dzndc=True, bla=True, iter_budget=b)
        nZ = 2
        tile_kw = dict(ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m,
                       drift_e=w.drift_e, i_dzndc=1)
        run = ctx.perturb_tiles
    pix = (np.asarray(xs)[None, :] + 1j * np.asarray(ys)[:, None]).ravel()
    n = pix.size

    def launch(p, budget):
        p = np.ascontiguousarray(p)
        Z = np.zeros((nZ, p.size), dtype=np.complex128)
        sr = -np.ones((1, p.size), dtype=np.int8)
        si = np.zeros((1, p.size), dtype=np.int32)
        t = nat.make_tile(pix=p, lin_mat=LIN, Z=Z, stop_reason=sr, stop_iter=si, **tile_kw)
        rc = run(mk_calc(budget), [t])
        return rc, Z, sr[0], si[0]

    rc, Zf, srf, sif = launch(pix, 0)
    assert rc == nat.FSG_OK
    # a fifth of the image's iterations; 1 % on the standard view, where
    # pixels escaping in a few iterations claim the rest of the image before
    # the interior ones, which carry most of the iterations, finish
    budget = int(sif.astype(np.int64).sum() // (100 if kind == "std" else 5))
    rc, Z1, sr1, si1 = launch(pix, budget)
    assert rc == nat.FSG_BUDGET
    left = np.flatnonzero(sr1 == -1)
    assert 0 < left.size < n
    # claims stop only once the finished pixels reach the budget
    assert si1[sr1 != -1].astype(np.int64).sum() >= budget
    rc, Z2, sr2, si2 = launch(pix[left], 0)
    assert rc == nat.FSG_OK
    Z1[:, left], sr1[left], si1[left] = Z2, sr2, si2
    assert np.array_equal(si1, sif) and np.array_equal(sr1, srf)
    assert np.array_equal(Z1.view(np.uint64), Zf.view(np.uint64))
    if ref is not None:
        ref.free()


@pytest.mark.parametrize("mode", ["fe32", "fp64"])
def test_streamed_host_call_equals_device_call(ctx, mode):
    """A host-buffer perturbation call of more than 2^21 pixels runs as
    consecutive launch segments whose outputs travel back while the next
    segment computes: the caller's arrays equal, bit for bit, those of one
    launch on device buffers; with an iteration budget the call returns
    FSG_BUDGET, the segments after the budget ran out leave stop_reason -1,
    and resubmitting those pixels completes the image exactly."""
    import torch
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    w = syn.seahorse_workload(nx=1536, max_iter=1500)
    n = w.nx * w.ny
    ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, calc_dzndc=True,
                        scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
    kw = dict(ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
              i_dzndc=1)

    def calc(budget=0):
        return nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=mode, calc_dzndc=True,
                             bla=True, iter_budget=budget)

    def host(xs, ys, budget=0, pix=None):
        m = pix.size if pix is not None else n
        Z = np.zeros((2, m), dtype=np.complex128)
        U = np.zeros(m, dtype=np.int32)
        sr = -np.ones(m, dtype=np.int8)
        si = np.zeros(m, dtype=np.int32)
        pot, dem = np.zeros(m), np.zeros(m)
        if pix is not None:
            t = nat.make_tile(pix=pix, lin_mat=LIN, Z=Z, U=U, stop_reason=sr, stop_iter=si,
                              potential=pot, dem=dem, **kw)
        else:
            t = nat.make_tile(xs=xs, ys=ys, lin_mat=LIN, Z=Z, U=U, stop_reason=sr,
                              stop_iter=si, potential=pot, dem=dem, **kw)
        rc = ctx.perturb_tiles(calc(budget), [t], nat.HOST)
        return rc, {"Z": Z, "U": U, "sr": sr, "si": si, "pot": pot, "dem": dem}

    dev = torch.device("cuda:0")
    f64 = dict(dtype=torch.float64, device=dev)
    xs, ys = torch.from_numpy(w.xs).to(dev), torch.from_numpy(w.ys).to(dev)
    d = {"Z": torch.zeros((2, n, 2), **f64), "U": torch.zeros(n, dtype=torch.int32, device=dev),
         "sr": torch.zeros(n, dtype=torch.int8, device=dev),
         "si": torch.zeros(n, dtype=torch.int32, device=dev),
         "pot": torch.zeros(n, **f64), "dem": torch.zeros(n, **f64)}
    t = nat.make_tile_ptrs(nx=w.nx, ny=w.ny, xs_ptr=xs.data_ptr(), ys_ptr=ys.data_ptr(),
                           lin_mat=LIN, Z_ptr=d["Z"].data_ptr(), nZ=2,
                           stop_reason_ptr=d["sr"].data_ptr(), stop_iter_ptr=d["si"].data_ptr(),
                           U_ptr=d["U"].data_ptr(), potential_ptr=d["pot"].data_ptr(),
                           dem_ptr=d["dem"].data_ptr(), **kw)
    assert ctx.perturb_tiles(calc(), [t], nat.DEVICE) == nat.FSG_OK
    ctx.sync()
    want = {k: v.cpu().numpy() for k, v in d.items()}
    want["Z"] = want["Z"].view(np.complex128).reshape(2, n)
    rc, got = host(w.xs, w.ys)
    assert rc == nat.FSG_OK
    for k in want:
        assert np.array_equal(got[k].view(np.uint8), want[k].view(np.uint8)), k
    # budget: a quarter of the image's iterations
    budget = int(want["si"].astype(np.int64).sum() // 4)
    rc, b = host(w.xs, w.ys, budget)
    assert rc == nat.FSG_BUDGET
    left = np.flatnonzero(b["sr"] == -1)
    assert 0 < left.size < n and left[-1] == n - 1
    pix = (np.asarray(w.xs)[None, :] + 1j * np.asarray(w.ys)[:, None]).ravel()[left]
    rc, r = host(None, None, pix=np.ascontiguousarray(pix))
    assert rc == nat.FSG_OK
    done = b["sr"] != -1
    for k in ("Z", "sr", "si"):
        a = b[k].copy()
        if k == "Z":
            a[:, left] = r[k]
            assert np.array_equal(a.view(np.uint8), want[k].view(np.uint8)), k
        else:
            a[left] = r[k]
            assert np.array_equal(a, want[k]), k
    assert done.sum() > 0
    ref.free()


@pytest.mark.parametrize("kind", ["std", "fe32", "fp64"])
def test_pinned_host_buffers_written_in_place(ctx, kind):
    """Page-locked host buffers are read and written in place by the kernels
    (no staging, no copy-back): the outputs equal the staged (pageable) call's
    bit for bit, and a Z row the kernel does not produce keeps the caller's
    values, where the staged call returns zeros."""
    import torch
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    w = syn.seahorse_workload(nx=256, max_iter=1500)
    n = w.nx * w.ny
    ref = None
    if kind == "std":
        calc = nat.make_calc(max_iter=1000, M_divergence=1000., epsilon_stationnary=0.01)
        kw = dict(center=-0.5 + 0j, dx=3.0)
        nZ, run, spare = 3, ctx.std_tiles, None
    else:
        ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, calc_dzndc=True,
                            scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
        calc = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=kind, calc_dzndc=True,
                             bla=True)
        kw = dict(ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
                  i_dzndc=1)
        nZ, run, spare = 3, ctx.perturb_tiles, 2          # row 2: no code writes it

    def arrays(pin):
        def mk(shape, dtype, fill):
            if pin:
                a = torch.empty(shape, dtype=dtype, pin_memory=True).numpy()
            else:
                a = np.empty(shape, dtype=torch.empty(0, dtype=dtype).numpy().dtype)
            a[...] = fill
            return a
        Zf = mk((nZ, n, 2), torch.float64, 7.0)
        d = {"Z": Zf.view(np.complex128).reshape(nZ, n),
             "sr": mk(n, torch.int8, -1), "si": mk(n, torch.int32, 0),
             "xs": mk(w.nx, torch.float64, 0.), "ys": mk(w.ny, torch.float64, 0.)}
        d["xs"][:] = w.xs
        d["ys"][:] = w.ys
        if kind != "std":
            d["pot"] = mk(n, torch.float64, 0.)
            d["dem"] = mk(n, torch.float64, 0.)
        return d

    out = {}
    for pin in (False, True):
        d = arrays(pin)
        extra = {} if kind == "std" else dict(potential=d["pot"], dem=d["dem"])
        t = nat.make_tile(xs=d["xs"], ys=d["ys"], lin_mat=LIN, Z=d["Z"], stop_reason=d["sr"],
                          stop_iter=d["si"], **kw, **extra)
        assert run(calc, [t], nat.HOST) == nat.FSG_OK
        out[pin] = d
    a, b = out[False], out[True]
    rows = [r for r in range(nZ) if r != spare]
    assert np.array_equal(a["Z"][rows].view(np.uint64), b["Z"][rows].view(np.uint64))
    for k in ("sr", "si", "pot", "dem"):
        if k in a:
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
    if spare is not None:
        assert np.all(a["Z"][spare] == 0)                 # staged: zeros
        assert np.all(b["Z"][spare] == 7.0 + 7.0j)        # in place: the caller's values
    if ref is not None:
        ref.free()


@pytest.mark.parametrize("mode", ["fe32", "fp64"])
def test_longest_first_claim_order(ctx, mode):
    """With claim_order "longest", a perturbation launch of 2^18 pixels or
    more claims its pixels longest first (a capped pre-pass over one pixel per
    8 x 8 block, then every pixel by its block's count): the outputs equal,
    bit for bit, those of the same image launched as row bands below that size
    (claimed in pixel order), and the statistics count the image's iterations
    once."""
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    w = syn.seahorse_workload(nx=640, max_iter=3000)
    ny = 480
    ys_all = np.ascontiguousarray(w.ys[(w.ny - ny) // 2:(w.ny - ny) // 2 + ny])
    ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, calc_dzndc=True,
                        scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
    calc = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=mode, calc_dzndc=True,
                         bla=True, claim_order="longest")
    kw = dict(ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
              i_dzndc=1)

    def run(ys):
        n = w.nx * ys.size
        o = {"Z": np.zeros((2, n), dtype=np.complex128), "sr": -np.ones(n, dtype=np.int8),
             "si": np.zeros(n, dtype=np.int32), "pot": np.zeros(n), "dem": np.zeros(n)}
        t = nat.make_tile(xs=w.xs, ys=ys, lin_mat=LIN, Z=o["Z"], stop_reason=o["sr"],
                          stop_iter=o["si"], potential=o["pot"], dem=o["dem"], **kw)
        assert ctx.perturb_tiles(calc, [t]) == nat.FSG_OK
        return o, ctx.stats()

    whole, st = run(ys_all)
    assert w.nx * ny >= 2 ** 18
    assert st["pixel_iters"] == int(whole["si"].astype(np.int64).sum())
    bands = [run(np.ascontiguousarray(ys_all[k:k + 120]))[0] for k in range(0, ny, 120)]
    for key in ("Z", "sr", "si", "pot", "dem"):
        b = np.concatenate([o[key] for o in bands], axis=-1)
        assert np.array_equal(whole[key].view(np.uint8), b.view(np.uint8)), key
    ref.free()
