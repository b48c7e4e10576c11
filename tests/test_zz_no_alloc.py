"""
fsg_std_tiles_noalloc -- the allocation-free entry point for callers that
cannot call cudaMalloc (device memory reserved up front by another allocator,
or no implicit device synchronisation allowed inside a frame loop).  Called
through the C-ABI, on device buffers the test owns, twice in a row: each
result must equal the one of fsg_std_tiles (same kernel: bit-exact).

This file is collected last so that a run stopping at the first failure has
run every other test first; it passes alone in a fresh process as well as
after the others (the first call on the device does the set-up).
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_case(torch, dev, nx, ny, flavor):
    n = nx * ny
    kx, ky = 0.5 / (nx - 1), 0.5 / (ny - 1)
    xs = np.linspace(kx * (-nx + 1), kx * (nx - 1), nx)
    ys = -np.linspace(ky * (-ny + 1), ky * (ny - 1), ny)
    nZ = 3 if flavor == 0 else 6
    zw = 2 if flavor == 0 else 1          # complex128 as 2 doubles
    bufs = {
        "xs": torch.from_numpy(xs).to(dev), "ys": torch.from_numpy(ys).to(dev),
        "Z": torch.zeros((nZ, n * zw), dtype=torch.float64, device=dev),
        "sr": torch.zeros(n, dtype=torch.int8, device=dev),
        "si": torch.zeros(n, dtype=torch.int32, device=dev),
        "pot": torch.zeros(n, dtype=torch.float64, device=dev),
        "dem": torch.zeros(n, dtype=torch.float64, device=dev),
    }
    return bufs, nZ


def _tile(nat, b, nx, ny, nZ, center, dx):
    return nat.make_tile_ptrs(
        nx=nx, ny=ny, xs_ptr=b["xs"].data_ptr(), ys_ptr=b["ys"].data_ptr(),
        lin_mat=np.array([[1., -0.], [0., 1.]]), Z_ptr=b["Z"].data_ptr(), nZ=nZ,
        stop_reason_ptr=b["sr"].data_ptr(), stop_iter_ptr=b["si"].data_ptr(),
        center=center, dx=dx, potential_ptr=b["pot"].data_ptr(), dem_ptr=b["dem"].data_ptr())


def _snapshot(b):
    return {k: b[k].cpu().numpy().copy() for k in ("Z", "sr", "si", "pot", "dem")}


@pytest.mark.parametrize("flavor,center,dx", [(0, -0.5 + 0j, 3.0), (1, -0.5 - 0.5j, 3.5)])
def test_noalloc_matches_std_tiles_twice(flavor, center, dx):
    torch = pytest.importorskip("torch")
    from fractalshades_gb300 import _native as nat
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = nat.load()
    L.fsg_std_tiles_noalloc.argtypes = [ct.POINTER(nat.Calc), ct.POINTER(nat.Tile), ct.c_int32,
                                        ct.c_void_p]
    nx, ny = 320, 240
    calc = nat.make_calc(max_iter=600, M_divergence=1000., epsilon_stationnary=0.01,
                         flavor=flavor)

    # the existing entry point, with its context, on the same device buffers
    b, nZ = _device_case(torch, dev, nx, ny, flavor)
    ctx = nat.Context(0)
    stream = torch.cuda.current_stream(dev)
    ctx.std_tiles(calc, [_tile(nat, b, nx, ny, nZ, center, dx)], nat.DEVICE)
    ctx.sync()
    expected = _snapshot(b)
    ctx.close()

    tiles = (nat.Tile * 1)(_tile(nat, b, nx, ny, nZ, center, dx))
    for call in range(2):
        for k in ("Z", "pot", "dem"):
            b[k].fill_(-7.0)
        b["sr"].fill_(99)
        b["si"].fill_(-1)
        torch.cuda.synchronize(dev)
        rc = L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, 1, ct.c_void_p(stream.cuda_stream))
        assert rc == nat.FSG_OK, f"call {call}: code {rc}"
        torch.cuda.synchronize(dev)
        got = _snapshot(b)
        for k in expected:
            assert np.array_equal(got[k].view(np.uint8), expected[k].view(np.uint8)), (call, k)


def test_noalloc_several_tiles_pix_and_power_n():
    """Three tiles of different sizes in one call -- a rectangle, an explicit
    list of pixel positions (pix) and a smaller rectangle -- on the power-3
    model: the per-tile offsets, the pix input and the power-n kernel all go
    through the allocation-free path; bit-exact against fsg_std_tiles, twice."""
    torch = pytest.importorskip("torch")
    from fractalshades_gb300 import _native as nat
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = nat.load()
    L.fsg_std_tiles_noalloc.argtypes = [ct.POINTER(nat.Calc), ct.POINTER(nat.Tile), ct.c_int32,
                                        ct.c_void_p]
    calc = nat.make_calc(max_iter=500, M_divergence=1000., epsilon_stationnary=0.01, nexp=3)
    a, nza = _device_case(torch, dev, 200, 150, 0)
    c, nzc = _device_case(torch, dev, 64, 48, 0)
    rng = np.random.default_rng(11)
    npix = 777
    pos = (rng.uniform(-0.5, 0.5, npix) + 1j * rng.uniform(-0.5, 0.5, npix)).astype(np.complex128)
    pix = torch.from_numpy(pos.view(np.float64).copy()).to(dev)
    b = {"Z": torch.zeros((3, 2 * npix), dtype=torch.float64, device=dev),
         "sr": torch.zeros(npix, dtype=torch.int8, device=dev),
         "si": torch.zeros(npix, dtype=torch.int32, device=dev),
         "pot": torch.zeros(npix, dtype=torch.float64, device=dev),
         "dem": torch.zeros(npix, dtype=torch.float64, device=dev)}
    tb = _tile(nat, dict(b, xs=pix, ys=pix), npix, 1, 3, -0.2 + 0.1j, 2.5)
    tb.xs, tb.ys, tb.pix = None, None, pix.data_ptr()
    tiles_py = [_tile(nat, a, 200, 150, nza, 0.1 + 0.2j, 2.8), tb,
                _tile(nat, c, 64, 48, nzc, -0.6 + 0.6j, 0.3)]
    bufs = [a, b, c]

    ctx = nat.Context(0)
    ctx.std_tiles(calc, tiles_py, nat.DEVICE)
    ctx.sync()
    expected = [_snapshot(x) for x in bufs]
    ctx.close()
    assert any((e["sr"] == 1).any() and (e["sr"] != 1).any() for e in expected)

    stream = torch.cuda.current_stream(dev)
    tiles = (nat.Tile * 3)(*tiles_py)
    for call in range(2):
        for x in bufs:
            for k in ("Z", "pot", "dem"):
                x[k].fill_(-7.0)
            x["sr"].fill_(99)
            x["si"].fill_(-1)
        torch.cuda.synchronize(dev)
        rc = L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, 3, ct.c_void_p(stream.cuda_stream))
        assert rc == nat.FSG_OK, f"call {call}: code {rc}"
        torch.cuda.synchronize(dev)
        for i, x in enumerate(bufs):
            got = _snapshot(x)
            for k in expected[i]:
                assert np.array_equal(got[k].view(np.uint8), expected[i][k].view(np.uint8)), \
                    (call, i, k)


def test_noalloc_max_iter_bound_matches_std_tiles():
    """Both entry points accept max_iter up to FSG_MAX_ITER_LIMIT and refuse
    the next value."""
    torch = pytest.importorskip("torch")
    from fractalshades_gb300 import _native as nat
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = nat.load()
    L.fsg_std_tiles_noalloc.argtypes = [ct.POINTER(nat.Calc), ct.POINTER(nat.Tile), ct.c_int32,
                                        ct.c_void_p]
    b, nZ = _device_case(torch, dev, 16, 16, 0)
    t = _tile(nat, b, 16, 16, nZ, 20. + 20.j, 1.0)      # every pixel escapes at once
    tiles = (nat.Tile * 1)(t)
    stream = torch.cuda.current_stream(dev)
    ctx = nat.Context(0)
    try:
        for mi, ok in ((nat.FSG_MAX_ITER_LIMIT, True), (nat.FSG_MAX_ITER_LIMIT + 1, False)):
            calc = nat.make_calc(max_iter=mi, M_divergence=1000.)
            rc = L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, 1, ct.c_void_p(stream.cuda_stream))
            assert (rc == nat.FSG_OK) == ok, (mi, rc)
            rc2 = L.fsg_std_tiles(ctx.h, ct.byref(calc), tiles, 1, nat.DEVICE)
            assert (rc2 == nat.FSG_OK) == ok, (mi, rc2)
            torch.cuda.synchronize(dev)
            ctx.sync()
    finally:
        ctx.close()


def test_noalloc_rejects_too_many_tiles():
    pytest.importorskip("torch")
    from fractalshades_gb300 import _native as nat
    L = nat.load()
    L.fsg_std_tiles_noalloc.argtypes = [ct.POINTER(nat.Calc), ct.POINTER(nat.Tile), ct.c_int32,
                                        ct.c_void_p]
    calc = nat.make_calc(max_iter=10, M_divergence=1000.)
    n = nat.FSG_NOALLOC_MAX_TILES + 1
    tiles = (nat.Tile * n)()
    assert L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, n, None) == nat.FSG_ERR_LIMIT


def test_noalloc_captured_in_cuda_graph():
    """A frame loop's use of the allocation-free call: captured once into a
    CUDA graph (it allocates, copies and synchronises nothing: the upload
    kernel carries the descriptors), then replayed.  Every replay equals the
    eager call bit for bit, and a replay after the axes were rewritten in
    place renders the new view (the graph reads the buffers, not a copy)."""
    torch = pytest.importorskip("torch")
    from fractalshades_gb300 import _native as nat
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = nat.load()
    L.fsg_std_tiles_noalloc.argtypes = [ct.POINTER(nat.Calc), ct.POINTER(nat.Tile), ct.c_int32,
                                        ct.c_void_p]
    nx, ny = 256, 192
    calc = nat.make_calc(max_iter=500, M_divergence=1000., epsilon_stationnary=0.01)
    b, nZ = _device_case(torch, dev, nx, ny, 0)
    tiles = (nat.Tile * 1)(_tile(nat, b, nx, ny, nZ, -0.75 + 0.1j, 0.5))
    xs0, ys0 = b["xs"].clone(), b["ys"].clone()

    def junk():
        for k in ("Z", "pot", "dem"):
            b[k].fill_(-7.0)
        b["sr"].fill_(99)
        b["si"].fill_(-1)

    def eager():
        junk()
        s = torch.cuda.current_stream(dev)
        rc = L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, 1, ct.c_void_p(s.cuda_stream))
        assert rc == nat.FSG_OK
        torch.cuda.synchronize(dev)
        return _snapshot(b)

    # eager results of two views (the first call also does the set-up, before
    # any capture); the second view is the first zoomed 4x, axes scaled in place
    first = eager()
    b["xs"].mul_(0.25)
    b["ys"].mul_(0.25)
    second = eager()
    assert not np.array_equal(first["si"], second["si"])
    b["xs"].copy_(xs0)
    b["ys"].copy_(ys0)
    torch.cuda.synchronize(dev)

    g = torch.cuda.CUDAGraph()
    rcs = []
    with torch.cuda.graph(g):
        s = torch.cuda.current_stream(dev)
        rcs.append(L.fsg_std_tiles_noalloc(ct.byref(calc), tiles, 1, ct.c_void_p(s.cuda_stream)))
    assert rcs == [nat.FSG_OK]

    for expected, scale in ((first, 1.0), (first, 1.0), (second, 0.25)):
        b["xs"].copy_(xs0 * scale)
        b["ys"].copy_(ys0 * scale)
        junk()
        g.replay()
        torch.cuda.synchronize(dev)
        got = _snapshot(b)
        for k in expected:
            assert np.array_equal(got[k].view(np.uint8), expected[k].view(np.uint8)), (scale, k)
