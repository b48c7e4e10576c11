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
