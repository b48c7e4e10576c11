"""
Launch shapes on the GPU: every candidate shape of the autotuner gives the
same outputs bit for bit (pixels are independent; the shape only changes
which thread takes which pixel), shapes outside a kernel's launch bounds are
refused, and autotune returns and caches one of the candidates.
"""
import json

import numpy as np
import pytest

from tests.test_gpu_kernels import _ref_from_golden, axes, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from fractalshades_gb300 import _native as nat
    c = nat.Context(0)
    yield c
    c.close()


def _m2_case(ctx, mode):
    from fractalshades_gb300 import _native as nat
    d = load("pert_m2_cycle")
    ref = _ref_from_golden(ctx, d, False)
    nx = int(round(np.sqrt(d["pix"].size)))
    xs, ys = axes(d["pix"], nx)
    n = d["pix"].size
    interior = bool(d["interior"])
    nZ = 2 + int(interior)
    bufs = dict(Z=np.zeros((nZ, n), dtype=np.complex128), U=np.zeros((1, n), dtype=np.int32),
                stop_reason=-np.ones((1, n), dtype=np.int8),
                stop_iter=np.zeros((1, n), dtype=np.int32))
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=d["lin_mat"], ref=ref, dx_m=float(d["dx_m"]),
                      dx_e=int(d["dx_e"]), drift_m=complex(d["drift_m"]),
                      drift_e=int(d["drift_e"]), i_dzndz=1 if interior else -1,
                      i_dzndc=1 + int(interior), **bufs)
    calc = nat.make_calc(max_iter=int(d["max_iter"]), M_divergence=float(d["M"]),
                         epsilon_stationnary=float(d["eps_stat"]), mode=mode, calc_dzndc=True,
                         interior=interior, bla=True)
    return calc, t, bufs, ref


@pytest.mark.parametrize("mode", ["fe32", "fp64"])
def test_every_shape_gives_the_same_outputs(ctx, mode):
    from fractalshades_gb300 import tune
    calc, t, bufs, ref = _m2_case(ctx, mode)
    ctx.perturb_tiles(calc, [t])
    want = {k: v.copy() for k, v in bufs.items()}
    for block, ctas in tune.candidates(calc, True):
        for v in bufs.values():
            v[...] = 0
        ctx.perturb_tiles(tune._shaped(calc, block, ctas), [t])
        for k in want:
            assert np.array_equal(bufs[k], want[k]), (mode, block, ctas, k)


def test_shapes_outside_the_bounds_are_refused(ctx):
    from fractalshades_gb300 import tune
    calc, t, bufs, ref = _m2_case(ctx, "fe32")
    for block, ctas in ((256, 0), (48, 0), (-32, 0), (128, -1)):
        with pytest.raises(RuntimeError):
            ctx.perturb_tiles(tune._shaped(calc, block, ctas), [t])


def test_autotune_returns_a_candidate(ctx, tmp_path, monkeypatch):
    from fractalshades_gb300 import tune
    monkeypatch.setenv("FSG_TUNE_CACHE", str(tmp_path / "shapes.json"))
    calc, t, bufs, ref = _m2_case(ctx, "fe32")
    out = tune.autotune(ctx, calc, [t], perturb=True, repeats=1, device="dev")
    assert (out["block"], out["ctas_per_sm"]) in tune.candidates(calc, True)
    assert len(out["table"]) == len(tune.candidates(calc, True))
    assert all(e["kernel_ms"] > 0 for e in out["table"])
    data = json.loads((tmp_path / "shapes.json").read_text())
    assert data["dev|" + tune.kernel_kind(calc, True)]["block"] == out["block"]
