"""
The serving queue of the C-ABI (fsg_serve_open / fsg_submit / fsg_poll) on
the GPU: requests of host-buffer tiles overlap on several slots and each
result equals the synchronous call's on the same tiles, bit for bit; the HBM
budget bounds what is staged at once and refuses a request larger than
itself; shortest-expected-work-first admission lets small requests overtake a
large queued one, and the response-ratio order lets a long-waiting one go
first; an interruption leaves the caller's arrays untouched.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIN = np.array([[1., -0.], [0., 1.]])


@pytest.fixture(scope="module")
def ctx():
    from fractalshades_gb300 import _native as nat
    c = nat.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def seahorse(ctx):
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    w = syn.seahorse_workload(nx=64, max_iter=3000)
    ref = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order, calc_dzndc=True,
                        scale_m=w.dx_m, scale_e=w.dx_e, bla=True, kc=w.kc, bla_eps=1e-6)
    yield w, ref
    ref.free()


def _perturb_tile(nat, w, ref, side, shift):
    """A side x side tile of the seahorse view moved by `shift` widths; the
    returned dict holds its outputs and (under "_in") the input arrays the
    tile points to."""
    from fractalshades_gb300 import synthetic as syn
    xs, ys = syn.image_axes(side, side)
    xs, ys = np.ascontiguousarray(xs + shift[0]), np.ascontiguousarray(ys + shift[1])
    n = side * side
    out = {"Z": np.zeros((2, n), dtype=np.complex128), "sr": -np.ones((1, n), dtype=np.int8),
           "si": np.zeros((1, n), dtype=np.int32), "pot": np.zeros(n), "dem": np.zeros(n)}
    keep = [xs, ys]
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=LIN, Z=out["Z"], stop_reason=out["sr"],
                      stop_iter=out["si"], ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m,
                      drift_e=w.drift_e, i_dzndc=1, potential=out["pot"], dem=out["dem"],
                      keep=keep)
    out["_in"] = keep
    return t, out


def _std_tile(nat, side):
    from fractalshades_gb300 import synthetic as syn
    xs, ys = syn.image_axes(side, side)
    n = side * side
    out = {"Z": np.zeros((3, n), dtype=np.complex128), "sr": -np.ones((1, n), dtype=np.int8),
           "si": np.zeros((1, n), dtype=np.int32)}
    keep = [xs, ys]
    t = nat.make_tile(xs=xs, ys=ys, lin_mat=LIN, Z=out["Z"], stop_reason=out["sr"],
                      stop_iter=out["si"], center=-0.5 + 0j, dx=3.0, keep=keep)
    out["_in"] = keep
    return t, out


def _same(a, b):
    for k in a:
        if not k.startswith("_"):
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def _wait(ctx, tickets, timeout=60.):
    rcs, order = {}, []
    t0 = time.perf_counter()
    while len(rcs) < len(tickets):
        for t in tickets:
            if t not in rcs:
                rc = ctx.poll(t)
                if rc is not None:
                    rcs[t] = rc
                    order.append(t)
        assert time.perf_counter() - t0 < timeout
        time.sleep(0.0005)
    return rcs, order


def test_queue_results_equal_synchronous_calls(ctx, seahorse):
    from fractalshades_gb300 import _native as nat
    w, ref = seahorse
    specs = [("fe32", 96, (0., 0.)), ("fp64", 64, (0.3, -0.2)), ("std", 80, None),
             ("fe32", 128, (-0.4, 0.1)), ("fp64", 48, (0.1, 0.4)), ("std", 40, None),
             ("fe32", 64, (0.2, 0.2))]

    def build(kind, side, shift):
        if kind == "std":
            t, out = _std_tile(nat, side)
            c = nat.make_calc(max_iter=1000, M_divergence=1000., epsilon_stationnary=0.01)
        else:
            t, out = _perturb_tile(nat, w, ref, side, shift)
            c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=kind, calc_dzndc=True,
                              bla=True)
        return t, out, c

    expected = []
    for kind, side, shift in specs:
        t, out, c = build(kind, side, shift)
        (ctx.std_tiles if kind == "std" else ctx.perturb_tiles)(c, [t])
        expected.append(out)
    ctx.serve_open(64 << 20, slots=3)
    try:
        tickets, outs = [], []
        for kind, side, shift in specs:
            t, out, c = build(kind, side, shift)
            tickets.append(ctx.submit(c, [t], keep=out))
            outs.append(out)
        rcs, _ = _wait(ctx, tickets)
        assert all(rc == nat.FSG_OK for rc in rcs.values())
        info = ctx.serve_info()
        assert info["queued"] == 0 and info["running"] == 0 and info["reserved_bytes"] == 0
        assert 0 < info["peak_reserved_bytes"] <= 64 << 20
    finally:
        ctx.serve_close()
    for a, b in zip(outs, expected):
        _same(a, b)


def test_queue_budget_binds_and_refuses_oversize(ctx, seahorse):
    from fractalshades_gb300 import _native as nat
    w, ref = seahorse
    c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode="fe32", calc_dzndc=True,
                      bla=True)
    # an upper bound of one 128^2 request's staged bytes (256-byte aligned parts)
    one = 128 * 128 * (16 * 2 + 4 + 1 + 4 + 8 + 8) + 2 * 128 * 8 + 8 * 256
    budget = int(1.6 * one)
    ctx.serve_open(budget, slots=4)
    try:
        keep, tickets = [], []
        for k in range(6):
            t, out = _perturb_tile(nat, w, ref, 128, (0.1 * k, 0.))
            keep.append(out)
            tickets.append(ctx.submit(c, [t], keep=out))
        rcs, _ = _wait(ctx, tickets)
        assert all(rc == nat.FSG_OK for rc in rcs.values())
        # one request fits the budget, two do not: never more than one staged
        assert ctx.serve_info()["peak_reserved_bytes"] <= budget
        t, _out = _perturb_tile(nat, w, ref, 256, (0., 0.))
        with pytest.raises(nat.GPUError):
            ctx.submit(c, [t], keep=_out)
    finally:
        ctx.serve_close()


def test_queue_shortest_first_overtakes(ctx, seahorse):
    from fractalshades_gb300 import _native as nat
    w, ref = seahorse
    c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode="fp64", calc_dzndc=True,
                      bla=True)
    ctx.serve_open(1 << 30, slots=1, order="shortest")
    try:
        keep, tickets = [], []
        for side, shift in ((128, (0., 0.)), (128, (0.5, 0.)), (32, (0., 0.5)), (32, (0.2, 0.2))):
            t, out = _perturb_tile(nat, w, ref, side, shift)
            keep.append(out)
            tickets.append(ctx.submit(c, [t], expected_work=float(side * side), keep=out))
        _, order = _wait(ctx, tickets)
        # the first large request started at once; the two small ones, queued
        # after the second large one, finish before it
        assert order[0] == tickets[0]
        assert order.index(tickets[2]) < order.index(tickets[1])
        assert order.index(tickets[3]) < order.index(tickets[1])
    finally:
        ctx.serve_close()


def test_queue_hrrn_ages_a_long_wait(ctx, seahorse):
    """FSG_SERVE_HRRN: a queued request that has waited long against its own
    expected service time goes before a shorter one that arrived late (the
    shortest-first order would take the short one)."""
    from fractalshades_gb300 import _native as nat
    w, ref = seahorse
    c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode="fp64", calc_dzndc=True,
                      bla=True)
    # the blocker's duration, from a synchronous call
    tb, outb = _perturb_tile(nat, w, ref, 1024, (0., 0.))
    t0 = time.perf_counter()
    ctx.perturb_tiles(c, [tb])
    dur = time.perf_counter() - t0
    ctx.serve_open(1 << 32, slots=1, order="hrrn")
    try:
        keep = []
        # a first request measures the work rate
        t, out = _perturb_tile(nat, w, ref, 32, (0., 0.))
        keep.append(out)
        first = ctx.submit(c, [t], expected_work=1.0, keep=out)
        _wait(ctx, [first])
        tb, outb = _perturb_tile(nat, w, ref, 1024, (0., 0.))
        tl, outl = _perturb_tile(nat, w, ref, 32, (0.5, 0.))
        ts, outs = _perturb_tile(nat, w, ref, 32, (0., 0.5))
        keep += [outb, outl, outs]
        blocker = ctx.submit(c, [tb], expected_work=1.0, keep=outb)
        long_ = ctx.submit(c, [tl], expected_work=2e-3, keep=outl)
        time.sleep(0.75 * dur)
        short = ctx.submit(c, [ts], expected_work=1e-3, keep=outs)
        _, order = _wait(ctx, [blocker, long_, short])
        # when the blocker retires, the long request has waited ~dur against
        # twice the short one's service time, the short one ~dur / 4
        assert order.index(long_) < order.index(short)
    finally:
        ctx.serve_close()


def test_queue_interruption_leaves_arrays_untouched(ctx, seahorse):
    from fractalshades_gb300 import _native as nat
    w, ref = seahorse
    c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode="fp64", calc_dzndc=True,
                      bla=True)
    ctx.serve_open(1 << 30, slots=2)
    try:
        ctx.cancel()
        keep, tickets = [], []
        for k in range(3):
            t, out = _perturb_tile(nat, w, ref, 64, (0.1 * k, 0.))
            keep.append(out)
            tickets.append(ctx.submit(c, [t], keep=out))
        rcs, _ = _wait(ctx, tickets)
        assert all(rc == nat.FSG_INTERRUPTED for rc in rcs.values())
        for out in keep:
            assert (out["sr"] == -1).all() and (out["si"] == 0).all()
    finally:
        ctx.clear_cancel()
        ctx.serve_close()


def test_queue_pinned_request_written_in_place(ctx, seahorse):
    """A request whose arrays are all page-locked stages nothing on the
    device (the kernels write it in place): its results equal the
    synchronous call's bit for bit, and the budget reserves no bytes for it."""
    import torch
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn
    w, ref = seahorse
    c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode="fe32", calc_dzndc=True,
                      bla=True)
    side = 96
    n = side * side
    xs, ys = syn.image_axes(side, side)

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0].copy()).dtype, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()
    xs_p, ys_p = pinned(xs), pinned(ys)
    Zf = torch.zeros((2, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    out = {"Z": Zf.view(np.complex128).reshape(2, n),
           "sr": pinned(-np.ones(n, dtype=np.int8)), "si": pinned(np.zeros(n, dtype=np.int32)),
           "pot": pinned(np.zeros(n)), "dem": pinned(np.zeros(n))}
    t = nat.make_tile(xs=xs_p, ys=ys_p, lin_mat=LIN, Z=out["Z"], stop_reason=out["sr"],
                      stop_iter=out["si"], ref=ref, dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m,
                      drift_e=w.drift_e, i_dzndc=1, potential=out["pot"], dem=out["dem"],
                      keep=[xs_p, ys_p])
    ts, outs = _perturb_tile(nat, w, ref, side, (0., 0.))
    assert ctx.perturb_tiles(c, [ts]) == nat.FSG_OK
    ctx.serve_open(1 << 20, slots=1, order="fifo")
    try:
        ticket = ctx.submit(c, [t], keep=out)
        assert ctx.serve_info()["reserved_bytes"] == 0
        rcs, _ = _wait(ctx, [ticket])
        assert rcs[ticket] == nat.FSG_OK
        assert ctx.serve_info()["peak_reserved_bytes"] == 0
    finally:
        ctx.serve_close()
    _same({k: v for k, v in outs.items() if not k.startswith("_")},
          {"Z": out["Z"], "sr": out["sr"].reshape(1, n), "si": out["si"].reshape(1, n),
           "pot": out["pot"], "dem": out["dem"]})
