#!/usr/bin/env python
"""
Headline benchmark: pixel-iterations per second of the power-2 Mandelbrot
perturbation loop at dx = 1e-300, FP32-mantissa + int32-exponent deltas
versus the FP64 path, with the p50 / p99 latency of a stream of tiles.

Workload (seeded, synthetic): 2048 x 2048 pixels, width 1e-300, centred on
the nucleus of a period-p component (p ~ U[300, 3000], seed 2) found by
Newton at 400 digits; reference orbit at 400 digits, max_iter 200000, escape
radius 1e3, BLA eps 1e-6, outputs iteration count, smoothed potential and the
dzndc distance estimate.  One step = one launch over the whole image.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

Prints one JSON line.  With torchrun (N > 1) every rank renders its own
replica of the image (the pixels are independent) and rank 0 prints.
"""
import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pixel-iter/s at 1e-300 zoom, FP32+exp vs FP64 path; p50/p99 tile latency"
FLOPS_FULL = 35      # M2 perturbation step with dzndc (zn 17 + dzndc 18)
FLOPS_BLA = 23       # M2 BLA step with dzndc (17 + 6)
LIN = np.array([[1., -0.], [0., 1.]])


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--serving-requests", type=int, default=2000,
                    help="requests of the serving stream (0: skip)")
    ap.add_argument("--no-supplementary", action="store_true",
                    help="skip the standard-loop, 1e-1000 and Burning Ship configurations")
    ap.add_argument("--legs", default="std,deep,edge,seahorse,bs,bs_edge,model_api,host",
                    help="supplementary configurations to run (std, deep, edge, seahorse, bs, "
                         "bs_edge, model_api, host)")
    ap.add_argument("--bs-tiles", type=int, default=64,
                    help="Burning Ship tiles of the 64 to run (a smaller case for profiling)")
    ap.add_argument("--parity-pixels", type=int, default=262144,
                    help="seeded pixels of the headline image checked against the oracle "
                         "(0: skip)")
    ap.add_argument("--edge-nx", type=int, default=1024,
                    help="side of the boundary-straddling view (supplementary leg 'edge')")
    ap.add_argument("--no-headline", action="store_true",
                    help="run the supplementary legs only (a profiling case: no headline "
                         "steps, no bench line)")
    ap.add_argument("--bs-max-iter", type=int, default=50000,
                    help="max_iter of the Burning Ship configuration (its own, 5e4; FP64 runs "
                         "on a subset of the tiles)")
    return ap.parse_args()


def _serve_once(srv, centers, reqs, budget, order, device, n_slots=None):
    server = srv.TileServer(centers, hbm_budget=budget, n_slots=n_slots,
                            max_batch_pixels=8 * 2 ** 20, mode="fe32", device=device,
                            keep_results=False, order=order)
    slots = len(server.slots)
    t0 = time.perf_counter()
    try:
        done = server.run(reqs, realtime=True, timeout=600)
    finally:
        wall = time.perf_counter() - t0
        server.close()
    lat = np.array([(r.done - r.arrival) * 1e3 for r in done])
    sides = np.array([r.side for r in done])
    iters = float(sum(r.pixel_iters for r in done))

    def pct(a):
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)),
                "max": float(a.max()), "n": int(a.size)}
    return {"order": order, "slots": slots, "hbm_budget_gb": budget / 2 ** 30,
            "peak_reserved_gb": server.max_reserved / 2 ** 30, "requests": len(done),
            "wall_s": wall, "pixel_iters": iters, "pixel_iter_per_s": iters / wall,
            "latency_ms": pct(lat),
            "latency_ms_by_side": {str(k): pct(lat[sides == k]) for k in sorted(set(sides))},
            "results_to_host_gb": float(sum(r.side ** 2 for r in done) * srv.BYTES_PER_PIXEL
                                        / 1e9)}


def serving_leg(n_requests, device):
    """The serving stream: Poisson arrivals at 200/s, tiles of 256..2048
    squared, widths log-uniform in [1e-1000, 1e-10] around 8 seeded period-p
    nuclei (1100 digits), max_iter 2e5, FP32+exp deltas, 120 GB HBM budget --
    served in arrival order, shortest-expected-work first and by highest
    response ratio (shortest first, aged by waiting time); then the first 300
    requests under a 1 GB budget, where admission by HBM binds."""
    from fractalshades_gb300 import serving as srv
    rng = np.random.default_rng(5)
    periods = [int(p) for p in rng.integers(300, 3001, 8)]
    t0 = time.perf_counter()
    centers = [srv.make_center(p, 1100, 200000) for p in periods]
    setup_s = time.perf_counter() - t0
    out = {"rate_per_s": 200.0, "centers": periods, "center_setup_s": setup_s,
           "sides": [256, 512, 1024, 2048], "widths": "1e-1000 .. 1e-10 log-uniform",
           "slots_rule": "as many as the budget holds 8 Mpixel batches, at most 4 (one "
                         "persistent launch fills the GPU)"}
    for order in ("fifo", "shortest", "hrrn"):
        reqs = srv.request_stream(centers, n_requests, rate=200.0, seed=5)
        out[order] = _serve_once(srv, centers, reqs, 120 * 2 ** 30, order, device)
    reqs = srv.request_stream(centers, min(300, n_requests), rate=200.0, seed=5)
    out["fifo_1gb"] = _serve_once(srv, centers, reqs, 2 ** 30, "fifo", device)
    return out


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
def supplementary(ctx, nat, syn, torch, dev, stream, flush, bs_max_iter,
                  legs=("std", "deep", "edge", "seahorse", "bs", "bs_edge", "model_api", "host"),
                  bs_tiles=64,
                  edge_nx=1024,
                  parity_pixels=16384):
    """The other measured configurations, one launch each (kernel time from
    the library's CUDA events, L2 flushed before each launch):
    the standard loop (800 x 600, width 3) "std", the 1e-1000 zoom with
    interior detection (FE32 against XR64) "deep", the Burning Ship tiles in
    one launch "bs" (the first bs_tiles of the 64) and the host side at 1100
    digits "host"."""
    out = {}
    f64 = dict(dtype=torch.float64, device=dev)

    def timed(fn, k, warm):
        for _ in range(warm):
            fn()
        ks = []
        for _ in range(k):
            flush.fill_(1.0)
            stream.synchronize()
            fn()
            ks.append(ctx.stats()["kernel_ms"])
        return float(np.median(ks)), ctx.stats()

    if "std" in legs:
        # standard loop, bit-exact against the oracle in the GPU tests
        w1 = syn.config1_workload()
        n1 = w1.nx * w1.ny
        xs = torch.from_numpy(w1.xs).to(dev)
        ys = torch.from_numpy(w1.ys).to(dev)
        Z1 = torch.zeros((3, n1, 2), **f64)
        sr1 = torch.zeros(n1, dtype=torch.int8, device=dev)
        si1 = torch.zeros(n1, dtype=torch.int32, device=dev)
        pot1 = torch.zeros(n1, **f64)
        t1 = nat.make_tile_ptrs(nx=w1.nx, ny=w1.ny, xs_ptr=xs.data_ptr(), ys_ptr=ys.data_ptr(),
                                lin_mat=LIN, Z_ptr=Z1.data_ptr(), nZ=3,
                                stop_reason_ptr=sr1.data_ptr(), stop_iter_ptr=si1.data_ptr(),
                                center=w1.center, dx=w1.dx, i_dzndz=1, i_dzndc=2,
                                potential_ptr=pot1.data_ptr())
        c1 = nat.make_calc(max_iter=w1.max_iter, M_divergence=w1.M, epsilon_stationnary=w1.eps)
        kms, st = timed(lambda: ctx.std_tiles(c1, [t1], nat.DEVICE), 10, 3)
        out["standard_m2"] = {
            "workload": "standard power-2 Mandelbrot 800x600, centre -0.5, width 3, max_iter 1000, "
                        "M 1e3, eps 0.01 (interior detection, dzndc, potential)",
            "pixels": n1, "pixel_iters": int(st["pixel_iters"]), "kernel_ms": kms,
            "value": st["pixel_iters"] / (kms * 1e-3), "unit": "pixel-iter/s", "dtype": "f64",
            "parity": "bit-exact vs the oracle (tests/test_gpu_kernels.py)"}
        del Z1, sr1, si1, pot1

    if "deep" in legs:
        # 1e-1000, 4096^2, interior detection: FE32 against XR64
        w3 = syn.config3_workload()
        n3 = w3.nx * w3.ny
        ref3 = nat.Reference(ctx, w3.Zn, div_iter=w3.div_iter, order=w3.order, xr_idx=w3.xr_idx,
                             xr_m=w3.xr_m, xr_e=w3.xr_e, xr_paths=w3.xr_mode, calc_dzndc=True,
                             calc_dzndz=True, scale_m=w3.dx_m, scale_e=w3.dx_e, bla=True,
                             kc=w3.kc, bla_eps=1e-6)
        xs = torch.from_numpy(w3.xs).to(dev)
        ys = torch.from_numpy(w3.ys).to(dev)
        Z3 = torch.zeros((3, n3, 2), **f64)
        sr3 = torch.zeros(n3, dtype=torch.int8, device=dev)
        si3 = torch.zeros(n3, dtype=torch.int32, device=dev)
        t3 = nat.make_tile_ptrs(nx=w3.nx, ny=w3.ny, xs_ptr=xs.data_ptr(), ys_ptr=ys.data_ptr(),
                                lin_mat=LIN, Z_ptr=Z3.data_ptr(), nZ=3,
                                stop_reason_ptr=sr3.data_ptr(), stop_iter_ptr=si3.data_ptr(),
                                ref=ref3, dx_m=w3.dx_m, dx_e=w3.dx_e, drift_m=w3.drift_m,
                                drift_e=w3.drift_e, i_dzndz=1, i_dzndc=2)

        def c3(mode):
            return nat.make_calc(max_iter=w3.max_iter, M_divergence=w3.M, epsilon_stationnary=1e-3,
                                 mode=mode, calc_dzndc=True, interior=True, bla=True,
                                 xr_semantics=w3.xr_mode)
        idx3 = sample_indices(n3, parity_pixels, 13)
        idx3_dev = torch.from_numpy(idx3).to(dev)
        k_fe, st_fe = timed(lambda: ctx.perturb_tiles(c3("fe32"), [t3], nat.DEVICE), 3, 1)
        si_fe, sr_fe = si3.cpu().numpy().copy(), sr3.cpu().numpy().copy()
        s_fe = gather_outputs(idx3_dev, Z3, si3, sr3, 2)
        k_xr, st_xr = timed(lambda: ctx.perturb_tiles(c3("xr64"), [t3], nat.DEVICE), 1, 0)
        si_xr, sr_xr = si3.cpu().numpy(), sr3.cpu().numpy()
        s_xr = gather_outputs(idx3_dev, Z3, si3, sr3, 2)
        if parity_pixels > 0:
            t0 = time.perf_counter()
            o3 = oracle_pixels(w3, idx3, oracle_kw(w3, interior=True, eps_stat=1e-3))
            par3 = {"sample": f"{idx3.size} seeded random pixels", "oracle_s": time.perf_counter() - t0,
                    "oracle": "strict C restatement, Xrange branch, interior detection",
                    "fe32": parity_table(s_fe, o3, w3.M), "xr64": parity_table(s_xr, o3, w3.M),
                    "stop_reasons_oracle": {str(k): int(v) for k, v in zip(
                        *np.unique(o3["sr"], return_counts=True))}}
        else:
            par3 = None
        out["deep_m2_1e-1000"] = {
            "workload": f"perturbation Mandelbrot {w3.nx}x{w3.ny} at dx=1e-1000 on a period-{w3.p} "
                        "nucleus, 1100 digits, max_iter 1e6, interior detection eps 1e-3, dzndc",
            "pixels": n3, "pixel_iters": int(st_fe["pixel_iters"]),
            "fe32": {"kernel_ms": k_fe, "value": st_fe["pixel_iters"] / (k_fe * 1e-3)},
            "xr64": {"kernel_ms": k_xr, "value": st_xr["pixel_iters"] / (k_xr * 1e-3)},
            "speedup_fe32_vs_xr64": (st_fe["pixel_iters"] / k_fe) / (st_xr["pixel_iters"] / k_xr),
            "fe32_vs_xr64": {"iter_count_differs_frac": float(np.mean(si_fe != si_xr)),
                             "stop_reason_differs_frac": float(np.mean(sr_fe != sr_xr)),
                             "iter_count_max_abs_diff": int(np.max(np.abs(
                                 si_fe.astype(np.int64) - si_xr)))},
            "vs_oracle": par3,
            "unit": "pixel-iter/s"}
        ref3.free()
        del Z3, sr3, si3

    if "edge" in legs:
        # the headline's nucleus at width 1.6e-9: the minibrot and its
        # surroundings, about half the pixels escape (FP64 branch at this
        # width; XR64 on the same view with the Xrange branch forced)
        we = syn.edge_workload(nx=edge_nx)
        out["edge_m2_p2562"] = view_leg(
            ctx, nat, torch, dev, timed, we, syn.edge_workload(nx=edge_nx, xr_mode=True),
            min(parity_pixels, 8192), 17,
            f"perturbation Mandelbrot {we.nx}x{we.ny} at dx=1.6e-9 on the period-{we.p} nucleus "
            "of the headline (400 digits), max_iter 2e5, BLA eps 1e-6, dzndc, potential, DEM")

    if "seahorse" in legs:
        ws = syn.seahorse_workload(nx=1024)
        out["seahorse_m2"] = view_leg(
            ctx, nat, torch, dev, timed, ws, None, min(parity_pixels, 16384), 19,
            "perturbation Mandelbrot 1024x1024, seahorse valley -0.743643887037151 + "
            "0.131825904205330i, width 2e-9, reference at the centre (no period), max_iter 6000, "
            "every pixel escapes (median 1061 iterations)")

    if "bs" in legs:
        # Burning Ship: 64 tiles of 256..2048 squared at max_iter 5e4 -- FE32
        # over all of them in one launch; FP64 (and FE32 again) on a subset of
        # ~2.5 % of the pixels, labelled (FP64 over all 64 tiles takes ~14 min
        # on GB300's FP64 pipe)
        out["burning_ship_64_tiles"] = bs_leg(
            ctx, nat, torch, dev, timed, syn.config4_workload(max_iter=bs_max_iter)[:bs_tiles],
            bs_max_iter, 0.025,
            f"Burning Ship, {{n}} tiles of side 256..2048 (log-uniform), widths 1e-200..1e-30, "
            f"centres from the BS ball method + Newton at 250 digits, max_iter {bs_max_iter}, "
            "M 1e3, Hessian, one launch")
    if "bs_edge" in legs:
        # the same centres, each tile four times its nucleus' size estimate
        # wide (boundary-straddling: pixels escape), first 16 tiles; FP64 on
        # a labelled subset of about a quarter of the pixels
        out["burning_ship_edge_16_tiles"] = bs_leg(
            ctx, nat, torch, dev, timed,
            syn.config4_workload(max_iter=bs_max_iter, n_tiles=16, edge=True),
            bs_max_iter, 0.25,
            f"Burning Ship, {{n}} tiles of the 64-tile workload's first centres, each 4 x its "
            f"nucleus size estimate wide, max_iter {bs_max_iter}, M 1e3, Hessian, one launch")
    if "model_api" in legs:
        out["model_api_e2e"] = model_api_leg(syn)
    if "host" in legs:
        out["host_1100_digits"] = host_leg(syn)
    return out


def bs_leg(ctx, nat, torch, dev, timed, tiles4, max_iter, fp64_frac, workload):
    """Burning Ship tiles in one launch: FE32 over all of them, then FP64 and
    FE32 over the first tiles holding ``fp64_frac`` of the pixels (the
    like-for-like ratio and the iteration-count agreement are taken there)."""
    f64 = dict(dtype=torch.float64, device=dev)
    refs4, keep, ts = [], [], []
    for t in tiles4:
        r = nat.Reference(ctx, t.Zn, div_iter=t.div_iter, order=t.ref_order, flavor=1,
                          calc_dzndc=True, scale_m=t.dx_m, scale_e=t.dx_e, bla=True, kc=t.kc,
                          bla_eps=1e-6)
        m = t.side * t.side
        xs = torch.from_numpy(t.xs).to(dev)
        ys = torch.from_numpy(t.ys).to(dev)
        Z = torch.zeros((6, m), **f64)
        sr = torch.zeros(m, dtype=torch.int8, device=dev)
        si = torch.zeros(m, dtype=torch.int32, device=dev)
        U = torch.zeros(m, dtype=torch.int32, device=dev)
        keep.append((xs, ys, Z, sr, si, U))
        refs4.append(r)
        ts.append(nat.make_tile_ptrs(nx=t.side, ny=t.side, xs_ptr=xs.data_ptr(),
                                     ys_ptr=ys.data_ptr(), lin_mat=LIN, Z_ptr=Z.data_ptr(), nZ=6,
                                     stop_reason_ptr=sr.data_ptr(), stop_iter_ptr=si.data_ptr(),
                                     U_ptr=U.data_ptr(), ref=r, dx_m=t.dx_m, dx_e=t.dx_e,
                                     drift_m=t.driftx_m, drift_e=t.driftx_e,
                                     drifty_m=t.drifty_m, drifty_e=t.drifty_e))

    def c4(mode):
        return nat.make_calc(max_iter=max_iter, M_divergence=1000., flavor=1,
                             calc_dzndc=True, bla=True, mode=mode)
    npx = np.array([t.side ** 2 for t in tiles4])
    k_sub = int(np.searchsorted(np.cumsum(npx), fp64_frac * npx.sum(), side="right"))
    k_sub = max(1, min(len(tiles4), k_sub))
    sub = ts[:k_sub]

    def counts(k):
        return np.concatenate([keep[i][4].cpu().numpy() for i in range(k)])
    k_all, st_all = timed(lambda: ctx.perturb_tiles(c4("fe32"), ts, nat.DEVICE), 1, 0)
    esc = float(np.mean(np.concatenate([keep[i][3].cpu().numpy() for i in range(len(ts))]) == 1))
    kf, stf = timed(lambda: ctx.perturb_tiles(c4("fe32"), sub, nat.DEVICE), 1, 0)
    si_fe = counts(k_sub)
    k64, st64 = timed(lambda: ctx.perturb_tiles(c4("fp64"), sub, nat.DEVICE), 1, 0)
    si_64 = counts(k_sub)
    for r in refs4:
        r.free()
    v_fe, v_64 = stf["pixel_iters"] / (kf * 1e-3), st64["pixel_iters"] / (k64 * 1e-3)
    return {
        "workload": workload.format(n=len(tiles4)),
        "pixels": int(npx.sum()), "escaped_frac": esc,
        "periods": sorted({t.order for t in tiles4 if t.order}),
        "fe32": {"tiles": len(tiles4), "kernel_ms": k_all, "pixel_iters": int(st_all["pixel_iters"]),
                 "value": st_all["pixel_iters"] / (k_all * 1e-3), "full_steps": int(st_all["full_steps"]),
                 "bla_steps": int(st_all["bla_steps"])},
        "subset": {"tiles": k_sub, "pixels": int(npx[:k_sub].sum()),
                   "pixel_frac": float(npx[:k_sub].sum() / npx.sum()),
                   "fe32": {"kernel_ms": kf, "value": v_fe},
                   "fp64": {"kernel_ms": k64, "value": v_64, "pixel_iters": int(st64["pixel_iters"])},
                   "speedup_fe32_vs_fp64": v_fe / v_64,
                   "iter_count_differs_frac": float(np.mean(si_fe != si_64)),
                   "fp64_all_tiles_extrapolated_s": (k64 * 1e-3) * st_all["pixel_iters"]
                                                    / max(st64["pixel_iters"], 1)},
        "unit": "pixel-iter/s"}


def view_leg(ctx, nat, torch, dev, timed, we, wx, parity_pixels, seed, workload):
    """One view in the three forms, one launch each (L2 flushed, kernel time
    from the library's events): FE32 and FP64 on the reference's branch for
    the view's width (``we``), XR64 on the Xrange branch (``wx``, the same
    view with the branch forced; skipped when None).  On a seeded pixel
    sample the outputs are compared with the oracle per output: FE32 and
    FP64 with the oracle's branch of ``we``, XR64 with the oracle's Xrange
    branch; two oracle-only rows give the scale of the differences (the
    Xrange branch against the other, and the oracle against itself with
    every pixel's c offset moved by a relative 2^-24, one FP32 rounding)."""
    n = we.nx * we.ny
    f64 = dict(dtype=torch.float64, device=dev)
    refs = {}
    for key, wk in (("std", we), ("xr", wx)):
        if wk is None:
            continue
        refs[key] = nat.Reference(ctx, wk.Zn, div_iter=wk.div_iter, order=wk.order,
                                  xr_idx=wk.xr_idx, xr_m=wk.xr_m, xr_e=wk.xr_e,
                                  xr_paths=bool(wk.xr_mode), calc_dzndc=True, scale_m=wk.dx_m,
                                  scale_e=wk.dx_e, bla=True, kc=wk.kc, bla_eps=1e-6)
    xs = torch.from_numpy(we.xs).to(dev)
    ys = torch.from_numpy(we.ys).to(dev)
    Z = torch.zeros((2, n, 2), **f64)
    sr = torch.zeros(n, dtype=torch.int8, device=dev)
    si = torch.zeros(n, dtype=torch.int32, device=dev)
    U = torch.zeros(n, dtype=torch.int32, device=dev)
    pot = torch.zeros(n, **f64)
    dem = torch.zeros(n, **f64)
    idx = sample_indices(n, parity_pixels, seed)
    idx_dev = torch.from_numpy(idx).to(dev)
    out = {"workload": workload, "pixels": n}
    samples = {}
    # fe32_longest: the same FE32 launch claiming its pixels longest first
    # (fsg_calc.claim_order), timed beside the default order
    forms = [("fe32", "std", we), ("fe32_longest", "std", we), ("fp64", "std", we)]
    if wx is not None:
        forms.append(("xr64", "xr", wx))
    for form, key, wk in forms:
        mode = "fe32" if form.startswith("fe32") else form
        mode = mode if not (mode == "fp64" and wk.xr_mode) else "xr64"
        t = nat.make_tile_ptrs(nx=wk.nx, ny=wk.ny, xs_ptr=xs.data_ptr(), ys_ptr=ys.data_ptr(),
                               lin_mat=LIN, Z_ptr=Z.data_ptr(), nZ=2,
                               stop_reason_ptr=sr.data_ptr(), stop_iter_ptr=si.data_ptr(),
                               U_ptr=U.data_ptr(), ref=refs[key], dx_m=wk.dx_m, dx_e=wk.dx_e,
                               drift_m=wk.drift_m, drift_e=wk.drift_e, i_dzndc=1,
                               potential_ptr=pot.data_ptr(), dem_ptr=dem.data_ptr())
        c = nat.make_calc(max_iter=wk.max_iter, M_divergence=wk.M, mode=mode, calc_dzndc=True,
                          interior=False, bla=True, xr_semantics=bool(wk.xr_mode),
                          claim_order="longest" if form == "fe32_longest" else "pixels")
        fast = form.startswith("fe32")
        kms, st = timed(lambda: ctx.perturb_tiles(c, [t], nat.DEVICE), 3 if fast else 1,
                        1 if fast else 0)
        g = gather_outputs(idx_dev, Z, si, sr, 1, pot, dem)
        if form == "fe32_longest":
            same = all(np.array_equal(np.asarray(g[k]).view(np.uint8),
                                      np.asarray(samples["fe32"][k]).view(np.uint8)) for k in g)
        else:
            samples[form] = g
        srn = sr.cpu().numpy()
        out[form] = {"kernel_ms": kms, "value": st["pixel_iters"] / (kms * 1e-3),
                     "pixel_iters": int(st["pixel_iters"]), "full_steps": int(st["full_steps"]),
                     "bla_steps": int(st["bla_steps"]), "rebases": int(st["rebases"]),
                     "escaped_frac": float(np.mean(srn == 1))}
        if form == "fe32_longest":
            out[form]["outputs_equal_fe32_on_sample"] = bool(same)
    out["speedup_fe32_vs_fp64"] = out["fe32"]["value"] / out["fp64"]["value"]
    if "xr64" in out:
        out["speedup_fe32_vs_xr64"] = out["fe32"]["value"] / out["xr64"]["value"]
    for r in refs.values():
        r.free()
    if parity_pixels > 0:
        t0 = time.perf_counter()
        kw = oracle_kw(we)
        o_std = oracle_pixels(we, idx, kw)
        br = "Xrange" if we.xr_mode else "FP64"
        rows = {"sample": f"{idx.size} seeded random pixels",
                "oracle": f"strict C restatement; {br} branch (the reference's at this width)"}
        rows[f"fe32_vs_{br.lower()}_branch"] = parity_table(samples["fe32"], o_std, we.M)
        rows[f"fp64_vs_{br.lower()}_branch"] = parity_table(samples["fp64"], o_std, we.M)
        if wx is not None:
            o_xr = oracle_pixels(wx, idx, oracle_kw(wx))
            rows["xr64_vs_xrange_branch"] = parity_table(samples["xr64"], o_xr, we.M)
            rows["oracle_xrange_vs_fp64_branch"] = parity_table(o_xr, o_std, we.M)
        o_shift = oracle_pixels(we, idx, dict(kw, lin_mat=LIN * (1. + 2. ** -24)))
        rows[f"oracle_c_offset_2^-24_vs_{br.lower()}_branch"] = parity_table(o_shift, o_std, we.M)
        rows["oracle_s"] = time.perf_counter() - t0
        out["vs_oracle"] = rows
        # every form and the oracle against exact arithmetic on a sub-sample
        t0 = time.perf_counter()
        sub = np.sort(np.random.default_rng(seed + 1).choice(
            idx.size, size=min(DIRECT_PIXELS, idx.size), replace=False))
        exact = direct_pixels(we, idx[sub])
        pick = lambda s: {k: v[sub] for k, v in s.items()}     # noqa: E731
        rows = {"sample": f"{sub.size} of the seeded pixels above",
                "exact": f"z^2 + c iterated directly at {we.dps} digits (MPFR), dzndc along "
                         "the exact orbit in double",
                f"oracle_{br.lower()}_branch": parity_table(pick(o_std), exact, we.M)}
        for form in samples:
            rows[form] = parity_table(pick(samples[form]), exact, we.M)
        rows["direct_s"] = time.perf_counter() - t0
        out["vs_exact"] = rows
    return out


def model_api_leg(syn, nx=2048):
    """The headline view through the reference's model API, as a
    Fractalshades script runs it: Perturbation_mandelbrot.zoom ->
    calc_std_div -> calc_raw (precision_mode "fe32"), which computes the
    reference orbit on the host, renders the image on the GPU from pageable
    numpy arrays and writes the raw arrays to the memory maps on disk.  The
    first call includes the orbit (its Newton refinement and ball method at
    400 digits); the repeat, under a new calc name, reuses the stored orbit."""
    import tempfile
    import mpmath
    import fractalshades_gb300.models as fsm
    from fractalshades_gb300 import settings
    w = syn.config2_workload(nx=8)
    with mpmath.workdps(400):
        x, y = str(w.center.real), str(w.center.imag)
    old = settings.precision_mode
    settings.precision_mode = "fe32"
    res = {}
    try:
        with tempfile.TemporaryDirectory() as d:
            f = fsm.Perturbation_mandelbrot(d)
            f.zoom(precision=400, x=x, y=y, dx="1e-300", nx=nx, xy_ratio=1., theta_deg=0.)
            for key in ("first", "repeat"):
                f.calc_std_div(calc_name=key, subset=None, max_iter=200000, M_divergence=1000.,
                               epsilon_stationnary=1e-3, BLA_eps=1e-6, interior_detect=False,
                               calc_dzndc=True)
                t0 = time.perf_counter()
                f.calc_raw(key)
                dt = time.perf_counter() - t0
                it = float(f.get_raw(key, "stop_iter").astype(np.int64).sum())
                res[key] = {"s": dt, "pixel_iters": it, "value": it / dt}
    finally:
        settings.precision_mode = old
    return {"workload": f"the {nx}x{nx} 1e-300 view on the period-{w.p} nucleus through "
                        "Perturbation_mandelbrot.calc_raw (fe32), raw arrays written to the "
                        "memory maps", **res, "unit": "pixel-iter/s"}


def host_leg(syn):
    """The arbitrary-precision host side (libfsghost.so on MPFR / MPC) on the
    1e-1000 configuration's period-16607 nucleus at 1100 digits: orbit,
    ball-method period, Newton from a seed 1e-550 away, size estimate (one
    host thread each, the best of 3 for the orbit)."""
    import time
    import mpmath
    from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
    p, dps = 16607, 1100
    with mpmath.workdps(dps):
        c = syn.nucleus(p, dps)
        prec = mpmath.mp.prec
        sx, sy = str(c.real).encode(), str(c.imag).encode()
        orb = np.zeros(p + 1, dtype=np.complex128)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            fsFP.perturbation_mandelbrot_FP_loop(orb, True, p, 2000., sx, sy, prec)
            ts.append(time.perf_counter() - t0)
        t_orbit = min(ts)
        t0 = time.perf_counter()
        order = fsFP.perturbation_mandelbrot_ball_method(sx, sy, prec, b"1e-1000", p + 10, 1e5)
        t_ball = time.perf_counter() - t0
        seed = c + mpmath.mpf(10) ** -550
        t0 = time.perf_counter()
        ok, cn = fsFP.perturbation_mandelbrot_find_nucleus(
            str(seed.real).encode(), str(seed.imag).encode(), prec, p, 80,
            str(mpmath.mpf(2) ** -prec).encode(), b"1e-1000")
        t_newton = time.perf_counter() - t0
        t0 = time.perf_counter()
        fsFP.perturbation_mandelbrot_nucleus_size_estimate(sx, sy, prec, p)
        t_size = time.perf_counter() - t0
        newton_err = float(mpmath.log10(abs(cn - c))) if ok else None
    return {"workload": "period-16607 nucleus at 1100 digits (3654 bits)",
            "orbit_s": t_orbit, "orbit_it_per_s": p / t_orbit, "ball_s": t_ball,
            "ball_order": int(order), "newton_s": t_newton, "newton_converged": bool(ok),
            "newton_log10_err": newton_err, "size_estimate_s": t_size,
            "arithmetic": "MPFR 4.2 / MPC 1.3, the reference's call sequence"}


def traffic_per_launch(nx):
    """DRAM bytes of one FE32 launch from the committed ncu capture
    (profiles/dram_fe32_config2_2048.md), for the 2048² workload it was
    measured on; None for another size."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_fe32_config2_2048.json")) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return None
    return int(rec["bytes_per_launch"]) if nx == 2048 else None


# algorithmic bytes per pixel of a headline launch: the outputs zn and
# dzndc (complex128), U and stop_iter (int32), stop_reason (int8), potential
# and DEM (float64); the orbit tables are read once and stay in L2
BYTES_PER_PIXEL = 16 + 16 + 4 + 4 + 1 + 8 + 8


def hbm_roofline(npix, naxes, kernel_ms, traffic):
    """The launch against the HBM roofline: algorithmic bytes (outputs and
    the pixel axes) over the kernel time, against the measured copy bandwidth
    of this pool (6.8 TB/s fallback).  The kernel is bound by instruction
    issue, so this fraction is small by construction."""
    peak, src = 6800.0, "fallback (one earlier GB300 measurement)"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "measured copy bandwidth of this pool"
    except (OSError, ValueError, KeyError):
        pass
    nbytes = npix * BYTES_PER_PIXEL + 8 * naxes
    achieved = nbytes / (kernel_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes": nbytes,
            "peak_source": src}


class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0., set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU legs: the oracle (C restatement of the reference's loop) on host cores
# ---------------------------------------------------------------------------
CPU_TILE = 200          # the reference's tile side (settings.py:34)
DIRECT_PIXELS = 256     # pixels of a view checked against exact arithmetic


def oracle_kw(w, interior=False, eps_stat=0.):
    """Orbit-derived inputs of the oracle for a power-2 workload (BLA tree,
    derivative paths), the reference's branch given by ``w.xr_mode``."""
    from oracle import oracle as orc
    Mb, rb, _, st = orc.make_bla_m2(w.Zn, w.kc, 1e-6)
    dz = orc.dzndc_path_m2(w.Zn, w.div_iter, w.order, w.xr_mode, w.dx_m, w.dx_e,
                           w.xr_idx, w.xr_m, w.xr_e)
    kw = dict(Zn=w.Zn, ref_div_iter=w.div_iter, ref_order=w.order, lin_mat=LIN,
              dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
              max_iter=w.max_iter, M=w.M, eps_stat=eps_stat, xr_mode=w.xr_mode,
              bla=(Mb, rb, st), dZndc=dz, xr_idx=w.xr_idx, xr_m=w.xr_m, xr_e=w.xr_e,
              interior=interior)
    if interior:
        kw["dZndz"] = orc.dzndz_path_m2(w.Zn, w.div_iter, w.xr_mode, w.xr_idx, w.xr_m, w.xr_e)
    return kw


def oracle_threads():
    return os.cpu_count() or 1


def oracle_pixels(w, idx, kw, threads=None, fast=False):
    """The oracle at flat pixel indices ``idx`` (row-major, x fastest) of the
    workload's image, split over host threads (ctypes releases the GIL).
    Returns stop_iter, stop_reason, zn, dzndc (and dzndz with interior)."""
    from oracle import oracle as orc
    threads = threads or oracle_threads()
    pix = w.xs[idx % w.nx] + 1j * w.ys[idx // w.nx]
    parts = np.array_split(np.arange(idx.size), max(1, min(threads * 4, idx.size)))
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(lambda ii: orc.perturb_m2(pix[ii], fast=fast, **kw), parts))
    Z = np.concatenate([r[0] for r in res], axis=1)
    out = {"si": np.concatenate([r[3][0] for r in res]),
           "sr": np.concatenate([r[2][0] for r in res]),
           "zn": Z[0], "dzndc": Z[-1]}
    return out


def direct_pixels(w, idx, threads=None):
    """Exact-arithmetic outputs at flat pixel indices ``idx`` of a power-2
    workload: z -> z^2 + c iterated directly at the workload's digits (the
    MPFR orbit of the host library, every z_i rounded to double), c the
    pixel's point (the view centre + dx (x + i y)); stop_iter the first i
    with |z_i| > M (max_iter and stop reason 0 when there is none), zn = z_i,
    dzndc per unit of dx from the double recurrence d' = 2 z d + 1 along the
    exact orbit (linear: no chaotic growth of its rounding)."""
    import mpmath
    from fractalshades_gb300.mpmath_utils import FP_loop as fsFP
    threads = threads or oracle_threads()
    with mpmath.workdps(w.dps):
        prec = mpmath.mp.prec
        dx = mpmath.mpf(w.dx)
        cs = [w.center + dx * mpmath.mpc(float(w.xs[k % w.nx]), float(w.ys[k // w.nx]))
              for k in idx]
        pts = [(mpmath.nstr(c.real, w.dps + 5), mpmath.nstr(c.imag, w.dps + 5)) for c in cs]
    fdx = float(dx)

    def one(pt):
        buf = np.zeros(w.max_iter + 1, dtype=np.complex128)
        i = int(fsFP.perturbation_mandelbrot_FP_loop(buf, False, w.max_iter, w.M, pt[0], pt[1],
                                                     prec)[0])
        n = min(i, w.max_iter)
        d = 0j
        for z in buf[:n]:
            d = 2. * z * d + 1.
        return (n, 1 if i <= w.max_iter else 0, buf[n], d * fdx)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, pts))
    return {"si": np.array([r[0] for r in res], dtype=np.int32),
            "sr": np.array([r[1] for r in res], dtype=np.int8),
            "zn": np.array([r[2] for r in res]), "dzndc": np.array([r[3] for r in res])}


def potential_dem(zn, dzndc, n, M, d=2.):
    """Potential (postproc.py:352-406, Continuous_iter_pp_infinity
    :1001-1009 with a_d = 1) and distance estimate (postproc.py:684-731)
    from the raw outputs, in float64: the formula of the kernels' fused
    epilogue, applied to the oracle's outputs."""
    with np.errstate(all="ignore"):
        az = np.abs(zn)
        x = np.log(np.log(az) / np.log(M)) / np.log(d)
        q = np.floor(x)
        pot = (n.astype(np.float64) - q) - (x - q)
        dem = az * np.log(az) / np.abs(dzndc)
    return pot, dem


def parity_table(gpu, ref, M):
    """Per output, one GPU form against the oracle on the same pixels:
    iteration counts, stop reasons, and -- on the pixels whose counts agree --
    the largest relative error of zn and dzndc, and on those that escaped
    (stop reason 1) of the potential and the distance estimate."""
    si, so = gpu["si"].astype(np.int64), ref["si"].astype(np.int64)
    d = np.abs(si - so)
    same = d == 0
    esc = same & (ref["sr"] == 1) & (gpu["sr"] == 1)

    def rel(a, b, m):
        with np.errstate(all="ignore"):
            r = np.abs(a - b) / np.abs(b)
        r = r[m & np.isfinite(r)]
        return (float(r.max()), float(np.median(r))) if r.size else (0.0, 0.0)
    pg, dg = potential_dem(gpu["zn"], gpu["dzndc"], gpu["si"], M)
    pg, dg = gpu.get("pot", pg), gpu.get("dem", dg)      # the kernel's own epilogue
    po, do = potential_dem(ref["zn"], ref["dzndc"], ref["si"], M)
    t = {"pixels": int(si.size), "escaped": int((ref["sr"] == 1).sum()),
         "iter_count_differs_frac": float(np.mean(~same)),
         "iter_count_max_abs_diff": int(d.max()) if d.size else 0,
         "iter_count_differs_by_more_than_1_frac": float(np.mean(d > 1)),
         "stop_reason_differs_frac": float(np.mean(gpu["sr"] != ref["sr"]))}
    for k, (a, b, m) in {"zn": (gpu["zn"], ref["zn"], same),
                         "dzndc": (gpu["dzndc"], ref["dzndc"], same),
                         "potential": (pg, po, esc), "dem": (dg, do, esc)}.items():
        mx, md = rel(a, b, m)
        t[k + "_max_rel_err"], t[k + "_median_rel_err"] = mx, md
    return t


def sample_indices(n, k, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(k, n), replace=False)).astype(np.int64)


def gather_outputs(idx_dev, Z, si, sr, i_dzndc, pot=None, dem=None):
    """A GPU form's outputs at the sampled pixels (device gather, one copy);
    with ``pot`` / ``dem`` the kernel's own fused potential and distance
    estimate."""
    zn = Z[0].index_select(0, idx_dev).cpu().numpy()
    dz = Z[i_dzndc].index_select(0, idx_dev).cpu().numpy()
    out = {"si": si.index_select(0, idx_dev).cpu().numpy(),
           "sr": sr.index_select(0, idx_dev).cpu().numpy(),
           "zn": zn[:, 0] + 1j * zn[:, 1], "dzndc": dz[:, 0] + 1j * dz[:, 1]}
    if pot is not None:
        out["pot"] = pot.index_select(0, idx_dev).cpu().numpy()
    if dem is not None:
        out["dem"] = dem.index_select(0, idx_dev).cpu().numpy()
    return out


def image_tiles(nx, ny, side=CPU_TILE):
    """The reference's tiling of an image (core.py:1767-1830): origins and
    sizes of the side x side tiles, row-major."""
    return [(x0, y0, min(side, nx - x0), min(side, ny - y0))
            for y0 in range(0, ny, side) for x0 in range(0, nx, side)]


def cpu_baseline(w, target_s=10.0, threads=None, seed=7, min_tiles=4, n_tiles=None, kw=None):
    """The reference's CPU path restated: the -ffast-math oracle
    (numba fastmath=True, perturbation.py:988, 1075) over a seeded subset of
    whole 200 x 200 tiles of the image, one tile per task on a pool of one
    thread per host core (mthreading.py:48-68).  The subset is ``n_tiles``
    tiles, or sized from a one-tile calibration to about ``target_s`` of wall
    time (at least ``min_tiles`` and 1 % of the image)."""
    threads = threads or oracle_threads()
    kw = kw or oracle_kw(w)
    tiles = image_tiles(w.nx, w.ny)
    order = np.random.default_rng(seed).permutation(len(tiles))

    def run_tile(k):
        x0, y0, tx, ty = tiles[k]
        X, Y = np.meshgrid(w.xs[x0:x0 + tx], w.ys[y0:y0 + ty])
        from oracle import oracle as orc
        return orc.perturb_m2((X + 1j * Y).ravel(), fast=True, **kw)[3]

    if n_tiles is None:
        t0 = time.perf_counter()
        run_tile(order[0])
        per_tile = max(time.perf_counter() - t0, 1e-3)
        n_tiles = int(max(min_tiles, min(len(tiles), target_s * threads / per_tile)))
        n_tiles = max(n_tiles, int(np.ceil(0.01 * len(tiles))))
    k = min(int(n_tiles), len(tiles))
    pick = order[:k]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(run_tile, pick))
    dt = time.perf_counter() - t0
    iters = float(sum(float(r.sum()) for r in res))
    npx = int(sum(r.size for r in res))
    return {"value": iters / dt, "unit": "pixel-iter/s", "cores": threads, "kind": "port",
            "sample": f"{k} of the {len(tiles)} whole {CPU_TILE}x{CPU_TILE} tiles of the "
                      f"{w.nx}x{w.ny} image (seeded, {100.0 * npx / (w.nx * w.ny):.1f} % of the "
                      f"pixels, {iters:.3e} pixel-iterations in {dt:.2f} s), one tile per task "
                      f"on {threads} threads; Xrange branch, BLA on",
            "build": "oracle/fs_oracle.c at -O2 -ffast-math -fno-tree-vectorize "
                     "(libfs_oracle_fast.so)",
            "tiles": k, "extrapolated_full_image_s": dt * (w.nx * w.ny) / max(npx, 1)}


def run_reference(args):
    """--impl reference: the reference's CPU loop (oracle port; the reference
    itself needs numba, absent here) on every host core."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from fractalshades_gb300 import synthetic as syn
    w = syn.config2_workload(nx=args.nx)
    vals = []
    kw = oracle_kw(w)
    n_tiles = None          # sized once, by the first (warm-up) step's calibration
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(w, target_s=3.0, seed=7 + s, n_tiles=n_tiles, kw=kw)
        n_tiles = r["tiles"]
        if s >= args.warmup:
            vals.append(r["value"])
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pixel-iter/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+i32exp", "data": "synthetic",
            "config": config_dict(w, args),
            "cpu_baseline": {"value": v, "unit": "pixel-iter/s", "cores": r["cores"],
                             "kind": "port", "sample": "per step: " + r["sample"],
                             "build": r["build"]},
            "e2e": {"value": v, "unit": "pixel-iter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def job_seconds(rank_seconds, dist=None, device="cpu"):
    """The job's time over its replicas: the slowest rank's (max over ranks,
    returned on every rank); a rank's own time without a process group."""
    if dist is None:
        return float(rank_seconds)
    import torch
    t = torch.tensor([float(rank_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(pixel_iters_per_step, steps, world, seconds):
    """Whole-job pixel-iterations/s: every rank runs its own replica of the
    workload (weak scaling), the job takes the slowest rank's time."""
    return pixel_iters_per_step * steps * world / seconds


def config_dict(w, args):
    return {"workload": "perturbation Mandelbrot 2048x2048 at dx=1e-300 on a period-p nucleus",
            "nx": w.nx, "ny": w.ny, "dx": "1e-300", "period": w.p, "digits": w.dps,
            "max_iter": w.max_iter, "M_divergence": w.M, "BLA_eps": 1e-6,
            "outputs": ["stop_iter", "stop_reason", "zn", "dzndc", "potential", "DEM"],
            "seed": 2, "l2": "flushed between timed steps (256 MB write)"}


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from fractalshades_gb300 import _native as nat
    from fractalshades_gb300 import synthetic as syn

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    # a dedicated stream: the library launches on it and the CUDA events
    # that time the steps are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    ctx = nat.Context(local)
    ctx.set_stream(stream.cuda_stream)
    if args.no_headline:
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
        supp = supplementary(ctx, nat, syn, torch, dev, stream, flush, args.bs_max_iter,
                             legs=tuple(args.legs.split(",")), bs_tiles=args.bs_tiles,
                             edge_nx=args.edge_nx,
                             parity_pixels=min(16384, args.parity_pixels))
        print(json.dumps({"note": "supplementary legs only (--no-headline)",
                          "supplementary": supp}), flush=True)
        return 0
    w = syn.config2_workload(nx=args.nx)
    n = w.nx * w.ny
    peak32 = ctx.peak_tflops(False)
    peak64 = ctx.peak_tflops(True)

    refs = {}
    refs["xr"] = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order,
                               xr_idx=w.xr_idx, xr_m=w.xr_m, xr_e=w.xr_e, xr_paths=True,
                               calc_dzndc=True, scale_m=w.dx_m, scale_e=w.dx_e, bla=True,
                               kc=w.kc, bla_eps=1e-6)
    refs["std"] = nat.Reference(ctx, w.Zn, div_iter=w.div_iter, order=w.order,
                                xr_idx=w.xr_idx, xr_m=w.xr_m, xr_e=w.xr_e, xr_paths=False,
                                calc_dzndc=True, scale_m=w.dx_m, scale_e=w.dx_e, bla=True,
                                kc=w.kc, bla_eps=1e-6)

    f64 = dict(dtype=torch.float64, device=dev)
    xs = torch.from_numpy(w.xs).to(dev)
    ys = torch.from_numpy(w.ys).to(dev)
    Z = torch.zeros((2, n, 2), **f64)          # complex128 [zn, dzndc]
    U = torch.zeros(n, dtype=torch.int32, device=dev)
    sr = torch.zeros(n, dtype=torch.int8, device=dev)
    si = torch.zeros(n, dtype=torch.int32, device=dev)
    pot = torch.zeros(n, **f64)
    dem = torch.zeros(n, **f64)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    # seeded pixels of the image whose outputs are checked against the oracle
    idx = sample_indices(n, args.parity_pixels, 11)
    idx_dev = torch.from_numpy(idx).to(dev)
    samples = {}

    def tile(ref):
        return nat.make_tile_ptrs(
            nx=w.nx, ny=w.ny, xs_ptr=xs.data_ptr(), ys_ptr=ys.data_ptr(), lin_mat=LIN,
            Z_ptr=Z.data_ptr(), nZ=2, stop_reason_ptr=sr.data_ptr(),
            stop_iter_ptr=si.data_ptr(), U_ptr=U.data_ptr(), ref=ref, dx_m=w.dx_m,
            dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e, i_dzndc=1,
            potential_ptr=pot.data_ptr(), dem_ptr=dem.data_ptr())

    launch = {}    # mode -> (block, ctas_per_sm) chosen by the autotuner

    def calc(mode):
        c = nat.make_calc(max_iter=w.max_iter, M_divergence=w.M, mode=mode,
                          calc_dzndc=True, interior=False, bla=True,
                          xr_semantics=w.xr_mode)
        if mode in launch:
            c.block, c.ctas_per_sm = launch[mode]
        return c

    def timed_steps(mode, ref, k, warm):
        t, c = tile(ref), calc(mode)
        for _ in range(warm):
            ctx.perturb_tiles(c, [t], nat.DEVICE)
        torch.cuda.synchronize(dev)
        step_ms, kern_ms, stats = [], [], []
        if dist:
            dist.barrier()
        for _ in range(k):
            flush.fill_(1.0)
            stream.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.perturb_tiles(c, [t], nat.DEVICE)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            st = ctx.stats()
            kern_ms.append(st["kernel_ms"])
            stats.append(st)
        torch.cuda.synchronize(dev)
        return step_ms, kern_ms, stats

    def snapshot():
        return (si.cpu().numpy().copy(), sr.cpu().numpy().copy(),
                pot.cpu().numpy().copy(), dem.cpu().numpy().copy())

    # headline: FP32 + exponent, at the launch shape the autotuner picks on
    # this workload (untimed: one launch per candidate)
    from fractalshades_gb300 import tune
    tuned = tune.autotune(ctx, calc("fe32"), [tile(refs["xr"])], perturb=True, repeats=1,
                          store=False)
    launch["fe32"] = (tuned["block"], tuned["ctas_per_sm"])
    with ClockSampler(local) as clk:
        step_ms, kern_ms, stats = timed_steps("fe32", refs["xr"], args.steps, args.warmup)
    fe_out = snapshot()
    samples["fe32"] = gather_outputs(idx_dev, Z, si, sr, 1, pot, dem)
    pix_iters = stats[-1]["pixel_iters"]
    total_s = job_seconds(sum(step_ms) / 1e3, dist, dev)
    value = job_value(pix_iters, args.steps, world, total_s)
    st = stats[-1]
    flops = st["full_steps"] * FLOPS_FULL + st["bla_steps"] * FLOPS_BLA
    kms = float(np.mean(kern_ms))
    achieved = flops / (kms * 1e-3) / 1e12

    # the two FP64 forms of the reference (one or two steps each: slower)
    k64 = max(1, min(2, args.steps))
    xr_step, xr_kern, xr_stats = timed_steps("xr64", refs["xr"], k64, 1)
    xr_out = snapshot()
    samples["xr64"] = gather_outputs(idx_dev, Z, si, sr, 1, pot, dem)
    fp_step, fp_kern, fp_stats = timed_steps("fp64", refs["std"], k64, 1)
    samples["fp64"] = gather_outputs(idx_dev, Z, si, sr, 1, pot, dem)
    value_xr = xr_stats[-1]["pixel_iters"] / (np.mean(xr_step) / 1e3)
    value_fp = fp_stats[-1]["pixel_iters"] / (np.mean(fp_step) / 1e3)
    fl64 = xr_stats[-1]["full_steps"] * FLOPS_FULL + xr_stats[-1]["bla_steps"] * FLOPS_BLA
    achieved64 = fl64 / (np.mean(xr_kern) * 1e-3) / 1e12

    # accuracy of the FP32 form against the FP64 (Xrange) form, per output
    def relerr(a, b):
        m = np.isfinite(a) & np.isfinite(b) & (b != 0)
        return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m]))) if m.any() else 0.0
    accuracy = {
        "pixels": int(n),
        "iter_count_differs_frac": float(np.mean(fe_out[0] != xr_out[0])),
        "iter_count_max_abs_diff": int(np.max(np.abs(fe_out[0].astype(np.int64) - xr_out[0]))),
        "stop_reason_differs_frac": float(np.mean(fe_out[1] != xr_out[1])),
        "potential_max_rel_err": relerr(fe_out[2], xr_out[2]),
        "dem_max_rel_err": relerr(fe_out[3], xr_out[3]),
    }

    # end to end through the C-ABI with host buffers (pinned), FP32 form
    h = {}
    h["Z"] = torch.zeros((2, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    h["U"] = torch.zeros(n, dtype=torch.int32, pin_memory=True).numpy()
    h["sr"] = torch.zeros(n, dtype=torch.int8, pin_memory=True).numpy()
    h["si"] = torch.zeros(n, dtype=torch.int32, pin_memory=True).numpy()
    h["pot"] = torch.zeros(n, dtype=torch.float64, pin_memory=True).numpy()
    h["dem"] = torch.zeros(n, dtype=torch.float64, pin_memory=True).numpy()
    hxs = torch.from_numpy(w.xs).pin_memory().numpy()
    hys = torch.from_numpy(w.ys).pin_memory().numpy()
    Zc = h["Z"].view(np.complex128).reshape(2, n)
    ht = nat.make_tile(xs=hxs, ys=hys, lin_mat=LIN, Z=Zc, U=h["U"], stop_reason=h["sr"],
                       stop_iter=h["si"], ref=refs["xr"], dx_m=w.dx_m, dx_e=w.dx_e,
                       drift_m=w.drift_m, drift_e=w.drift_e, i_dzndc=1,
                       potential=h["pot"], dem=h["dem"])
    hc = calc("fe32")
    ctx.perturb_tiles(hc, [ht], nat.HOST)
    e2e_t = []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        ctx.perturb_tiles(hc, [ht], nat.HOST)
        e2e_t.append(time.perf_counter() - t0)
    e2e_val = int(h["si"].astype(np.int64).sum()) / float(np.mean(e2e_t))
    d2h = sum(a.nbytes for a in h.values())
    h2d = hxs.nbytes + hys.nbytes

    # tile latency: a seeded stream of tiles of 256..2048 squared through the
    # host-buffer call, with fresh pageable arrays per tile (the library
    # stages them) and with page-locked arrays reused per size (written in
    # place)
    sizes = [256, 512, 1024, 2048]
    pinned = {}
    for side in sizes:
        m = side * side
        pinned[side] = {
            "Z": torch.zeros((2, m, 2), dtype=torch.float64, pin_memory=True).numpy(),
            "U": torch.zeros(m, dtype=torch.int32, pin_memory=True).numpy(),
            "sr": torch.zeros(m, dtype=torch.int8, pin_memory=True).numpy(),
            "si": torch.zeros(m, dtype=torch.int32, pin_memory=True).numpy()}
        xs_t, ys_t = syn.image_axes(side, side)
        pinned[side]["xs"] = torch.from_numpy(xs_t).pin_memory().numpy()
        pinned[side]["ys"] = torch.from_numpy(ys_t).pin_memory().numpy()
    lat, lat_pin = [], []
    for kind, out in (("pageable", lat), ("pinned", lat_pin)):
        rng = np.random.default_rng(5)
        for i in range(24):
            side = int(rng.choice(sizes))
            m = side * side
            if kind == "pageable":
                xs_t, ys_t = syn.image_axes(side, side)
                bufs = {"Z": np.zeros((2, m), dtype=np.complex128),
                        "U": np.zeros(m, dtype=np.int32), "sr": np.zeros(m, dtype=np.int8),
                        "si": np.zeros(m, dtype=np.int32)}
            else:
                b = pinned[side]
                xs_t, ys_t = b["xs"], b["ys"]
                bufs = {"Z": b["Z"].view(np.complex128).reshape(2, m), "U": b["U"],
                        "sr": b["sr"], "si": b["si"]}
            tt = nat.make_tile(xs=xs_t, ys=ys_t, lin_mat=LIN, Z=bufs["Z"], U=bufs["U"],
                               stop_reason=bufs["sr"], stop_iter=bufs["si"], ref=refs["xr"],
                               dx_m=w.dx_m, dx_e=w.dx_e, drift_m=w.drift_m, drift_e=w.drift_e,
                               i_dzndc=1)
            t0 = time.perf_counter()
            ctx.perturb_tiles(hc, [tt], nat.HOST)
            out.append((time.perf_counter() - t0) * 1e3)
    lat, lat_pin = np.array(lat[2:]), np.array(lat_pin[2:])

    supp = None
    if not args.no_supplementary and rank == 0:
        supp = supplementary(ctx, nat, syn, torch, dev, stream, flush, args.bs_max_iter,
                             legs=tuple(args.legs.split(",")), bs_tiles=args.bs_tiles,
                             edge_nx=args.edge_nx,
                             parity_pixels=min(16384, args.parity_pixels))

    serving = None
    if args.serving_requests > 0 and rank == 0:
        serving = serving_leg(args.serving_requests, local)

    if rank != 0:
        if dist:
            dist.barrier()
        return 0

    # the headline's outputs against the oracle (the reference's Xrange
    # branch at this width) on the sampled pixels, per form and output
    parity = None
    if idx.size:
        t0 = time.perf_counter()
        o2 = oracle_pixels(w, idx, oracle_kw(w))
        parity = {"sample": f"{idx.size} seeded random pixels of the {w.nx}x{w.ny} image",
                  "oracle": "strict C restatement of the reference's loop, Xrange branch",
                  "oracle_s": time.perf_counter() - t0,
                  "forms": {k: parity_table(v, o2, w.M) for k, v in samples.items()}}

    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_baseline(w, target_s=10.0)

    line = {
        "metric": METRIC, "value": value, "unit": "pixel-iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32exp",
        "data": "synthetic",
        "config": dict(config_dict(w, args), launch={
            "block": tuned["block"], "ctas_per_sm": tuned["ctas_per_sm"],
            "autotuned_over": [[e["block"], e["ctas_per_sm"], round(e["kernel_ms"], 3)]
                               for e in tuned["table"]]}),
        "e2e": {"value": e2e_val, "unit": "pixel-iter/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "path": "fsg_perturb_tiles with page-locked host buffers: the kernel reads "
                        "the axes and writes every output in host memory (NVLink-C2C), "
                        "timed from the call to its return"},
        "gpu_launches": int(args.steps),
        "roofline": {"bound": "fp32-fma", "achieved": achieved, "peak": peak32,
                     "unit": "TFLOP/s", "frac": achieved / peak32 if peak32 else None,
                     "traffic": traffic_per_launch(args.nx),
                     "peak_source": "measured FFMA-chain kernel on this GPU (fsg_peak_flops)",
                     "flops_per_step": {"full": FLOPS_FULL, "bla": FLOPS_BLA},
                     "executed_steps": {"full": st["full_steps"], "bla": st["bla_steps"]},
                     "kernel_ms": kms},
        "roofline_hbm": hbm_roofline(n, w.nx + w.ny, kms, traffic_per_launch(args.nx)),
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "paths": {
            "fe32": {"value": value, "kernel_ms": kms},
            "xr64": {"value": value_xr, "kernel_ms": float(np.mean(xr_kern)),
                     "fp64_tflops": achieved64, "fp64_peak": peak64},
            "fp64": {"value": value_fp, "kernel_ms": float(np.mean(fp_kern))},
            "speedup_fe32_vs_xr64": value / value_xr if value_xr else None,
            "speedup_fe32_vs_fp64": value / value_fp if value_fp else None,
        },
        "accuracy_fe32_vs_xr64": accuracy,
        "parity_vs_oracle": parity,
        "serving": serving,
        "supplementary": supp,
        "tile_latency_ms": {"p50": float(np.percentile(lat, 50)),
                            "p99": float(np.percentile(lat, 99)), "tiles": int(lat.size),
                            "sizes": sizes,
                            "path": "C-ABI host buffers, FP32+exp, fresh pageable arrays",
                            "pinned": {"p50": float(np.percentile(lat_pin, 50)),
                                       "p99": float(np.percentile(lat_pin, 99)),
                                       "path": "page-locked arrays reused per size, "
                                               "written in place"}},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
