"""
Request loop for interactive deep zoom: tiles of different sizes and depths
arrive over time, are admitted against an HBM budget as GPU slots and memory
free up, and run concurrently on the device (continuous batching).

* Slots: each slot owns a library context bound to its own CUDA stream; a slot
  runs one launch at a time (a batch of tiles, each with its own reference),
  so up to ``n_slots`` batches overlap on the GPU.
* Admission: a request is admitted when a slot is free and its output buffers
  plus any new reference tables fit in the HBM budget still unreserved;
  memory is released when its results have been copied back.
* Reference cache: the orbit of a centre does not depend on the view, the
  derivative paths scale linearly with dx and only the BLA radii depend on
  kc.  One base reference per (centre, Xrange branch, max_iter) holds the
  orbit and the derivative paths at unit scale; each tile sets its dzndc
  scale 2^(e - 1) (dx = m 2^e, m in [0.5, 1)) with fsg_tile.dzndc_scale_e and
  the output is rescaled by dx / 2^(e - 1).  BLA trees are derived from the
  base (fsg_ref_derive_bla) per kc bucket: kc rounded up to 2^(8 ceil(e/8))
  (smaller, still valid, radii), or 0 below the double range -- where the
  reference's own kc, to_standard(kc), is 0 too.  Every request of a bucket
  uses the same tables whether it runs alone or in a mix, so its result does
  not depend on what else is on the GPU.
* References are built on a context of their own (its own stream) with
  stream-ordered allocation, so a build does not wait for running tiles.
* Latency of a request = arrival -> results on the host.

The reference has no serving mode; this replaces its interactive GUI loop
(gui/guimodel.py runs one script at a time) for headless use.
"""
import collections
import dataclasses
import math
import threading
import time

import mpmath
import numpy as np

from . import _native as nat
from . import synthetic as syn
from . import tune
from .numpy_utils import xrange as fsx
from . import settings

BYTES_PER_PIXEL = 16 * 2 + 4 + 1 + 4 + 8 + 8   # Z (zn, dzndc), U, stop_reason, stop_iter, pot, dem


@dataclasses.dataclass
class Center:
    """A reference point: a nucleus with its FP64 orbit (wrapped at the period)."""
    c: object            # mpmath mpc
    p: int
    dps: int
    Zn: np.ndarray
    xr_idx: np.ndarray
    xr_m: np.ndarray
    xr_e: np.ndarray


@dataclasses.dataclass
class Request:
    rid: int
    center: int          # index into the server's centres
    side: int
    dx: str              # decimal string (may be below the double range)
    offset: tuple        # view centre - nucleus, in units of dx
    max_iter: int
    arrival: float = 0.0
    # filled by the server
    admitted: float = 0.0
    done: float = 0.0
    result: dict = None
    pixel_iters: int = 0


def make_center(p, dps, max_iter):
    c = syn.nucleus(p, dps)
    w = syn.prepare_m2(p=p, dps=dps, dx="1e-10", nx=2, max_iter=max_iter, center=c)
    return Center(c=c, p=p, dps=dps, Zn=w.Zn, xr_idx=w.xr_idx, xr_m=w.xr_m, xr_e=w.xr_e)


class _Slot:
    def __init__(self, torch, device, idx):
        self.torch = torch
        self.stream = torch.cuda.Stream(device)
        self.ctx = nat.Context(device.index or 0)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.busy = False
        self.batch = None
        self.event = None
        self.idx = idx


class TileServer:
    """Continuous-batching server of perturbation tiles (FP32+exponent kernel
    by default)."""

    def __init__(self, centers, *, hbm_budget=120 * 2 ** 30, n_slots=None, max_slots=4,
                 max_batch_pixels=8 * 2 ** 20, mode="fe32", M=1000., bla_eps=1e-6,
                 device=0, keep_results=True, order="fifo"):
        """n_slots None: as many slots as the HBM budget holds batches of
        max_batch_pixels, at most max_slots (one persistent launch already
        fills the GPU; more concurrent launches only fill the tails).
        order "fifo" admits by arrival, "shortest" the smallest expected work
        first (``expected_work``), "hrrn" the highest response ratio
        (wait + S) / S first, S the expected service time (expected work over
        the work rate measured on finished batches): short requests first,
        and a long one once it has waited about its own service time."""
        import torch
        self.torch = torch
        self.device = torch.device("cuda", device)
        self.centers = centers
        self.hbm_budget = int(hbm_budget)
        self.reserved = 0
        self.mode = mode
        self.M = M
        self.bla_eps = bla_eps
        self.max_batch_pixels = int(max_batch_pixels)
        if n_slots is None:
            n_slots = max(1, min(int(max_slots),
                                 self.hbm_budget // (self.max_batch_pixels * BYTES_PER_PIXEL)))
        if order not in ("fifo", "shortest", "hrrn"):
            raise ValueError("order: 'fifo', 'shortest' or 'hrrn'")
        self.order = order
        self.work_rate = 0.0        # expected work per second of a batch, measured
        self.slots = [_Slot(torch, self.device, i) for i in range(n_slots)]
        # reference builds on a high-priority stream of their own: their
        # kernels are scheduled first as SMs free up, and launches wait for
        # them on the device (fsg_ref_derive_bla does not block the host)
        self.builder = nat.Context(self.device.index or 0)
        self.builder_stream = torch.cuda.Stream(self.device, priority=-1)
        self.builder.set_stream(self.builder_stream.cuda_stream)
        self.bases = {}                          # (centre, xr, max_iter) -> (Reference, bytes)
        self.cache = collections.OrderedDict()   # + kc bucket -> (derived Reference, bytes)
        self.cache_bytes = 0
        self.pending = collections.deque()
        self.done = []
        self.max_reserved = 0
        # False: results reach the host (pinned buffers) and are dropped once
        # counted, so that the pinned pool is recycled (load tests)
        self.keep_results = keep_results

    # ------------------------------------------------------------------
    def _view(self, req):
        cen = self.centers[req.center]
        with mpmath.workdps(cen.dps):
            dx = mpmath.mpf(req.dx)
            dx_xr = fsx.mpf_to_Xrange(dx)
            drift = fsx.mpc_to_Xrange(mpmath.mpc(req.offset[0], req.offset[1]) * dx)
            half = dx / 2
            shift = -mpmath.mpc(req.offset[0], req.offset[1]) * dx
            kc = max(abs(shift - mpmath.mpc(sx * half, sy * half))
                     for sx in (1, -1) for sy in (1, -1)) * mpmath.mpf(1.1)
            kc_xr = fsx.mpf_to_Xrange(kc)
            xr = bool(dx < settings.xrange_zoom_level)
        # dx = m 2^e with m in [0.5, 1): bucket scale 2^(e - 1)
        return dx_xr, drift, kc_xr, xr

    @staticmethod
    def kc_bucket(kc_xr):
        """kc rounded up to 2^(8 ceil(e / 8)) (kc = m 2^e, m in [0.5, 1)),
        0 below the smallest double (the reference's to_standard(kc))."""
        if kc_xr.e < -1074 or kc_xr.m == 0:
            return 0.0
        e8 = 8 * -(-kc_xr.e // 8)
        return math.ldexp(1.0, min(e8, 1023))

    def _base(self, req, xr):
        key = (req.center, xr, req.max_iter)
        if key not in self.bases:
            cen = self.centers[req.center]
            ref = nat.Reference(self.builder, cen.Zn, div_iter=req.max_iter + 1, order=cen.p,
                                xr_idx=cen.xr_idx if cen.xr_idx.size else None,
                                xr_m=cen.xr_m if cen.xr_idx.size else None,
                                xr_e=cen.xr_e if cen.xr_idx.size else None,
                                xr_paths=xr, calc_dzndc=True, scale_m=0.5, scale_e=1,
                                bla=False)
            nbytes = ref.len * (16 * 6 + 64)
            self.bases[key] = (ref, nbytes)
            self.cache_bytes += nbytes
        return self.bases[key][0]

    def _reference(self, req, dx_xr, kc_xr, xr):
        kc_b = self.kc_bucket(kc_xr)
        key = (req.center, xr, req.max_iter, kc_b)
        if key in self.cache:
            self.cache.move_to_end(key)
            return self.cache[key][0], 0
        ref = self._base(req, xr).derive_bla(kc_b, self.bla_eps, ctx=self.builder)
        nbytes = ref.bla_len * 112
        self.cache[key] = (ref, nbytes)
        self.cache_bytes += nbytes
        return ref, nbytes

    def _evict(self, need):
        while self.cache and self.reserved + self.cache_bytes + need > self.hbm_budget:
            key, (ref, nb) = self.cache.popitem(last=False)
            self.torch.cuda.synchronize(self.device)
            ref.free()
            self.cache_bytes -= nb

    def submit(self, req):
        req.arrival = req.arrival or time.perf_counter()
        self.pending.append(req)

    # ------------------------------------------------------------------
    def _launch(self, slot, batch):
        torch = self.torch
        tiles = []
        for req in batch:
            n = req.side * req.side
            dx_xr, drift, kc_xr, xr = req._view
            xs, ys = syn.image_axes(req.side, req.side)
            with torch.cuda.stream(slot.stream):
                b = {
                    "xs": torch.from_numpy(xs).to(self.device, non_blocking=False),
                    "ys": torch.from_numpy(ys).to(self.device, non_blocking=False),
                    "Z": torch.empty((2, n, 2), dtype=torch.float64, device=self.device),
                    "U": torch.empty(n, dtype=torch.int32, device=self.device),
                    "sr": torch.empty(n, dtype=torch.int8, device=self.device),
                    "si": torch.empty(n, dtype=torch.int32, device=self.device),
                    "pot": torch.empty(n, dtype=torch.float64, device=self.device),
                    "dem": torch.empty(n, dtype=torch.float64, device=self.device),
                }
            req._bufs = b
            t = nat.make_tile_ptrs(
                nx=req.side, ny=req.side, xs_ptr=b["xs"].data_ptr(), ys_ptr=b["ys"].data_ptr(),
                lin_mat=np.array([[1., -0.], [0., 1.]]), Z_ptr=b["Z"].data_ptr(), nZ=2,
                stop_reason_ptr=b["sr"].data_ptr(), stop_iter_ptr=b["si"].data_ptr(),
                U_ptr=b["U"].data_ptr(), ref=req._ref, dx_m=dx_xr.m, dx_e=dx_xr.e,
                drift_m=drift.m, drift_e=drift.e, i_dzndc=1,
                potential_ptr=b["pot"].data_ptr(), dem_ptr=b["dem"].data_ptr(),
                dzndc_scale_e=dx_xr.e - 1)
            tiles.append(t)
        calc = nat.make_calc(max_iter=batch[0].max_iter, M_divergence=self.M, mode=self.mode,
                             calc_dzndc=True, interior=False, bla=True,
                             xr_semantics=batch[0]._view[3])
        # the launch shape the autotuner cached for this kernel kind, if any
        calc = tune.apply(calc, True, tune._device_name(slot.ctx))
        slot.ctx.perturb_tiles(calc, tiles, nat.DEVICE)
        with torch.cuda.stream(slot.stream):
            for req in batch:
                b = req._bufs
                # dzndc was computed with the bucket scale 2^(e - 1): rescale to
                # dx on the device, then copy into pinned host memory
                ratio = 2.0 * req._view[0].m
                b["Z"][1].mul_(ratio)
                b["dem"].div_(ratio)
                req._host = {}
                for k, v in b.items():
                    if k in ("xs", "ys"):
                        continue
                    h = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
                    h.copy_(v, non_blocking=True)
                    req._host[k] = h
            slot.event = torch.cuda.Event()
            slot.event.record(slot.stream)
        slot.busy = True
        slot.batch = batch

    def _finish(self, slot):
        now = time.perf_counter()
        # the work rate of one slot, an average over the finished batches
        work = sum(self.expected_work(r) for r in slot.batch)
        dt = now - min(r.admitted for r in slot.batch)
        if dt > 0:
            rate = work / dt
            self.work_rate = rate if self.work_rate == 0 else 0.8 * self.work_rate + 0.2 * rate
        for req in slot.batch:
            h = req._host
            si = h["si"].numpy()
            req.pixel_iters = int(si.sum(dtype=np.int64))
            if self.keep_results:
                req.result = {"Z": h["Z"].numpy().view(np.complex128).reshape(2, -1),
                              "U": h["U"].numpy(), "stop_reason": h["sr"].numpy(),
                              "stop_iter": si, "potential": h["pot"].numpy(),
                              "dem": h["dem"].numpy()}
            req.done = now
            self.reserved -= req._bytes
            del req._bufs, req._host
            self.done.append(req)
        slot.busy = False
        slot.batch = None

    def expected_work(self, req):
        """Expected executed steps of a request: its pixels times the orbit
        periods up to max_iter times the steps of a period (about log2 p BLA
        steps and ten full steps; interior pixels run to max_iter)."""
        p = max(self.centers[req.center].p, 2)
        return req.side * req.side * (req.max_iter / p) * (math.log2(p) + 10.)

    def priority(self, req, now):
        """Sort key of the admission order (smallest first)."""
        if self.order == "hrrn" and self.work_rate > 0:
            service = self.expected_work(req) / self.work_rate
            return -(now - req.arrival + service) / service
        return self.expected_work(req)

    def _admit(self, slot):
        if self.order in ("shortest", "hrrn") and len(self.pending) > 1:
            now = time.perf_counter()
            self.pending = collections.deque(
                sorted(self.pending, key=lambda r: self.priority(r, now)))
        batch = []
        pixels = 0
        while self.pending:
            req = self.pending[0]
            n = req.side * req.side
            if batch and (pixels + n > self.max_batch_pixels
                          or req.max_iter != batch[0].max_iter
                          or self._view_cached(req)[3] != batch[0]._view[3]):
                break
            view = self._view_cached(req)
            need = n * BYTES_PER_PIXEL
            self._evict(need)
            if self.reserved + self.cache_bytes + need > self.hbm_budget:
                break           # wait for memory
            ref, _ = self._reference(req, view[0], view[2], view[3])
            req._ref = ref
            req._bytes = need
            self.reserved += need
            self.max_reserved = max(self.max_reserved, self.reserved + self.cache_bytes)
            req.admitted = time.perf_counter()
            self.pending.popleft()
            batch.append(req)
            pixels += n
        if batch:
            self._launch(slot, batch)

    def _view_cached(self, req):
        if not hasattr(req, "_view"):
            req._view = self._view(req)
        return req._view

    def step(self):
        """One pass of the server loop: retire finished batches, admit and
        launch new ones on free slots."""
        for slot in self.slots:
            if slot.busy and slot.event.query():
                self._finish(slot)
        for slot in self.slots:
            if not slot.busy and self.pending:
                self._admit(slot)

    def idle(self):
        return not self.pending and not any(s.busy for s in self.slots)

    def run(self, requests, realtime=True, timeout=None):
        """Serve ``requests`` (sorted by arrival offsets in seconds when
        realtime).  Returns the finished requests."""
        t0 = time.perf_counter()
        reqs = sorted(requests, key=lambda r: r.arrival)
        i = 0
        while i < len(reqs) or not self.idle():
            now = time.perf_counter()
            while i < len(reqs) and (not realtime or t0 + reqs[i].arrival <= now):
                r = reqs[i]
                r.arrival = t0 + r.arrival if realtime else now
                self.pending.append(r)
                i += 1
            self.step()
            if timeout is not None and now - t0 > timeout:
                raise TimeoutError("serving loop timed out")
            if not any(s.busy for s in self.slots) and i < len(reqs) and realtime:
                time.sleep(max(0.0, min(0.002, t0 + reqs[i].arrival - now)))
            else:
                time.sleep(0.0002)
        return self.done

    def close(self):
        self.torch.cuda.synchronize(self.device)
        for _, (ref, _) in self.cache.items():
            ref.free()
        self.cache.clear()
        for _, (ref, _) in self.bases.items():
            ref.free()
        self.bases.clear()
        for s in self.slots:
            s.ctx.close()
        self.builder.close()


def request_stream(centers, n, rate, seed, sides=(256, 512, 1024, 2048),
                   log10_width=(-1000, -10), max_iter=200000):
    """Seeded Poisson stream: exponential gaps at ``rate`` per second, side
    uniform in ``sides``, width log-uniform in 10^log10_width around one of the
    centres, offset < 0.1 width."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        ci = int(rng.integers(0, len(centers)))
        side = int(rng.choice(sides))
        e = rng.uniform(*log10_width)
        mant = 10 ** (e - math.floor(e))
        dx = f"{mant:.6f}e{int(math.floor(e))}"
        off = tuple(float(v) for v in rng.uniform(-0.1, 0.1, 2))
        out.append(Request(rid=k, center=ci, side=side, dx=dx, offset=off, max_iter=max_iter,
                           arrival=t))
    return out
