"""
ctypes binding of libfsgpu.so (declared in include/fsgpu.h).

The GPU library is the only compute path of this package: there is no CPU
fallback.  Loading fails with an explicit error when the library has not been
built (``python -c "import __graft_entry__ as g; g.build()"``) or when no CUDA
device is visible.
"""
import ctypes as ct
import os
import threading

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libfsgpu.so")

FSG_OK = 0
FSG_INTERRUPTED = 1
FSG_BUDGET = 2
FSG_ERR_ARG = -1
FSG_ERR_CUDA = -2
FSG_ERR_NOMEM = -3
FSG_ERR_NODEV = -4
FSG_ERR_LIMIT = -5
FSG_NOALLOC_MAX_TILES = 64
FSG_MN_MAX_EXP = 32
FSG_MAX_ITER_LIMIT = (1 << 30) - 1

MODE_FP64 = 0
MODE_XR64 = 1
MODE_FE32 = 2
MODES = {"fp64": MODE_FP64, "xr64": MODE_XR64, "fe32": MODE_FE32}

HOST = 0
DEVICE = 1

P = ct.c_void_p
I32, I64, F64 = ct.c_int32, ct.c_int64, ct.c_double


class RefDesc(ct.Structure):
    _fields_ = [
        ("Zn", P), ("len", I64), ("div_iter", I64), ("order", I64),
        ("n_xr", I32), ("xr_idx", P), ("xr_m", P), ("xr_e", P),
        ("flavor", I32), ("xr_paths", I32), ("calc_dzndc", I32), ("calc_dzndz", I32),
        ("scale_m", F64), ("scale_e", I32), ("bla", I32), ("kc", F64), ("bla_eps", F64),
        ("nexp", I32),
    ]


class Calc(ct.Structure):
    _fields_ = [
        ("max_iter", I64), ("M_divergence", F64), ("epsilon_stationnary", F64),
        ("mode", I32), ("calc_dzndc", I32), ("interior", I32), ("bla", I32),
        ("flavor", I32), ("xr_semantics", I32), ("nexp", I32),
        ("backshift", I32), ("calc_d2zndc2", I32), ("block", I32), ("ctas_per_sm", I32),
        ("iter_budget", I64), ("claim_order", I32),
    ]


class Tile(ct.Structure):
    _fields_ = [
        ("nx", I32), ("ny", I32), ("xs", P), ("ys", P), ("pix", P), ("lin_mat", F64 * 4),
        ("center_re", F64), ("center_im", F64), ("dx", F64),
        ("dx_m", F64), ("dx_e", I32), ("drift_re", F64), ("drift_im", F64),
        ("drift_e", I32), ("drifty_m", F64), ("drifty_e", I32), ("ref", P),
        ("Z", P), ("nZ", I32), ("i_dzndz", I32), ("i_dzndc", I32),
        ("U", P), ("stop_reason", P), ("stop_iter", P), ("potential", P), ("dem", P),
        ("dzndc_scale_e", I32), ("i_znorbit", I32),
        ("proj", I32), ("proj_h", F64), ("proj_ht_re", F64), ("proj_ht_im", F64),
    ]


class FieldlinesArgs(ct.Structure):
    _fields_ = [
        ("npix", I64), ("model", I32), ("c", P), ("z", P), ("nu_frac", P), ("n", P),
        ("is_backward", I32), ("backshift", I32), ("n_iter", I32), ("k", P), ("phi", P),
        ("out", P),
    ]


class NormalArgs(ct.Structure):
    _fields_ = [
        ("npix", I64), ("kind", I32), ("zn", P), ("dzndc", P), ("d2zndc2", P), ("skew", P),
        ("out", P),
    ]


class Stats(ct.Structure):
    _fields_ = [
        ("kernel_ms", F64), ("pixels", I64), ("pixel_iters", I64),
        ("full_steps", I64), ("bla_steps", I64), ("rebases", I64),
    ]


_lock = threading.Lock()
_lib = None

#: exported symbols (include/fsgpu.h)
SYMBOLS = [
    "fsg_version", "fsg_ctx_create", "fsg_ctx_destroy", "fsg_last_error",
    "fsg_set_stream", "fsg_sync", "fsg_ref_create", "fsg_ref_destroy",
    "fsg_ref_info", "fsg_ref_download", "fsg_std_tiles", "fsg_perturb_tiles",
    "fsg_last_stats", "fsg_cancel", "fsg_clear_cancel", "fsg_peak_flops",
    "fsg_std_tiles_noalloc", "fsg_ref_derive_bla", "fsg_postproc_fieldlines",
    "fsg_postproc_normal", "fsg_serve_open", "fsg_submit", "fsg_poll", "fsg_serve_info",
    "fsg_serve_close",
]

FSG_SERVE_FIFO = 0
FSG_SERVE_SHORTEST = 1
FSG_SERVE_HRRN = 2
FSG_ORDER_PIXELS = 0
FSG_ORDER_LONGEST = 1
FSG_PENDING = 3


class ServeStats(ct.Structure):
    _fields_ = [("queued", I64), ("running", I64), ("reserved_bytes", I64),
                ("peak_reserved_bytes", I64), ("budget_bytes", I64), ("slots", I32)]

FSG_FIELDLINES_MAX_ITER = 64


class GPUError(RuntimeError):
    pass


def load():
    """Load libfsgpu.so and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise GPUError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c \"import __graft_entry__ as g; g.build()\"` "
                "(this package has no CPU fallback)")
        L = ct.CDLL(LIB_PATH)
        L.fsg_version.restype = ct.c_char_p
        L.fsg_ctx_create.argtypes = [ct.c_int, ct.POINTER(P)]
        L.fsg_ctx_destroy.argtypes = [P]
        L.fsg_last_error.argtypes = [P]
        L.fsg_last_error.restype = ct.c_char_p
        L.fsg_set_stream.argtypes = [P, P]
        L.fsg_sync.argtypes = [P]
        L.fsg_ref_create.argtypes = [P, ct.POINTER(RefDesc), ct.POINTER(P)]
        L.fsg_ref_destroy.argtypes = [P, P]
        L.fsg_ref_derive_bla.argtypes = [P, P, ct.c_double, ct.c_double, ct.POINTER(P)]
        L.fsg_ref_info.argtypes = [P, ct.POINTER(I64), ct.POINTER(I64), ct.POINTER(I32)]
        L.fsg_ref_download.argtypes = [P, P, ct.c_int, P, P]
        L.fsg_std_tiles.argtypes = [P, ct.POINTER(Calc), ct.POINTER(Tile), I32, I32]
        L.fsg_perturb_tiles.argtypes = [P, ct.POINTER(Calc), ct.POINTER(Tile), I32, I32]
        L.fsg_last_stats.argtypes = [P, ct.POINTER(Stats)]
        L.fsg_peak_flops.argtypes = [P, I32, ct.POINTER(F64)]
        L.fsg_cancel.argtypes = [P]
        L.fsg_postproc_fieldlines.argtypes = [P, ct.POINTER(FieldlinesArgs), I32]
        L.fsg_postproc_normal.argtypes = [P, ct.POINTER(NormalArgs), I32]
        L.fsg_clear_cancel.argtypes = [P]
        L.fsg_serve_open.argtypes = [P, I64, I32, I32]
        L.fsg_submit.argtypes = [P, ct.POINTER(Calc), ct.POINTER(Tile), I32, F64, ct.POINTER(I64)]
        L.fsg_poll.argtypes = [P, I64]
        L.fsg_serve_info.argtypes = [P, ct.POINTER(ServeStats)]
        L.fsg_serve_close.argtypes = [P]
        _lib = L
        return L


def _p(a):
    return None if a is None else ct.c_void_p(a.ctypes.data)


class Context:
    """One CUDA device context of the library (stream, counters, cancel flag)."""

    def __init__(self, device=0):
        self.L = load()
        h = P()
        rc = self.L.fsg_ctx_create(int(device), ct.byref(h))
        if rc != FSG_OK:
            raise GPUError(f"fsg_ctx_create failed with code {rc} "
                           "(no CUDA device visible?)")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.fsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc, what):
        if rc == FSG_OK or rc == FSG_INTERRUPTED or rc == FSG_BUDGET:
            return rc
        msg = self.L.fsg_last_error(self.h).decode()
        raise GPUError(f"{what} failed (code {rc}): {msg}")

    def set_stream(self, stream_ptr):
        self.check(self.L.fsg_set_stream(self.h, ct.c_void_p(stream_ptr or 0)), "fsg_set_stream")

    def sync(self):
        return self.check(self.L.fsg_sync(self.h), "fsg_sync")

    def cancel(self):
        self.L.fsg_cancel(self.h)

    def clear_cancel(self):
        self.L.fsg_clear_cancel(self.h)

    def peak_tflops(self, fp64=False):
        """Measured FMA-pipe throughput (TFLOP/s) of this GPU."""
        v = F64()
        self.check(self.L.fsg_peak_flops(self.h, int(bool(fp64)), ct.byref(v)), "fsg_peak_flops")
        return v.value

    def stats(self):
        s = Stats()
        self.check(self.L.fsg_last_stats(self.h, ct.byref(s)), "fsg_last_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    # ------------------------------------------------------------------
    def std_tiles(self, calc, tiles, where=HOST):
        arr = (Tile * len(tiles))(*tiles)
        return self.check(self.L.fsg_std_tiles(self.h, ct.byref(calc), arr, len(tiles), where),
                          "fsg_std_tiles")

    def perturb_tiles(self, calc, tiles, where=HOST):
        arr = (Tile * len(tiles))(*tiles)
        return self.check(self.L.fsg_perturb_tiles(self.h, ct.byref(calc), arr, len(tiles), where),
                          "fsg_perturb_tiles")

    # ------------------------------------------------------------------
    # serving queue (fsg_serve_open / fsg_submit / fsg_poll)
    def serve_open(self, hbm_budget, slots, order="fifo"):
        o = {"fifo": FSG_SERVE_FIFO, "shortest": FSG_SERVE_SHORTEST, "hrrn": FSG_SERVE_HRRN}[order]
        self._serve_keep = {}
        self.check(self.L.fsg_serve_open(self.h, int(hbm_budget), int(slots), o),
                   "fsg_serve_open")

    def submit(self, calc, tiles, expected_work=0.0, keep=None):
        """Queue host-buffer tiles; returns the ticket.  The tiles' arrays
        (and ``keep``) are held until the request is polled finished."""
        arr = (Tile * len(tiles))(*tiles)
        t = I64(0)
        self.check(self.L.fsg_submit(self.h, ct.byref(calc), arr, len(tiles),
                                     float(expected_work), ct.byref(t)), "fsg_submit")
        self._serve_keep[t.value] = (arr, calc, tiles, keep)
        return t.value

    def poll(self, ticket):
        """None while the request is queued or running, else its outcome
        (FSG_OK, FSG_BUDGET or FSG_INTERRUPTED; errors raise)."""
        rc = self.L.fsg_poll(self.h, int(ticket))
        if rc == FSG_PENDING:
            return None
        self._serve_keep.pop(int(ticket), None)
        return self.check(rc, "fsg_poll")

    def serve_info(self):
        st = ServeStats()
        self.check(self.L.fsg_serve_info(self.h, ct.byref(st)), "fsg_serve_info")
        return {k: getattr(st, k) for k, _ in ServeStats._fields_}

    def serve_close(self):
        self.check(self.L.fsg_serve_close(self.h), "fsg_serve_close")
        self._serve_keep = {}

    # ------------------------------------------------------------------
    def fieldlines(self, *, model, c, z, nu_frac, n, k, phi, is_backward, backshift):
        """Fieldlines_pp on the device (host arrays in and out): model 0 for
        z^2 + c, n for z^n + c, -flavor for the Burning Ship family; z the
        start points (complex; Burning Ship x + i y)."""
        c = np.ascontiguousarray(c, dtype=np.complex128)
        z = np.ascontiguousarray(z, dtype=np.complex128)
        nu = np.ascontiguousarray(nu_frac, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.int32)
        k = np.ascontiguousarray(k, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        out = np.empty(c.size, dtype=np.float64)
        a = FieldlinesArgs()
        a.npix, a.model = c.size, int(model)
        a.c, a.z, a.nu_frac, a.n = _p(c), _p(z), _p(nu), _p(nn)
        a.is_backward, a.backshift, a.n_iter = int(bool(is_backward)), int(backshift), k.size
        a.k, a.phi, a.out = _p(k), _p(phi), _p(out)
        self.check(self.L.fsg_postproc_fieldlines(self.h, ct.byref(a), HOST),
                   "fsg_postproc_fieldlines")
        return out

    def normal(self, *, kind, zn, dzndc, d2zndc2=None, skew=None):
        """DEM_normal_pp on the device: kind 0 "potential", 1 "Milnor", 2 the
        Burning Ship family (dzndc = the 4 Jacobian rows).  Returns the
        complex unit normal."""
        zn = np.ascontiguousarray(zn, dtype=np.complex128)
        dz = np.ascontiguousarray(dzndc, dtype=np.float64 if kind == 2 else np.complex128)
        d2 = None if d2zndc2 is None else np.ascontiguousarray(d2zndc2, dtype=np.complex128)
        sk = None if skew is None else np.ascontiguousarray(skew, dtype=np.float64).ravel()
        out = np.empty(zn.size, dtype=np.complex128)
        a = NormalArgs()
        a.npix, a.kind = zn.size, int(kind)
        a.zn, a.dzndc, a.d2zndc2, a.skew, a.out = _p(zn), _p(dz), _p(d2), _p(sk), _p(out)
        self.check(self.L.fsg_postproc_normal(self.h, ct.byref(a), HOST), "fsg_postproc_normal")
        return out


class Reference:
    """A reference orbit resident on the device with its derived tables
    (derivative paths, BLA tree, fe copies), built by fsg_ref_create."""

    def __init__(self, ctx, Zn, *, div_iter, order, flavor=0, xr_idx=None, xr_m=None,
                 xr_e=None, xr_paths=False, calc_dzndc=True, calc_dzndz=False,
                 scale_m=1.0, scale_e=0, bla=True, kc=0.0, bla_eps=1e-6, nexp=0):
        self.ctx = ctx
        self.Zn = np.ascontiguousarray(Zn, dtype=np.complex128)
        n_xr = 0 if xr_idx is None else len(xr_idx)
        self._keep = [self.Zn]
        d = RefDesc()
        d.Zn = _p(self.Zn)
        d.len = self.Zn.size
        d.div_iter = int(div_iter)
        d.order = int(order) if order is not None else 0
        d.n_xr = n_xr
        if n_xr:
            idx = np.ascontiguousarray(xr_idx, dtype=np.int32)
            m = np.ascontiguousarray(xr_m, dtype=np.complex128 if flavor == 0 else np.float64)
            e = np.ascontiguousarray(xr_e, dtype=np.int32)
            self._keep += [idx, m, e]
            d.xr_idx, d.xr_m, d.xr_e = _p(idx), _p(m), _p(e)
        d.flavor = int(flavor)
        d.xr_paths = int(bool(xr_paths))
        d.calc_dzndc = int(bool(calc_dzndc))
        d.calc_dzndz = int(bool(calc_dzndz))
        d.scale_m, d.scale_e = float(scale_m), int(scale_e)
        d.bla = int(bool(bla))
        d.kc = float(kc)
        d.bla_eps = float(bla_eps)
        d.nexp = int(nexp)
        h = P()
        ctx.check(ctx.L.fsg_ref_create(ctx.h, ct.byref(d), ct.byref(h)), "fsg_ref_create")
        self.h = h
        self.flavor = flavor
        self.nexp = int(nexp)
        self.xr_paths = bool(xr_paths)
        ln, bl, st = I64(), I64(), I32()
        ctx.L.fsg_ref_info(h, ct.byref(ln), ct.byref(bl), ct.byref(st))
        self.len, self.bla_len, self.stages = ln.value, bl.value, st.value

    def derive_bla(self, kc, bla_eps=1e-6, ctx=None):
        """A Reference that shares this one's orbit and derivative tables and
        owns a BLA tree built for ``kc`` (fsg_ref_derive_bla).  It keeps this
        reference alive."""
        ctx = ctx or self.ctx
        h = P()
        ctx.check(ctx.L.fsg_ref_derive_bla(ctx.h, self.h, float(kc), float(bla_eps), ct.byref(h)),
                  "fsg_ref_derive_bla")
        r = Reference.__new__(Reference)
        r.ctx, r.h, r._base, r._keep = ctx, h, self, []
        r.Zn, r.flavor, r.xr_paths, r.nexp = self.Zn, self.flavor, self.xr_paths, self.nexp
        ln, bl, st = I64(), I64(), I32()
        ctx.L.fsg_ref_info(h, ct.byref(ln), ct.byref(bl), ct.byref(st))
        r.len, r.bla_len, r.stages = ln.value, bl.value, st.value
        return r

    def free(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.ctx.check(self.ctx.L.fsg_ref_destroy(self.ctx.h, self.h), "fsg_ref_destroy")
        self.h = None
        self._base = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def download(self, which):
        """Tables built on the device: 'dzndc', 'dzndz', 'bla', 'bs_paths',
        'bs_xpaths' (Xrange branch: mantissas and exponents)."""
        n = self.len
        L, c = self.ctx.L, self.ctx
        if which in ("dzndc", "dzndz"):
            k = 0 if which == "dzndc" else 1
            m = np.zeros(n + k, dtype=np.complex128)
            e = np.zeros(n + k, dtype=np.int32)
            c.check(L.fsg_ref_download(c.h, self.h, k, _p(m), _p(e)), "fsg_ref_download")
            return (m, e) if self.xr_paths else m
        if which == "bla":
            r = np.zeros(self.bla_len)
            if self.flavor == 0:
                M = np.zeros(2 * self.bla_len, dtype=np.complex128)
            else:
                M = np.zeros(8 * self.bla_len)
            c.check(L.fsg_ref_download(c.h, self.h, 2, _p(M), _p(r)), "fsg_ref_download")
            return M, r
        if which == "bs_paths":
            out = np.zeros(4 * n)
            c.check(L.fsg_ref_download(c.h, self.h, 3, _p(out), None), "fsg_ref_download")
            return out.reshape(4, n)
        if which == "bs_xpaths":
            m = np.zeros(4 * n)
            e = np.zeros(4 * n, dtype=np.int32)
            c.check(L.fsg_ref_download(c.h, self.h, 4, _p(m), _p(e)), "fsg_ref_download")
            return m.reshape(4, n), e.reshape(4, n)
        raise ValueError(which)


def _set_proj(t, proj):
    """proj = (kind, h, Re ht, Im ht) of projection.kernel_params, or None
    (Cartesian)."""
    kind, h, hr, hi = proj if proj is not None else (0, 0., 0., 0.)
    t.proj, t.proj_h, t.proj_ht_re, t.proj_ht_im = int(kind), float(h), float(hr), float(hi)


def make_tile(*, lin_mat, Z, stop_reason, stop_iter, xs=None, ys=None, pix=None, U=None,
              ref=None, center=0j, dx=0.0, dx_m=0.0, dx_e=0, drift_m=0j, drift_e=0,
              drifty_m=0.0, drifty_e=0, i_dzndz=-1, i_dzndc=-1, potential=None,
              dem=None, keep=None, dzndc_scale_e=0, i_znorbit=0, proj=None):
    """Fill a Tile from numpy (host) arrays: either the axes xs / ys of a
    rectangle or an explicit complex128 list of pixel positions ``pix``.
    Inputs are taken as contiguous copies when needed (kept with the Tile);
    outputs are written in place and must be C-contiguous of the kernels'
    dtypes."""
    t = Tile()
    if pix is not None:
        pix = np.ascontiguousarray(pix, dtype=np.complex128)
        t.nx, t.ny = int(pix.size), 1
        t.pix = _p(pix)
    else:
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        ys = np.ascontiguousarray(ys, dtype=np.float64)
        t.nx, t.ny = len(xs), len(ys)
        t.xs, t.ys = _p(xs), _p(ys)
    t._inputs = (xs, ys, pix)
    for name, a, dts in (("Z", Z, (np.complex128, np.float64)), ("U", U, (np.int32,)),
                         ("stop_reason", stop_reason, (np.int8,)),
                         ("stop_iter", stop_iter, (np.int32,)),
                         ("potential", potential, (np.float64,)), ("dem", dem, (np.float64,))):
        if a is not None and (not a.flags.c_contiguous or a.dtype not in dts):
            raise ValueError(f"{name}: a C-contiguous array of dtype {dts[0].__name__} is needed")
    lm = np.asarray(lin_mat, dtype=np.float64).ravel()
    for k in range(4):
        t.lin_mat[k] = lm[k]
    t.center_re, t.center_im, t.dx = complex(center).real, complex(center).imag, float(dx)
    t.dx_m, t.dx_e = float(dx_m), int(dx_e)
    t.drift_re, t.drift_im, t.drift_e = complex(drift_m).real, complex(drift_m).imag, int(drift_e)
    t.drifty_m, t.drifty_e = float(drifty_m), int(drifty_e)
    t.ref = ref.h if ref is not None else None
    t.Z = _p(Z)
    t.nZ = Z.shape[0]
    t.i_dzndz, t.i_dzndc = int(i_dzndz), int(i_dzndc)
    t.U = _p(U)
    t.stop_reason, t.stop_iter = _p(stop_reason), _p(stop_iter)
    t.potential, t.dem = _p(potential), _p(dem)
    t.dzndc_scale_e = int(dzndc_scale_e)
    t.i_znorbit = int(i_znorbit)
    _set_proj(t, proj)
    if keep is not None:
        keep.extend([xs, ys, pix, Z, U, stop_reason, stop_iter, potential, dem])
    return t


def make_tile_ptrs(*, nx, ny, xs_ptr, ys_ptr, lin_mat, Z_ptr, nZ, stop_reason_ptr,
                   stop_iter_ptr, U_ptr=0, ref=None, center=0j, dx=0.0, dx_m=0.0,
                   dx_e=0, drift_m=0j, drift_e=0, drifty_m=0.0, drifty_e=0, i_dzndz=-1,
                   i_dzndc=-1, potential_ptr=0, dem_ptr=0, dzndc_scale_e=0, i_znorbit=0,
                   proj=None):
    """Fill a Tile from raw device pointers (ints)."""
    t = Tile()
    t.nx, t.ny = int(nx), int(ny)
    t.xs, t.ys = xs_ptr, ys_ptr
    lm = np.asarray(lin_mat, dtype=np.float64).ravel()
    for k in range(4):
        t.lin_mat[k] = lm[k]
    t.center_re, t.center_im, t.dx = complex(center).real, complex(center).imag, float(dx)
    t.dx_m, t.dx_e = float(dx_m), int(dx_e)
    t.drift_re, t.drift_im, t.drift_e = complex(drift_m).real, complex(drift_m).imag, int(drift_e)
    t.drifty_m, t.drifty_e = float(drifty_m), int(drifty_e)
    t.ref = ref.h if ref is not None else None
    t.Z, t.nZ = Z_ptr, int(nZ)
    t.i_dzndz, t.i_dzndc = int(i_dzndz), int(i_dzndc)
    t.U = U_ptr or None
    t.stop_reason, t.stop_iter = stop_reason_ptr, stop_iter_ptr
    t.potential, t.dem = potential_ptr or None, dem_ptr or None
    t.dzndc_scale_e = int(dzndc_scale_e)
    t.i_znorbit = int(i_znorbit)
    _set_proj(t, proj)
    return t


def make_calc(*, max_iter, M_divergence, epsilon_stationnary=0.0, mode="fp64",
              calc_dzndc=True, interior=False, bla=True, flavor=0, xr_semantics=False,
              nexp=0, backshift=0, calc_d2zndc2=False, block=0, ctas_per_sm=0,
              iter_budget=0, claim_order="pixels"):
    c = Calc()
    c.max_iter = int(max_iter)
    c.M_divergence = float(M_divergence)
    c.epsilon_stationnary = float(epsilon_stationnary)
    c.mode = MODES[mode] if isinstance(mode, str) else int(mode)
    c.calc_dzndc = int(bool(calc_dzndc))
    c.interior = int(bool(interior))
    c.bla = int(bool(bla))
    c.flavor = int(flavor)
    c.xr_semantics = int(bool(xr_semantics))
    c.nexp = int(nexp)
    c.backshift = int(backshift)
    c.calc_d2zndc2 = int(bool(calc_d2zndc2))
    c.block = int(block)
    c.ctas_per_sm = int(ctas_per_sm)
    c.iter_budget = int(iter_budget)
    c.claim_order = {"pixels": FSG_ORDER_PIXELS, "longest": FSG_ORDER_LONGEST}[claim_order] \
        if isinstance(claim_order, str) else int(claim_order)
    return c
