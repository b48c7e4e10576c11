"""
ctypes front-end of the CPU oracle (fs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, as the result the GPU path is compared with.  The
product package never imports it.  Array conventions follow the reference: complex128 arrays, Z[nZ, npts],
U int32[nU, npts], stop_reason int8[1, npts], stop_iter int32[1, npts].
"""
import ctypes as ct
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfs_oracle.so")
FAST_LIB_PATH = os.path.join(HERE, "_build", "libfs_oracle_fast.so")
_lock = threading.Lock()
_libs = {}

P = ct.c_void_p
I32, I64, F64 = ct.c_int32, ct.c_int64, ct.c_double


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(fast=False):
    """The strict build (the parity checker), or with ``fast`` the
    -ffast-math build that times the CPU baseline (oracle/Makefile)."""
    with _lock:
        if fast not in _libs:
            path = FAST_LIB_PATH if fast else LIB_PATH
            src = os.path.join(HERE, "fs_oracle.c")
            if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
                build()
            L = ct.CDLL(path)
            _declare(L)
            _libs[fast] = L
        return _libs[fast]


class PM2Args(ct.Structure):
    _fields_ = [
        ("Zn", P), ("ref_len", I64), ("ref_div_iter", I64), ("ref_order", I64),
        ("n_xr", I32), ("xr_idx", P), ("xr_re", P), ("xr_im", P), ("xr_e", P),
        ("dZndc", P), ("dZndc_re", P), ("dZndc_im", P), ("dZndc_e", P),
        ("dZndz", P), ("dZndz_re", P), ("dZndz_im", P), ("dZndz_e", P),
        ("M_bla", P), ("r_bla", P), ("stages_bla", I32), ("bla_on", I32),
        ("max_iter", I64), ("M2", F64), ("eps2", F64), ("xr_mode", I32),
        ("i_dzndz", I32), ("i_dzndc", I32), ("dzndz_carryover", I32),
        ("lin_mat", F64 * 4), ("dx_m", F64), ("dx_e", I32),
        ("drift_re", F64), ("drift_im", F64), ("drift_e", I32), ("nexp", I32),
        ("backshift", I32), ("i_znorbit", I32),
    ]


class PBSXArgs(ct.Structure):
    _fields_ = [
        ("Zn", P), ("ref_len", I64), ("ref_div_iter", I64), ("ref_order", I64),
        ("n_xr", I32), ("xr_idx", P), ("xr_xm", P), ("xr_xe", P), ("xr_ym", P), ("xr_ye", P),
        ("path_m", P), ("path_e", P),
        ("M_bla", P), ("r_bla", P), ("stages_bla", I32), ("bla_on", I32),
        ("max_iter", I64), ("M2", F64), ("flavor", I32), ("calc_hessian", I32),
        ("lin_mat", F64 * 4), ("dx_m", F64), ("dx_e", I32),
        ("driftx_m", F64), ("driftx_e", I32), ("drifty_m", F64), ("drifty_e", I32),
    ]


class PBSArgs(ct.Structure):
    _fields_ = [
        ("Zn", P), ("ref_len", I64), ("ref_div_iter", I64), ("ref_order", I64),
        ("dXa", P), ("dXb", P), ("dYa", P), ("dYb", P),
        ("M_bla", P), ("r_bla", P), ("stages_bla", I32), ("bla_on", I32),
        ("max_iter", I64), ("M2", F64), ("flavor", I32), ("calc_hessian", I32),
        ("lin_mat", F64 * 4), ("dx_m", F64), ("dx_e", I32),
        ("driftx_m", F64), ("driftx_e", I32), ("drifty_m", F64), ("drifty_e", I32),
        ("backshift", I32), ("i_xnorbit", I32),
    ]


def _declare(L):
    L.orc_xr_binop.argtypes = [ct.c_int, I64] + [P] * 9
    L.orc_std_m2.argtypes = [I64, P, F64, F64, P, F64, I64, F64, F64, P, P, P, I32, I32, I32]
    L.orc_std_m2.restype = ct.c_int
    L.orc_std_bs.argtypes = [I64, P, F64, F64, P, F64, I32, I64, F64, P, P, P, I32, I32]
    L.orc_std_bs.restype = ct.c_int
    L.orc_stages_bla.argtypes = [I64]
    L.orc_stages_bla.restype = I32
    L.orc_make_bla_m2.argtypes = [P, I64, F64, F64, P, P, I32]
    L.orc_make_bla_m2.restype = I32
    L.orc_make_bla_bs.argtypes = [P, I64, I32, F64, F64, P, P]
    L.orc_make_bla_bs.restype = I32
    L.orc_dzndc_path_m2.argtypes = [P, I64, I64, I64, I32, I32, P, P, P, P,
                                    F64, I32, P, P, P, P, I32]
    L.orc_dzndz_path_m2.argtypes = [P, I64, I64, I32, I32, P, P, P, P, P, P, P, P, I32]
    L.orc_std_mn.argtypes = [I64, P, F64, F64, P, F64, I64, F64, F64, I32, P, P, P, I32, I32,
                             I32]
    L.orc_std_mn.restype = ct.c_int
    L.orc_dzndc_path_bs.argtypes = [P, I64, I64, I64, I32, F64, P, P, P, P]
    L.orc_perturb_m2.argtypes = [ct.POINTER(PM2Args), I64, P, P, I32, P, P, P]
    L.orc_perturb_m2.restype = ct.c_int
    L.orc_perturb_bs.argtypes = [ct.POINTER(PBSArgs), I64, P, P, I32, P, P, P]
    L.orc_perturb_bs.restype = ct.c_int
    L.orc_dzndc_path_bs_xr.argtypes = [P, I64, I64, I64, I32, F64, I32, I32, P, P, P, P, P,
                                       P, P]
    L.orc_perturb_bs_xr.argtypes = [ct.POINTER(PBSXArgs), I64, P, P, I32, P, P, P]
    L.orc_perturb_bs_xr.restype = ct.c_int


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ---------------------------------------------------------------------------
# Xrange arithmetic
# ---------------------------------------------------------------------------
XR_OPS = {"add": 0, "mul": 1, "abs2": 2, "to_standard": 3, "add_std": 4,
          "from_std": 5}


def xr_binop(op, am, ae, bm=None, be=None):
    am = _c(am, np.complex128)
    n = am.size
    ae = _c(ae, np.int32)
    bm = _c(am if bm is None else bm, np.complex128)
    be = _c(ae if be is None else be, np.int32)
    are, aim = _c(am.real, np.float64), _c(am.imag, np.float64)
    bre, bim = _c(bm.real, np.float64), _c(bm.imag, np.float64)
    ore, oim = np.empty(n), np.empty(n)
    oe = np.empty(n, dtype=np.int32)
    lib().orc_xr_binop(XR_OPS[op], n, _p(are), _p(aim), _p(ae), _p(bre), _p(bim),
                       _p(be), _p(ore), _p(oim), _p(oe))
    return _cx(ore, oim), oe


def _cx(re, im):
    out = np.empty(re.shape, dtype=np.complex128)
    out.real, out.imag = re, im
    return out


# ---------------------------------------------------------------------------
# Standard loops
# ---------------------------------------------------------------------------
def std_m2(pix, center, lin_mat, dx, max_iter, M, eps, calc_d2zndc2=False, backshift=0):
    """Standard power-2 loop; Z rows zn, dzndz, dzndc, [d2zndc2], [zn_orbit]
    (zn_orbit when backshift > 0, the reference's calc_orbit)."""
    pix = _c(pix, np.complex128)
    n = pix.size
    nZ = 3 + int(bool(calc_d2zndc2)) + int(backshift > 0)
    Z = np.zeros((nZ, n), dtype=np.complex128)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lm = _c(lin_mat, np.float64).ravel()
    lib().orc_std_m2(n, _p(pix), center.real, center.imag, _p(lm), dx,
                     max_iter, M * M, eps * eps, _p(Z), _p(si), _p(sr), nZ,
                     int(bool(calc_d2zndc2)), int(backshift))
    return Z, si, sr


def std_mn(pix, center, lin_mat, dx, max_iter, M, eps, nexp, calc_d2zndc2=False, backshift=0):
    """Standard power-n Mandelbrot (models/mandelbrot_Mn.py:317-355); rows as
    std_m2."""
    pix = _c(pix, np.complex128)
    n = pix.size
    nZ = 3 + int(bool(calc_d2zndc2)) + int(backshift > 0)
    Z = np.zeros((nZ, n), dtype=np.complex128)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lm = _c(lin_mat, np.float64).ravel()
    lib().orc_std_mn(n, _p(pix), center.real, center.imag, _p(lm), dx,
                     max_iter, M * M, eps * eps, int(nexp), _p(Z), _p(si), _p(sr), nZ,
                     int(bool(calc_d2zndc2)), int(backshift))
    return Z, si, sr


def std_bs(pix, center, lin_mat, dx, flavor, max_iter, M, backshift=0):
    """Standard Burning Ship loop; rows xn, yn, dxnda, dxndb, dynda, dyndb,
    [xn_orbit, yn_orbit]."""
    pix = _c(pix, np.complex128)
    n = pix.size
    nZ = 8 if backshift > 0 else 6
    Z = np.zeros((nZ, n), dtype=np.float64)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lm = _c(lin_mat, np.float64).ravel()
    lib().orc_std_bs(n, _p(pix), center.real, center.imag, _p(lm), dx, flavor,
                     max_iter, M * M, _p(Z), _p(si), _p(sr), nZ, int(backshift))
    return Z, si, sr


# ---------------------------------------------------------------------------
# Orbit-derived tables
# ---------------------------------------------------------------------------
def make_bla_m2(Zn, kc, eps, nexp=0):
    """nexp 0: the power-2 model (dfdz = 2 z); n >= 2: power n (n z^(n-1))."""
    Zn = _c(Zn, np.complex128)
    L = Zn.size // 8
    M = np.zeros(2 * L * 2, dtype=np.complex128)
    r = np.zeros(2 * L, dtype=np.float64)
    st = lib().orc_make_bla_m2(_p(Zn), Zn.size, kc, eps, _p(M), _p(r), int(nexp))
    return M, r, 2 * L, st


def make_bla_bs(Zn, flavor, kc, eps):
    Zn = _c(Zn, np.complex128)
    L = Zn.size // 8
    M = np.zeros(2 * L * 8, dtype=np.float64)
    r = np.zeros(2 * L, dtype=np.float64)
    st = lib().orc_make_bla_bs(_p(Zn), Zn.size, flavor, kc, eps, _p(M), _p(r))
    return M, r, 2 * L, st


def _xr_table(xr_idx, xr_m, xr_e):
    xr_idx = _c(np.zeros(0) if xr_idx is None else xr_idx, np.int32)
    xr_m = _c(np.zeros(max(xr_idx.size, 1)) if xr_m is None else xr_m, np.complex128)
    xr_e = _c(np.zeros(max(xr_idx.size, 1)) if xr_e is None else xr_e, np.int32)
    return xr_idx, _c(xr_m.real, np.float64), _c(xr_m.imag, np.float64), xr_e


def dzndc_path_m2(Zn, ref_div_iter, ref_order, xr_mode, scale_m, scale_e,
                  xr_idx=None, xr_m=None, xr_e=None, nexp=0):
    Zn = _c(Zn, np.complex128)
    n = Zn.size
    idx, re, im, e = _xr_table(xr_idx, xr_m, xr_e)
    std = np.zeros(n, dtype=np.complex128)
    ore, oim = np.zeros(n), np.zeros(n)
    oe = np.zeros(n, dtype=np.int32)
    lib().orc_dzndc_path_m2(_p(Zn), n, ref_div_iter, ref_order, int(xr_mode),
                            idx.size, _p(idx), _p(re), _p(im), _p(e),
                            scale_m, scale_e, _p(std), _p(ore), _p(oim), _p(oe), int(nexp))
    if xr_mode:
        return _cx(ore, oim), oe
    return std


def dzndz_path_m2(Zn, ref_div_iter, xr_mode, xr_idx=None, xr_m=None, xr_e=None, nexp=0):
    Zn = _c(Zn, np.complex128)
    n = Zn.size
    idx, re, im, e = _xr_table(xr_idx, xr_m, xr_e)
    std = np.zeros(n + 1, dtype=np.complex128)
    ore, oim = np.zeros(n + 1), np.zeros(n + 1)
    oe = np.zeros(n + 1, dtype=np.int32)
    lib().orc_dzndz_path_m2(_p(Zn), n, ref_div_iter, int(xr_mode), idx.size,
                            _p(idx), _p(re), _p(im), _p(e), _p(std), _p(ore),
                            _p(oim), _p(oe), int(nexp))
    if xr_mode:
        return _cx(ore, oim), oe
    return std


def dzndc_path_bs(Zn, ref_div_iter, ref_order, flavor, scale):
    Zn = _c(Zn, np.complex128)
    n = Zn.size
    out = [np.zeros(n) for _ in range(4)]
    lib().orc_dzndc_path_bs(_p(Zn), n, ref_div_iter, ref_order, flavor, scale,
                            *[_p(o) for o in out])
    return out


# ---------------------------------------------------------------------------
# Perturbation loops
# ---------------------------------------------------------------------------
def perturb_m2(pix, *, Zn, ref_div_iter, ref_order, lin_mat, dx_m, dx_e,
               drift_m, drift_e, max_iter, M, eps_stat, xr_mode,
               calc_dzndc=True, interior=False, bla=None, dZndc=None,
               dZndz=None, xr_idx=None, xr_m=None, xr_e=None,
               carryover=False, Z0=None, nexp=0, backshift=0, fast=False):
    """bla: (M_bla complex flat, r_bla, stages) or None.  dZndc / dZndz are
    complex arrays (standard form) or (mantissa, exp) tuples (Xrange form).
    fast: the -ffast-math build (timing only)."""
    pix = _c(pix, np.complex128)
    n = pix.size
    Zn = _c(Zn, np.complex128)
    keep = []
    a = PM2Args()
    a.Zn, a.ref_len, a.ref_div_iter, a.ref_order = _p(Zn), Zn.size, int(ref_div_iter), int(ref_order)
    idx, re, im, e = _xr_table(xr_idx, xr_m, xr_e)
    keep += [idx, re, im, e]
    a.n_xr, a.xr_idx, a.xr_re, a.xr_im, a.xr_e = idx.size, _p(idx), _p(re), _p(im), _p(e)

    def put_path(path, pre):
        if path is None:
            return
        if isinstance(path, tuple):
            m, ex = _c(path[0], np.complex128), _c(path[1], np.int32)
            r_, i_ = _c(m.real, np.float64), _c(m.imag, np.float64)
            keep.extend([r_, i_, ex])
            setattr(a, pre + "_re", _p(r_))
            setattr(a, pre + "_im", _p(i_))
            setattr(a, pre + "_e", _p(ex))
        else:
            s = _c(path, np.complex128)
            keep.append(s)
            setattr(a, pre, _p(s))

    put_path(dZndc, "dZndc")
    put_path(dZndz, "dZndz")
    if bla is not None:
        Mb = _c(bla[0], np.complex128)
        rb = _c(bla[1], np.float64)
        keep += [Mb, rb]
        a.M_bla, a.r_bla, a.stages_bla, a.bla_on = _p(Mb), _p(rb), int(bla[2]), 1
    else:
        a.bla_on = 0
    a.max_iter, a.M2, a.eps2, a.xr_mode = int(max_iter), M * M, eps_stat ** 2, int(xr_mode)
    codes = ["zn"]
    if interior:
        codes.append("dzndz")
    if calc_dzndc:
        codes.append("dzndc")
    a.i_dzndz = codes.index("dzndz") if interior else -1
    a.i_dzndc = codes.index("dzndc") if calc_dzndc else -1
    a.dzndz_carryover = int(carryover)
    lm = np.asarray(lin_mat, dtype=np.float64).ravel()
    for k in range(4):
        a.lin_mat[k] = lm[k]
    a.dx_m, a.dx_e = float(dx_m), int(dx_e)
    a.drift_re, a.drift_im, a.drift_e = float(np.real(drift_m)), float(np.imag(drift_m)), int(drift_e)
    a.nexp = int(nexp)
    if backshift > 0:
        codes.append("zn_orbit")
    a.backshift = int(backshift)
    a.i_znorbit = codes.index("zn_orbit") if backshift > 0 else -1
    nZ = len(codes)
    Z = np.zeros((nZ, n), dtype=np.complex128) if Z0 is None else _c(Z0, np.complex128).copy()
    U = np.zeros((1, n), dtype=np.int32)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lib(fast).orc_perturb_m2(ct.byref(a), n, _p(pix), _p(Z), nZ, _p(U), _p(sr), _p(si))
    return Z, U, sr, si


def perturb_bs(pix, *, Zn, ref_div_iter, ref_order, lin_mat, dx_m, dx_e,
               driftx_m, driftx_e, drifty_m, drifty_e, max_iter, M, flavor,
               calc_hessian=True, bla=None, dpaths=None, backshift=0):
    pix = _c(pix, np.complex128)
    n = pix.size
    Zn = _c(Zn, np.complex128)
    keep = []
    a = PBSArgs()
    a.Zn, a.ref_len, a.ref_div_iter, a.ref_order = _p(Zn), Zn.size, int(ref_div_iter), int(ref_order)
    if dpaths is not None:
        ds = [_c(d, np.float64) for d in dpaths]
        keep += ds
        a.dXa, a.dXb, a.dYa, a.dYb = [_p(d) for d in ds]
    if bla is not None:
        Mb = _c(bla[0], np.float64)
        rb = _c(bla[1], np.float64)
        keep += [Mb, rb]
        a.M_bla, a.r_bla, a.stages_bla, a.bla_on = _p(Mb), _p(rb), int(bla[2]), 1
    else:
        a.bla_on = 0
    a.max_iter, a.M2, a.flavor, a.calc_hessian = int(max_iter), M * M, int(flavor), int(calc_hessian)
    lm = np.asarray(lin_mat, dtype=np.float64).ravel()
    for k in range(4):
        a.lin_mat[k] = lm[k]
    a.dx_m, a.dx_e = float(dx_m), int(dx_e)
    a.driftx_m, a.driftx_e = float(driftx_m), int(driftx_e)
    a.drifty_m, a.drifty_e = float(drifty_m), int(drifty_e)
    nZ = 6 if calc_hessian else 2
    a.backshift = int(backshift)
    a.i_xnorbit = nZ if backshift > 0 else -1
    nZ += 2 if backshift > 0 else 0
    Z = np.zeros((nZ, n), dtype=np.float64)
    U = np.zeros((1, n), dtype=np.int32)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lib().orc_perturb_bs(ct.byref(a), n, _p(pix), _p(Z), nZ, _p(U), _p(sr), _p(si))
    return Z, U, sr, si


# ---------------------------------------------------------------------------
# Burning Ship, Xrange branch (perturbation.py:1468-1791 with xr_detect_activated)
# ---------------------------------------------------------------------------
def _bs_xr_table(xr):
    """xr: (idx, xm, xe, ym, ye) or None -> contiguous arrays (at least one
    slot, as the reference's)."""
    if xr is None or len(xr[0]) == 0:
        return (np.zeros(0, np.int32), np.zeros(1), np.zeros(1, np.int32), np.zeros(1),
                np.zeros(1, np.int32))
    idx, xm, xe, ym, ye = xr
    return (_c(idx, np.int32), _c(xm, np.float64), _c(xe, np.int32), _c(ym, np.float64),
            _c(ye, np.int32))


def dzndc_path_bs_xr(Zn, ref_div_iter, ref_order, flavor, scale_m, scale_e, xr=None):
    """Xrange Jacobian paths (dXnda, dXndb, dYnda, dYndb): (m [4, len], e [4, len])."""
    Zn = _c(Zn, np.complex128)
    n = Zn.size
    idx, xm, xe, ym, ye = _bs_xr_table(xr)
    m = np.zeros((4, n))
    e = np.zeros((4, n), dtype=np.int32)
    lib().orc_dzndc_path_bs_xr(_p(Zn), n, int(ref_div_iter), int(ref_order), int(flavor),
                               float(scale_m), int(scale_e), idx.size, _p(idx), _p(xm),
                               _p(xe), _p(ym), _p(ye), _p(m), _p(e))
    return m, e


def perturb_bs_xr(pix, *, Zn, ref_div_iter, ref_order, lin_mat, dx_m, dx_e,
                  driftx_m, driftx_e, drifty_m, drifty_e, max_iter, M, flavor,
                  calc_hessian=True, bla=None, xpaths=None, xr=None):
    """The Xrange branch: xpaths the Xrange Jacobian paths (m, e), xr the
    orbit's side table (idx, xm, xe, ym, ye)."""
    pix = _c(pix, np.complex128)
    n = pix.size
    Zn = _c(Zn, np.complex128)
    keep = []
    a = PBSXArgs()
    a.Zn, a.ref_len, a.ref_div_iter, a.ref_order = _p(Zn), Zn.size, int(ref_div_iter), int(ref_order)
    t = _bs_xr_table(xr)
    keep += list(t)
    a.n_xr, a.xr_idx, a.xr_xm, a.xr_xe, a.xr_ym, a.xr_ye = t[0].size, *[_p(v) for v in t]
    if xpaths is not None:
        pm, pe = _c(xpaths[0], np.float64), _c(xpaths[1], np.int32)
        keep += [pm, pe]
        a.path_m, a.path_e = _p(pm), _p(pe)
    if bla is not None:
        Mb = _c(bla[0], np.float64)
        rb = _c(bla[1], np.float64)
        keep += [Mb, rb]
        a.M_bla, a.r_bla, a.stages_bla, a.bla_on = _p(Mb), _p(rb), int(bla[2]), 1
    else:
        a.bla_on = 0
    a.max_iter, a.M2, a.flavor, a.calc_hessian = int(max_iter), M * M, int(flavor), int(calc_hessian)
    lm = np.asarray(lin_mat, dtype=np.float64).ravel()
    for k in range(4):
        a.lin_mat[k] = lm[k]
    a.dx_m, a.dx_e = float(dx_m), int(dx_e)
    a.driftx_m, a.driftx_e = float(driftx_m), int(driftx_e)
    a.drifty_m, a.drifty_e = float(drifty_m), int(drifty_e)
    nZ = 6 if calc_hessian else 2
    Z = np.zeros((nZ, n), dtype=np.float64)
    U = np.zeros((1, n), dtype=np.int32)
    si = np.zeros((1, n), dtype=np.int32)
    sr = -np.ones((1, n), dtype=np.int8)
    lib().orc_perturb_bs_xr(ct.byref(a), n, _p(pix), _p(Z), nZ, _p(U), _p(sr), _p(si))
    return Z, U, sr, si
