"""
ctypes binding of libfsghost.so (declared in include/fsghost.h): the
arbitrary-precision host side on MPFR / MPC.

The library is built with the CUDA one (``python -c "import __graft_entry__
as g; g.build()"``); loading fails with an explicit error when it is missing.
The calls release the GIL (ctypes), so orbits of several references can be
computed on concurrent threads.
"""
import ctypes as ct
import os
import threading

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libfsghost.so")

FSH_OK = 0
FSH_ERR_ARG = -1
FSH_ERR_NOMEM = -3

I32, I64, U32, F64 = ct.c_int32, ct.c_int64, ct.c_uint32, ct.c_double
P, S = ct.c_void_p, ct.c_char_p
PI64 = ct.POINTER(I64)

#: exported symbols (include/fsghost.h)
SYMBOLS = {
    "fsh_registers_count": (I64, [P, I32]),
    "fsh_registers_copy": (ct.c_int, [P, I32, P, P, P]),
    "fsh_registers_free": (None, [P]),
    "fsh_orbit_mn": (I64, [S, S, I64, I64, U32, F64, I32, P, ct.POINTER(P)]),
    "fsh_orbit_bs": (I64, [S, S, I64, I64, I32, F64, I32, P, ct.POINTER(P)]),
    "fsh_ball_mn": (I64, [S, S, I64, S, U32, I64, F64]),
    "fsh_ball_bs": (I64, [S, S, I64, S, I32, I64, F64]),
    "fsh_nucleus_m2": (ct.c_int, [S, S, I64, I64, I64, S, S, S, S, I64, PI64, PI64]),
    "fsh_any_nucleus_mn": (ct.c_int, [S, S, I64, U32, I64, I64, S, S, S, S, I64, PI64, PI64]),
    "fsh_any_nucleus_bs": (ct.c_int, [S, S, I64, I32, I64, I64, S, S, S, S, I64, PI64, PI64]),
    "fsh_size_mn": (ct.c_int, [S, S, I64, U32, I64, P, P]),
    "fsh_size_bs": (ct.c_int, [S, S, I64, I32, I64, P, P, P]),
}

_lock = threading.Lock()
_lib = None


class HostError(RuntimeError):
    pass


def load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise HostError(f"{LIB_PATH} is missing: build it with "
                            "python -c 'import __graft_entry__ as g; g.build()'")
        L = ct.CDLL(LIB_PATH)
        for name, (res, args) in SYMBOLS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def _b(s):
    if isinstance(s, (bytes, bytearray)):
        return bytes(s)
    return str(s).encode("utf8")


def _check(rc, what):
    if rc < 0:
        raise HostError(f"{what} failed (code {rc})")
    return rc


def _p(a):
    return a.ctypes.data_as(P)


def _registers(L, h):
    """[(idx, mx, ex, my, ey)] of both registers, then free the handle."""
    out = []
    try:
        for which in (0, 1):
            n = _check(L.fsh_registers_count(h, which), "fsh_registers_count")
            idx = np.zeros(n, dtype=np.int64)
            m = np.zeros(2 * n, dtype=np.float64)
            e = np.zeros(2 * n, dtype=np.int64)
            if n:
                _check(L.fsh_registers_copy(h, which, _p(idx), _p(m), _p(e)),
                       "fsh_registers_copy")
            out.append([(int(idx[k]), float(m[2 * k]), int(e[2 * k]), float(m[2 * k + 1]),
                         int(e[2 * k + 1])) for k in range(n)])
    finally:
        L.fsh_registers_free(h)
    return out


def _orbit_buffer(orbit, max_iter):
    orb = orbit.view(np.float64) if orbit.dtype != np.float64 else orbit
    if orb.ndim != 1 or orb.size != 2 * (max_iter + 1) or not orb.flags.c_contiguous:
        raise ValueError("orbit must be a contiguous complex128 [max_iter + 1] (or its "
                         "float64 view)")
    return orb


def orbit_mn(orbit, need_xr, max_iter, exponent, M, seed_x, seed_y, seed_prec):
    """(i, xr entries, partial entries) with orbit filled in place."""
    L = load()
    orb = _orbit_buffer(orbit, int(max_iter))
    h = P()
    i = _check(L.fsh_orbit_mn(_b(seed_x), _b(seed_y), int(seed_prec), int(max_iter),
                              int(exponent), float(M), int(bool(need_xr)), _p(orb),
                              ct.byref(h)), "fsh_orbit_mn")
    xr, partials = _registers(L, h)
    return i, xr, partials


def orbit_bs(orbit, need_xr, max_iter, kind, M, seed_x, seed_y, seed_prec):
    L = load()
    orb = _orbit_buffer(orbit, int(max_iter))
    h = P()
    i = _check(L.fsh_orbit_bs(_b(seed_x), _b(seed_y), int(seed_prec), int(max_iter),
                              int(kind), float(M), int(bool(need_xr)), _p(orb), ct.byref(h)),
               "fsh_orbit_bs")
    xr, partials = _registers(L, h)
    return i, xr, partials


def ball_mn(seed_x, seed_y, seed_prec, seed_px, exponent, maxiter, M_divergence):
    """The period found, -1 when none (the reference's convention)."""
    r = _check(load().fsh_ball_mn(_b(seed_x), _b(seed_y), int(seed_prec), _b(seed_px),
                                  int(exponent), int(maxiter), float(M_divergence)),
               "fsh_ball_mn")
    return r if r > 0 else -1


def ball_bs(seed_x, seed_y, seed_prec, seed_px, kind, maxiter, M_divergence):
    r = _check(load().fsh_ball_bs(_b(seed_x), _b(seed_y), int(seed_prec), _b(seed_px),
                                  int(kind), int(maxiter), float(M_divergence)),
               "fsh_ball_bs")
    return r if r > 0 else -1


def _hex_value(digits, e):
    """sign * 0.d1 d2 ... (base 16) * 16^e as (mantissa, binary exponent)."""
    s = digits.decode("ascii")
    if "@" in s:
        return None
    neg = s.startswith("-")
    d = s.lstrip("-")
    man = int(d, 16)
    return (-man if neg else man), 4 * (e - len(d))


def _newton(fn, args, seed_prec):
    n = int(seed_prec) // 4 + 16
    bx = ct.create_string_buffer(n)
    by = ct.create_string_buffer(n)
    ex, ey = I64(), I64()
    rc = _check(fn(*args, bx, by, n, ct.byref(ex), ct.byref(ey)), fn.__name__)
    return rc == 1, _hex_value(bx.value, ex.value), _hex_value(by.value, ey.value)


def nucleus_m2(seed_x, seed_y, seed_prec, order, max_newton, seed_eps_cv, seed_eps_valid):
    L = load()
    return _newton(L.fsh_nucleus_m2, (_b(seed_x), _b(seed_y), int(seed_prec), int(order),
                                      int(max_newton), _b(seed_eps_cv), _b(seed_eps_valid)),
                   seed_prec)


def any_nucleus_mn(seed_x, seed_y, seed_prec, exponent, order, max_newton, seed_eps_cv,
                   seed_eps_valid):
    L = load()
    return _newton(L.fsh_any_nucleus_mn,
                   (_b(seed_x), _b(seed_y), int(seed_prec), int(exponent), int(order),
                    int(max_newton), _b(seed_eps_cv), _b(seed_eps_valid)), seed_prec)


def any_nucleus_bs(seed_x, seed_y, seed_prec, kind, order, max_newton, seed_eps_cv,
                   seed_eps_valid):
    L = load()
    return _newton(L.fsh_any_nucleus_bs,
                   (_b(seed_x), _b(seed_y), int(seed_prec), int(kind), int(order),
                    int(max_newton), _b(seed_eps_cv), _b(seed_eps_valid)), seed_prec)


def size_mn(seed_x, seed_y, seed_prec, exponent, order):
    """((re mantissa, exp), (im mantissa, exp)) of the size estimate."""
    out = np.zeros(2)
    eout = np.zeros(2, dtype=np.int64)
    _check(load().fsh_size_mn(_b(seed_x), _b(seed_y), int(seed_prec), int(exponent),
                              int(order), _p(out), _p(eout)), "fsh_size_mn")
    return (float(out[0]), int(eout[0])), (float(out[1]), int(eout[1]))


def size_bs(seed_x, seed_y, seed_prec, kind, order):
    """((mantissa, exp), skew[2, 2])"""
    out = np.zeros(1)
    eout = np.zeros(1, dtype=np.int64)
    skew = np.zeros(4)
    _check(load().fsh_size_bs(_b(seed_x), _b(seed_y), int(seed_prec), int(kind), int(order),
                              _p(out), _p(eout), _p(skew)), "fsh_size_bs")
    return (float(out[0]), int(eout[0])), skew.reshape(2, 2)
