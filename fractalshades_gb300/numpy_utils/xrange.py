"""
Extended-range ("Xrange") scalars on the host: conversions between mpmath
numbers and the (mantissa, base-2 exponent) records uploaded to the GPU.

Follows numpy_utils/xrange.py:8-63 of the reference (mpc_to_Xrange,
mpf_to_Xrange, the record dtype of a float64 / complex128 mantissa and an
int32 exponent, complex values sharing one exponent).  The full ndarray
subclass of the reference is not needed by the iteration path.
"""
import mpmath
import numpy as np


def get_xr_dtype(dtype):
    """Record dtype (mantissa, exp) of the reference (xrange.py:61-63)."""
    return np.dtype([("mantissa", dtype), ("exp", np.int32)], align=False)


class XrScalar:
    """A single Xrange value m * 2**e (m float or complex)."""
    __slots__ = ("m", "e")

    def __init__(self, m, e):
        self.m = m
        self.e = int(e)

    def to_standard(self):
        if isinstance(self.m, complex):
            return complex(np.ldexp(self.m.real, self.e), np.ldexp(self.m.imag, self.e))
        return float(np.ldexp(self.m, self.e))

    def to_mpmath(self):
        if isinstance(self.m, complex):
            return mpmath.mpc(mpmath.ldexp(self.m.real, self.e), mpmath.ldexp(self.m.imag, self.e))
        return mpmath.ldexp(self.m, self.e)

    def __repr__(self):
        return f"XrScalar({self.m!r}, {self.e})"


def mpf_to_Xrange(mpf, dtype=np.float64):
    """mantissa in [0.5, 1) and exponent (xrange.py:46-50)."""
    m, e = mpmath.frexp(mpmath.mpf(mpf))
    return XrScalar(float(dtype(float(m))), int(e))


def mpc_to_Xrange(mpc, dtype=np.complex128):
    """Complex value with a shared exponent (xrange.py:8-43)."""
    mpc = mpmath.mpc(mpc)
    mx, ex = mpmath.frexp(mpc.real)
    my, ey = mpmath.frexp(mpc.imag)
    mx, my = float(mx), float(my)
    if ex > ey:
        case = 1
    elif ex < ey:
        case = 2
    else:
        case = 3
    if ex == 0.:
        case = 2
    if ey == 0.:
        case = 1
    if case == 1:
        m = complex(mx, float(np.ldexp(my, ey - ex)))
        e = ex
    elif case == 2:
        m = complex(float(np.ldexp(mx, ex - ey)), my)
        e = ey
    else:
        m = complex(mx, my)
        e = ex
    return XrScalar(m, int(e))


def xr_from_mantissa_exp(mx, ex, my, ey):
    """Complex Xrange of (mx 2**ex) + i (my 2**ey) with a shared exponent:
    the larger exponent wins and the other part is scaled (exactly, unless it
    drops below the double range)."""
    if mx == 0.:
        return XrScalar(complex(0., my), ey)
    if my == 0.:
        return XrScalar(complex(mx, 0.), ex)
    e = max(ex, ey)
    return XrScalar(complex(float(np.ldexp(mx, ex - e)), float(np.ldexp(my, ey - e))), e)


def xr_table(xr_dict):
    """Sparse side table of an orbit (perturbation.py:317-375 get_path_data):
    sorted indices, complex mantissas and exponents."""
    keys = sorted(xr_dict.keys())
    vals = [_as_scalar(xr_dict[k]) for k in keys]
    idx = np.array(keys, dtype=np.int32)
    m = np.array([complex(v.m) for v in vals], dtype=np.complex128)
    e = np.array([v.e for v in vals], dtype=np.int32)
    return idx, m, e


def _as_scalar(v):
    """XrScalar of an XrScalar or of a (mantissa, exp) record array (the
    reference's Xrange values read from its pickles)."""
    if isinstance(v, XrScalar):
        return v
    rec = np.asarray(v).reshape(-1)[0]
    return XrScalar(rec["mantissa"].item(), int(rec["exp"]))


def xr_table_xy(xr_dict):
    """Burning Ship side table: indices and planar (x then y) mantissas and
    exponents of the register {i: (x, y)} -- x, y given as (mantissa, exp)
    pairs or as the reference's Xrange records."""
    keys = sorted(xr_dict)
    n = len(keys)
    idx = np.array(keys, dtype=np.int32)
    m = np.zeros(2 * n, dtype=np.float64)
    e = np.zeros(2 * n, dtype=np.int32)
    for k, key in enumerate(keys):
        for j, v in enumerate(xr_dict[key]):
            if isinstance(v, tuple):
                mv, ev = float(v[0]), int(v[1])
            else:
                sc = _as_scalar(v)
                mv, ev = float(np.real(sc.m)), int(sc.e)
            m[j * n + k], e[j * n + k] = mv, ev
    return idx, m, e
