"""
CPU restatement of the reference's field-lines and DEM-normal post-processing
-- TEST INFRASTRUCTURE (only tests use it): what the tests compare
csrc/fsg_postproc.cu with.

Follows src/fractalshades/postproc.py of the reference: Continuous_iter_pp's
context (:352-406, :1001-1009), Fieldlines_pp (:409-530) with
Fieldlines_pp_infinity (:1038-1091) / Fieldlines_pp_infinity_BS
(:1094-1160) and the Catmull-Rom weights (:1021-1035), DEM_normal_pp
(:533-628) with core.py:3147-3158 apply_unskew_1d.  numpy arrays, the
reference's operation order (x ** 2 written x * x).
"""
import numpy as np


def continuous_context(zn, stop_iter, d, M, a_d=1.):
    """(nu_frac, n) as Continuous_iter_pp leaves them in the context."""
    k = np.abs(a_d) ** (1. / (d - 1.))
    with np.errstate(all="ignore"):
        nu_frac = -(np.log(np.log(np.abs(zn * k)) / np.log(M * k)) / np.log(d))
        nu_div, nu_mod = np.divmod(-nu_frac, 1.)
        n = stop_iter - nu_div.astype(stop_iter.dtype)
    return -nu_mod, n


def _cm(d):
    return (0.5 * d * (-d + d * d), 0.5 * d * (1. + 4. * d - 3. * (d * d)),
            1. + 0.5 * d * (-5. * d + 3. * (d * d)), 0.5 * d * (-1. + 2. * d - d * d))


def fieldlines_params(n_iter, swirl, endpoint_k):
    k_arr = np.geomspace(1., endpoint_k, num=n_iter)
    k_arr = k_arr / np.sum(k_arr)
    phi_arr = np.random.default_rng(0).random(n_iter) * swirl * np.pi
    return k_arr, phi_arr


def _map(model, z, c):
    if model == 0:
        return z * z + c
    if model > 0:
        return z ** model + c
    x, y, a, b = z.real, z.imag, c.real, c.imag
    fl = -model
    if fl == 1:
        nx, ny = x * x - y * y + a, 2. * np.abs(x * y) - b
    elif fl == 2:
        nx, ny = x * x - y * y + a, 2. * x * np.abs(y) - b
    elif fl == 3:
        nx, ny = x * x - y * np.abs(y) + a, 2. * x * y - b
    elif fl == 4:
        nx, ny = np.abs(x * x - y * y) + a, 2. * x * y - b
    else:
        nx, ny = np.abs(x * x - y * y) + a, 2. * np.abs(x * y) - b
    return nx + 1j * ny


def fieldlines(model, c, z, nu_frac, n, k_arr, phi_arr, is_backward, backshift):
    """model 0: z^2 + c, n: z^n + c, -flavor: Burning Ship (z = x + i y)."""
    M_cutoff = 100000.
    nfl = len(k_arr)
    z = np.array(z, dtype=np.complex128)
    ang = [np.arctan2(z.imag, z.real)]
    for i in range(nfl + 2):
        big = np.abs(z) > M_cutoff
        zb = np.cos(ang[i]) * M_cutoff + 1j * (np.sin(ang[i]) * M_cutoff)
        with np.errstate(all="ignore"):
            z = np.where(big, _map(model, zb, 0j), _map(model, z, c))
        ang.append(np.arctan2(z.imag, z.real))
    d = -np.asarray(nu_frac, dtype=np.float64)
    if is_backward:
        d = np.where(backshift > np.asarray(n), 1., d)
    a0, a1, a2, a3 = _cm(d)
    val = np.zeros(z.shape)
    for i in range(nfl):
        ph = phi_arr[i]
        val += k_arr[i] * (a0 * np.sin(ang[i] + ph) + a1 * np.sin(ang[i + 1] + ph)
                           + a2 * np.sin(ang[i + 2] + ph) + a3 * np.sin(ang[i + 3] + ph))
    return val


def normal(kind, zn, dzndc=None, d2zndc2=None, jac=None, skew=None):
    """kind 0 "potential" (zn / dzndc), 1 "Milnor", 2 Burning Ship (J^T z)."""
    with np.errstate(all="ignore"):
        if kind == 0:
            nv = zn / dzndc
        elif kind == 1:
            lo = np.log(np.abs(zn))
            nv = zn * dzndc * ((1 + lo) * np.conj(dzndc * dzndc) - lo * np.conj(zn * d2zndc2))
        else:
            dXdA, dXdB, dYdA, dYdB = jac
            nv = (dXdA * zn.real + dYdA * zn.imag) + 1j * (dXdB * zn.real + dYdB * zn.imag)
        if skew is not None:
            nx, ny = nv.real.copy(), nv.imag.copy()
            nv = (skew[0, 0] * nx + skew[1, 0] * ny) + 1j * (skew[0, 1] * nx + skew[1, 1] * ny)
        return nv / np.abs(nv)
