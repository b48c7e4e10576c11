"""
Exact-arithmetic pins of the perturbation path, on CPU.  z -> z^2 + c is
iterated directly at the view's digits (the host library's MPFR orbit,
bench.direct_pixels) and compared with:

* a plain mpmath loop on one pixel (count, z_n and dz_n/dc);
* the oracle (the reference's algorithm, perturbation.py:988-1400, Xrange
  branch) on views of width 1e-300 centred one to three nucleus sizes away
  from the period-2562 nucleus that serves as the reference: each view lies
  outside the minibrot, every pixel escapes after one to four periods of the
  reference, and the oracle takes the exact count on every pixel.  (Farther
  into the spirals, after ten periods or more, the double-precision deltas
  and the BLA truncation of the reference's algorithm no longer resolve the
  count; the bench states those differences per output.)
"""
import os
import sys

import mpmath
import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

# (multiple of the nucleus size estimate 3.9e-10, quarter turns) -> views
# whose pixels escape after 1, 2, 3 and 4 periods
OFFSETS = [(3.0, 3), (2.0, 3), (1.0, 0), (1.0, 3)]


def offset_view(fac, quarter, dx="1e-300", nx=16):
    """A width-dx view at nucleus + fac * 3.9e-10 * i^quarter, with the
    period-2562 nucleus (400 digits) as its reference."""
    from fractalshades_gb300 import synthetic as syn
    with mpmath.workdps(400):
        o = (mpmath.mpf(fac) * mpmath.mpf("3.9e-10") * mpmath.mpc(0, 1) ** quarter
             / mpmath.mpf(dx))
    return syn.prepare_m2(p=2562, dps=400, dx=dx, nx=nx, max_iter=200000, M=1000.,
                          offset=(o.real, o.imag))


def test_direct_pixels_vs_mpmath_loop():
    w = offset_view(3.0, 3)
    d = bench.direct_pixels(w, np.array([5]), threads=1)
    with mpmath.workdps(w.dps):
        c = w.center + mpmath.mpf(w.dx) * mpmath.mpc(float(w.xs[5]), float(w.ys[0]))
        z, dz = mpmath.mpc(0), mpmath.mpc(0)
        for n in range(1, w.max_iter + 1):
            dz = 2 * z * dz + 1
            z = z * z + c
            if abs(z) > w.M:
                break
        dz = dz * mpmath.mpf(w.dx)
        assert int(d["si"][0]) == n and int(d["sr"][0]) == 1
        assert abs(complex(z) - d["zn"][0]) <= 1e-15 * abs(complex(z))
        assert abs(complex(dz) - d["dzndc"][0]) <= 1e-9 * abs(complex(dz))


@pytest.mark.parametrize("fac,quarter", OFFSETS)
def test_oracle_xrange_branch_vs_exact_counts(fac, quarter):
    w = offset_view(fac, quarter)
    assert w.xr_mode
    idx = bench.sample_indices(w.nx * w.ny, 12, 3)
    exact = bench.direct_pixels(w, idx)
    o = bench.oracle_pixels(w, idx, bench.oracle_kw(w), threads=2)
    assert (exact["sr"] == 1).all()
    assert len(np.unique(exact["si"])) == 1          # one count over 1e-300
    assert 2562 < exact["si"][0] < 5 * 2562
    np.testing.assert_array_equal(o["si"], exact["si"])
    np.testing.assert_array_equal(o["sr"], exact["sr"])
    # the potential (postproc.py:352-406) of the reference's algorithm is
    # within 1e-5 of the exact one
    po, _ = bench.potential_dem(o["zn"], o["dzndc"], o["si"], w.M)
    pe, _ = bench.potential_dem(exact["zn"], exact["dzndc"], exact["si"], w.M)
    assert np.max(np.abs(po - pe) / pe) < 1e-5
