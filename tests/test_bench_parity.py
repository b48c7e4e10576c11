"""
The bench's parity and CPU-baseline helpers on CPU: the reference's 200 x 200
tiling covers an image exactly once, the per-output parity table reports zero
error for identical outputs and catches a difference planted in a copy of the
oracle's output, and the tile-based CPU baseline runs the whole tiles it
reports.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("nx,ny", [(2048, 2048), (800, 600), (200, 200), (201, 37)])
def test_image_tiles_cover_image_once(nx, ny):
    seen = np.zeros((ny, nx), dtype=np.int32)
    for x0, y0, tx, ty in bench.image_tiles(nx, ny):
        assert 0 < tx <= bench.CPU_TILE and 0 < ty <= bench.CPU_TILE
        seen[y0:y0 + ty, x0:x0 + tx] += 1
    assert (seen == 1).all()


@pytest.fixture(scope="module")
def edge_small():
    from fractalshades_gb300 import synthetic as syn
    w = syn.edge_workload(nx=64, max_iter=20000)
    idx = bench.sample_indices(w.nx * w.ny, 256, 17)
    return w, idx, bench.oracle_pixels(w, idx, bench.oracle_kw(w), threads=2)


def test_parity_table_identical_outputs(edge_small):
    w, idx, o = edge_small
    t = bench.parity_table(o, o, w.M)
    assert t["pixels"] == idx.size and t["escaped"] > 0
    for k, v in t.items():
        if k not in ("pixels", "escaped"):
            assert v == 0, k


def test_parity_table_catches_planted_difference(edge_small):
    w, idx, o = edge_small
    bad = {k: v.copy() for k, v in o.items()}
    esc = np.flatnonzero(o["sr"] == 1)
    bad["si"][esc[0]] += 3                       # one count off by 3
    bad["zn"][esc[1]] *= 1 + 1e-9                # one zn off by 1e-9
    t = bench.parity_table(bad, o, w.M)
    assert t["iter_count_differs_frac"] == pytest.approx(1 / idx.size)
    assert t["iter_count_max_abs_diff"] == 3
    assert 5e-10 < t["zn_max_rel_err"] < 2e-9
    assert t["potential_max_rel_err"] > 0


def test_potential_dem_formula():
    """|zn| = M after n steps gives the potential n (nu_frac = 0), and
    |zn| = M^2 gives n - 1."""
    M = 1000.
    zn = np.array([M, M * M]).astype(np.complex128)
    pot, dem = bench.potential_dem(zn, np.array([1., 2.]), np.array([10, 10]), M)
    assert pot == pytest.approx([10., 9.])
    assert dem == pytest.approx([M * np.log(M), M * M * np.log(M * M) / 2.])


def test_cpu_baseline_whole_tiles():
    from fractalshades_gb300 import synthetic as syn
    w = syn.config2_workload(nx=256, max_iter=2000)
    r = bench.cpu_baseline(w, threads=2, n_tiles=2)
    assert r["tiles"] == 2 and r["cores"] == 2 and r["kind"] == "port"
    assert r["value"] > 0 and "whole 200x200 tiles" in r["sample"]
