"""Host-side logic, no GPU: geometry, waveforms, regularisers, the tiler and the C ABI exports."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import fdtd_oracle as orc

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_every_declared_symbol():
    from soundwavesimulation_gb300 import _lib
    lib = _lib.load()
    header = (ROOT / "include" / "fdtd_gb300.h").read_text()
    declared = set(re.findall(r"^\s*(?:int32_t|size_t|const char\*)\s+(fdtd_\w+)\s*\(", header, re.M))
    assert declared, "no declarations parsed"
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared in the header but not exported"
    assert declared == set(_lib.EXPORTED) | (declared - set(_lib.EXPORTED))
    missing_binding = declared - set(_lib.EXPORTED)
    assert not missing_binding, f"no ctypes binding for {missing_binding}"


@pytest.mark.parametrize("n_cells", [256, 512, 1024])
def test_ring_geometry_matches_reference(golden, n_cells):
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("geometry")
    n, h, n_el, radius = d[f"ring{n_cells}_meta"]
    ax = axis_centers(int(n), h)
    ring = RingArray(int(n_el), radius, ax, ax)
    np.testing.assert_array_equal(ring.rows, d[f"ring{n_cells}_rows"])
    np.testing.assert_array_equal(ring.cols, d[f"ring{n_cells}_cols"])
    np.testing.assert_array_equal(ring._row0, d[f"ring{n_cells}_row0"])
    np.testing.assert_array_equal(ring._col0, d[f"ring{n_cells}_col0"])
    for k in ("w00", "w10", "w01", "w11"):
        np.testing.assert_allclose(getattr(ring, "_" + k), d[f"ring{n_cells}_{k}"], rtol=0, atol=1e-14)


def test_arc_geometry_matches_reference(golden):
    from soundwavesimulation_gb300 import ArcArray, axis_centers
    d = golden("geometry")
    n, h, n_el, radius, span, center = d["arc41_meta"]
    ax = axis_centers(int(n), h)
    arc = ArcArray(int(n_el), radius, span, center, ax, ax)
    np.testing.assert_array_equal(arc.rows, d["arc41_rows"])
    np.testing.assert_array_equal(arc._col0, d["arc41_col0"])
    np.testing.assert_allclose(arc._w11, d["arc41_w11"], rtol=0, atol=1e-14)


def test_ring_errors_like_reference():
    from soundwavesimulation_gb300 import RingArray, axis_centers
    ax = axis_centers(41, 2e-3)
    with pytest.raises(ValueError):
        RingArray(1, 0.03, ax, ax)
    with pytest.raises(ValueError):
        RingArray(6, 0.045, ax, ax)        # touches the boundary
    with pytest.raises(ValueError):
        RingArray(400, 0.03, ax, ax)       # two elements per pixel
    with pytest.raises(ValueError):
        RingArray(6, 0.03, ax, ax).transmitter_index(6)


def test_chirp_and_helpers_match_oracle(golden):
    from soundwavesimulation_gb300 import linear_chirp, n_steps_for_crossing, stable_dt
    d = golden("ring41")
    np.testing.assert_allclose(linear_chirp(float(d["dt"]), 20e-6, 1e5, 2.5e5), d["pulse"], rtol=0, atol=1e-14)
    assert stable_dt(2000.0, 2e-3, 2e-3, 0.45) == pytest.approx(float(d["dt"]), rel=1e-15)
    assert n_steps_for_crossing(0.03, 1500.0, float(d["dt"])) == orc.n_steps_for_crossing(0.03, 1500.0, float(d["dt"]))


def test_record_adjoint_is_transpose():
    from soundwavesimulation_gb300 import RingArray, axis_centers
    ax = axis_centers(64, 1e-3)
    ring = RingArray(20, 0.025, ax, ax)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((64, 64))
    r = rng.standard_normal(20)
    assert np.dot(ring.record(f), r) == pytest.approx(np.sum(f * ring.record_adjoint(r)), rel=1e-12)


def test_regularisers_gradients():
    from soundwavesimulation_gb300 import interior_mask, m_from_c, tikhonov, total_variation, axis_centers
    rng = np.random.default_rng(1)
    ax = axis_centers(41, 2e-3)
    mask = interior_mask(ax, ax, 0.03, 0.0)
    m = m_from_c(np.where(mask, 1500.0 + 100.0 * rng.standard_normal((41, 41)), 1500.0))
    d = np.where(mask, rng.standard_normal((41, 41)), 0.0) * 1e-9
    for fn, args in ((tikhonov, (1e10,)), (total_variation, (1.0, 1e-9))):
        v, g = fn(m, mask, *args)
        fd = (fn(m + 1e-3 * d, mask, *args)[0] - fn(m - 1e-3 * d, mask, *args)[0]) / 2e-3
        assert fd == pytest.approx(np.sum(g * d), rel=1e-6)
        assert np.all(g[~mask] == 0.0) and v > 0.0


@pytest.mark.parametrize("n", [8, 9, 41, 64, 100, 127, 128, 129, 200, 255, 256, 257, 384, 511, 512, 1024])
@pytest.mark.parametrize("region,align,halo,band", [(128, 4, 13, 0), (128, 1, 13, 8), (64, 1, 5, 4),
                                                    (128, 4, 2, 0), (96, 1, 17, 8), (160, 1, 9, 8)])
def test_tiler_invariants(n, region, align, halo, band):
    """Owned ranges partition [0, n), interior borders keep the halo, edges share a band."""
    from soundwavesimulation_gb300 import _lib
    tiles = _lib.tile_axis(n, region, align, halo, band)
    assert tiles[0, 1] == 0 and tiles[-1, 2] == n
    assert np.all(tiles[1:, 1] == tiles[:-1, 2])
    for origin, o0, o1, flags in tiles:
        assert o1 > o0
        assert origin % align == 0
        if origin > 0:
            assert o0 >= origin + halo
        if origin + region < n:
            assert o1 <= origin + region - halo
        assert bool(flags & 1) == (origin <= 0)
        assert bool(flags & 2) == (origin + region >= n)
        if band > 1:
            if origin <= 0 < origin + region:
                assert (-origin) % band != band - 1
            if origin <= n - 1 < origin + region:
                assert (n - 1 - origin) % band != 0


@pytest.mark.parametrize("n", [256, 384, 512, 1024])
@pytest.mark.parametrize("band,halo", [(8, 16), (4, 16), (8, 11)])
def test_config_grids_take_the_compact_edge_path(n, band, halo):
    """At the configuration grid sizes the tiler puts row 0 at band row 0, row n-1
    at band row `band` - 1 and column n-1 at column 3 of a lane: the placements
    for which the temporally blocked kernel runs its compact edge loop."""
    from soundwavesimulation_gb300 import _lib
    ty = _lib.tile_axis(n, 128, 1, halo, band)
    assert ty[0, 0] == 0
    last = int(ty[-1, 0])
    assert (n - 1 - last) % band == band - 1
    tx = _lib.tile_axis(n, 128, 4, halo, 0)
    assert (n - 1 - int(tx[-1, 0])) % 4 == 3


def test_tap_table_sums_every_receiver_weight():
    from soundwavesimulation_gb300 import RingArray, axis_centers, _lib
    ax = axis_centers(41, 2e-3)
    ring = RingArray(16, 0.03, ax, ax)
    row0, col0, w = ring.receiver_taps()
    nodes, tw = _lib.tap_table(41, 41, row0, col0, w)
    assert np.unique(nodes[:, :2], axis=0).shape[0] == nodes.shape[0]
    total = np.zeros(16)
    for nd, ww in zip(nodes, tw):
        for rid, wq in zip(nd[2:], ww):
            if rid >= 0:
                total[rid] += wq
    np.testing.assert_allclose(total, 1.0, rtol=1e-6)


def test_engine_refuses_cpu_device():
    from soundwavesimulation_gb300 import torch_backend as tb
    with pytest.raises((ValueError, RuntimeError)):
        tb.TorchScalarWave2D(np.full((16, 16), 1500.0), 1e-3, device="cpu")
