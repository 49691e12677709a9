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


def test_oracle_regularisers_gradients():
    """The oracle's regularisers are consistent: central differences of the value
    along a random in-mask direction equal the gradient's projection."""
    from oracle import fdtd_oracle as orc
    rng = np.random.default_rng(1)
    ax = orc.axis_centers(41, 2e-3)
    mask = orc.interior_mask(ax, ax, 0.03, 0.0)
    m = 1.0 / np.where(mask, 1500.0 + 100.0 * rng.standard_normal((41, 41)), 1500.0) ** 2
    d = np.where(mask, rng.standard_normal((41, 41)), 0.0) * 1e-9
    for fn, args in ((orc.tikhonov, (1e10,)), (orc.total_variation, (1.0, 1e-9))):
        v, g = fn(m, mask, *args)
        fd = (fn(m + 1e-3 * d, mask, *args)[0] - fn(m - 1e-3 * d, mask, *args)[0]) / 2e-3
        assert fd == pytest.approx(np.sum(g * d), rel=1e-6)
        assert np.all(g[~mask] == 0.0) and v > 0.0


def test_medium_helpers_match_reference_definitions(golden):
    """m <-> c, clipping and the interior mask of the product follow the reference's
    definitions (fdtd2d/inversion/medium.py:15-40); the ring41 fixture holds the
    reference's own mask."""
    from soundwavesimulation_gb300 import c_from_m, clip_m, interior_mask, m_from_c
    from soundwavesimulation_gb300 import axis_centers, mute_transmitter, waveform_misfit
    c = np.array([[1400.0, 1500.0], [1600.0, 2100.0]])
    assert np.array_equal(m_from_c(c), 1.0 / (c * c))
    assert np.allclose(c_from_m(m_from_c(c)), c, rtol=1e-15)
    clipped = c_from_m(clip_m(m_from_c(c), 1450.0, 2000.0))
    assert np.allclose(clipped, [[1450.0, 1500.0], [1600.0, 2000.0]], rtol=1e-15)
    g = golden("ring41")
    x = axis_centers(41, 2.0e-3)
    assert np.array_equal(interior_mask(x, x, 0.030, margin_m=2 * 2.0e-3), g["mask"])
    with pytest.raises(ValueError):
        interior_mask(x, x, 0.01, 0.02)
    rng = np.random.default_rng(2)
    pred, obs = rng.standard_normal((5, 7)), rng.standard_normal((5, 7))
    r = pred - obs
    r[3] = 0.0
    assert waveform_misfit(pred, obs, 3) == pytest.approx(0.5 * np.sum(r * r), rel=1e-14)
    assert np.array_equal(mute_transmitter(pred, 3)[3], np.zeros(7))


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


def _fake_problem(wave=0, row=20, col=20, rx_row=10, n=64):
    """A problem description whose device pointers are placeholders: only the
    host-side argument checks run on it (they return before any device work)."""
    from soundwavesimulation_gb300 import _lib
    keep = {
        "row0": np.array([rx_row, 30], dtype=np.int32), "col0": np.array([10, 30], dtype=np.int32),
        "w": np.full(8, 0.25, dtype=np.float32), "srow": np.array([row, 5], dtype=np.int32),
        "scol": np.array([col, 5], dtype=np.int32), "sw": np.ones(2, dtype=np.float32),
        "swave": np.array([wave, -1], dtype=np.int32),
    }
    grid = _lib.Grid(n, n, n, 1e-3, 1e-3, 1e-7, 0x1000, 0x2000)
    rx = _lib.Receivers(2, keep["row0"].ctypes.data, keep["col0"].ctypes.data, keep["w"].ctypes.data)
    src = _lib.Sources(2, keep["srow"].ctypes.data, keep["scol"].ctypes.data, keep["sw"].ctypes.data,
                       keep["swave"].ctypes.data, 0x3000, 1, 100)
    return _lib.Problem(grid, 1, 10, rx, src), keep


@pytest.mark.parametrize("bad", [dict(wave=1), dict(wave=7), dict(row=64), dict(col=-1), dict(rx_row=63)])
def test_plain_entry_points_validate_sources_and_receivers(bad):
    """fdtd_forward_plain, fdtd_gradient_plain and fdtd_forward_plain_static return
    FDTD_ERR_INVALID for an out-of-range waveform index, source node or receiver
    before touching the device (the placeholder pointers are never dereferenced)."""
    import ctypes
    from soundwavesimulation_gb300 import _lib
    lib = _lib.load()
    prob, keep = _fake_problem(**bad)
    assert lib.fdtd_forward_plain(ctypes.byref(prob), 0x4000, 0x5000, 1 << 40, None) == 1
    assert lib.fdtd_forward_plain_static(ctypes.byref(prob), 0x4000, None) == 1
    msg = lib.fdtd_last_error().decode()
    assert "outside the grid" in msg or "waveform index" in msg, msg
    assert lib.fdtd_gradient_plain(ctypes.byref(prob), 0x4000, None, 0x6000, 0x7000, 0x5000, 1 << 40,
                                   None) == 1
    prob_ok, keep_ok = _fake_problem()
    # a valid problem passes the checks and fails only on the too-small workspace
    assert lib.fdtd_forward_plain(ctypes.byref(prob_ok), 0x4000, 0x5000, 16, None) == 3


def test_kept_segments_resolution_and_workspace():
    """fdtd_tuning.kept_segments on a gradient plan (host-side planning only, no
    device work): 0 keeps one segment (the recompute's own buffer), a negative
    count none (reported as -1), larger counts are capped at the number of
    checkpoint segments, and every kept segment beyond the first adds one segment
    buffer (ckpt_every fields) to the workspace."""
    import ctypes
    from soundwavesimulation_gb300 import _lib
    lib = _lib.load()
    prob, keep = _fake_problem(n=200)
    prob.n_steps = 300
    field = 1 * 200 * 200 * 4  # shots x ny x pitch x float32
    got = {}
    for kept in (0, -3, 1, 2, 100):
        t = _lib.Tuning(steps_per_launch=10, ckpt_every=30, kept_segments=kept)
        h = ctypes.c_void_p()
        assert lib.fdtd_plan_create(ctypes.byref(prob), ctypes.byref(t), 1, ctypes.byref(h)) == 0
        r = _lib.Tuning()
        nb = ctypes.c_size_t()
        assert lib.fdtd_plan_tuning(h, ctypes.byref(r)) == 0
        assert lib.fdtd_plan_workspace_bytes(h, ctypes.byref(nb)) == 0
        lib.fdtd_plan_destroy(h)
        got[kept] = (r.kept_segments, nb.value)
    assert [got[k][0] for k in (0, -3, 1, 2, 100)] == [1, -1, 1, 2, 10]
    assert got[0][1] == got[1][1] == got[-3][1]
    assert got[2][1] - got[1][1] == 30 * field
    assert got[100][1] - got[1][1] == 9 * 30 * field
    # a forward-only plan keeps nothing and reports the count it was given
    t = _lib.Tuning(steps_per_launch=10, kept_segments=0)
    h = ctypes.c_void_p()
    assert lib.fdtd_plan_create(ctypes.byref(prob), ctypes.byref(t), 0, ctypes.byref(h)) == 0
    r = _lib.Tuning()
    assert lib.fdtd_plan_tuning(h, ctypes.byref(r)) == 0
    lib.fdtd_plan_destroy(h)
    assert r.kept_segments == 0
