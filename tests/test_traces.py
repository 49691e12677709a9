"""Trace file format: the reference's npz keys (2DRingFDTD.py:291-327), pinned
against a file the reference's own ``save_traces`` wrote (tests/golden/trace_file.npz)."""

import numpy as np

from soundwavesimulation_gb300 import RingArray, axis_centers
from soundwavesimulation_gb300.traces import load_traces, save_traces


def _inputs():
    x = axis_centers(41, 2.0e-3)
    ring = RingArray(6, 0.030, x, x)
    traces = np.random.default_rng(3).standard_normal((6, 9)).astype(np.float32)
    return ring, traces


def test_reads_reference_file(golden):
    path = golden.path("trace_file")
    d = load_traces(path)
    ring, traces = _inputs()
    np.testing.assert_array_equal(d["traces"], traces)
    np.testing.assert_allclose(d["theta"], ring.theta, rtol=0, atol=1e-15)
    assert d["tx"] == 2 and list(d["transmitter_indices"]) == [2, 4]
    assert str(d["torch_device"]) == "cuda:0" and bool(d["torch_compiled"])


def test_writes_reference_layout(golden, tmp_path):
    ref = np.load(golden.path("trace_file"), allow_pickle=True)
    ring, traces = _inputs()
    dt = float(ref["dt"])
    out = save_traces(tmp_path / "t.npz", traces, np.arange(9) * dt, ring, 2, np.linspace(0.0, 1.0, 5), dt,
                      c_map=ref["sound_speed_m_s"], device="cuda:0", dtype="float32", compiled=True,
                      transmitter_indices=[2, 4])
    ours = np.load(out, allow_pickle=True)
    assert sorted(ours.files) == sorted(ref.files)
    for key in ref.files:
        assert ours[key].dtype == ref[key].dtype, key
        np.testing.assert_array_equal(ours[key], ref[key], err_msg=key)


def test_float16_storage_round_trip(tmp_path):
    ring, traces = _inputs()
    out = save_traces(tmp_path / "h.npz", traces, np.arange(9) * 1e-7, ring, 0, np.zeros(3), 1e-7,
                      trace_dtype="float16")
    raw = np.load(out)
    assert raw["traces"].dtype == np.float16
    d = load_traces(out)
    assert d["traces"].dtype == np.float32
    np.testing.assert_allclose(d["traces"], traces, rtol=1e-3, atol=1e-3)
