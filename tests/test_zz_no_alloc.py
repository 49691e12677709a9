"""The workspace-free forward entry point, checked against the workspace one.

``fdtd_forward_plain_static`` exists for callers that cannot allocate device
memory (a process whose device memory belongs to another allocator's pool, or a
binding of the C ABI that has only its own buffers and a stream); its scratch is
a fixed device array inside the library. This file is collected last so that a
run stopping at the first failure has run every other test before it; it also
passes on its own in a fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import RingArray, axis_centers, ricker, stable_dt, _lib
    from soundwavesimulation_gb300.engine import DeviceMedium, ProblemTables, forward_plain
    from soundwavesimulation_gb300.phantoms import random_ellipses
    n, dx, nt = 96, 0.5e-3, 220
    c, _ = random_ellipses(n, dx, 4, seed=21)
    dt = stable_dt(float(c.max()), dx, dx, cfl=0.3)
    x = axis_centers(n, dx)
    ring = RingArray(20, 0.42 * n * dx, x, x)
    tx = np.array([0, 5, 11])
    src = [t[:, None] if i < 2 else t for i, t in enumerate(
        (ring.rows[tx], ring.cols[tx], np.ones((3, 1)), np.zeros((3, 1), dtype=np.int64)))]
    medium = DeviceMedium(c, dx, dx, dt, "cuda")
    waves = torch.as_tensor(ricker(3e5, dt, nt)[None], dtype=torch.float32, device="cuda")
    tables = ProblemTables(medium, ring.receiver_taps(), tuple(src), waves, nt)
    expected = forward_plain(tables)
    torch.cuda.synchronize()
    return _lib, tables, expected


def _call(lib, tables, traces):
    prob = tables.problem()
    stream = torch.cuda.current_stream().cuda_stream
    return lib.load().fdtd_forward_plain_static(ctypes.byref(prob), traces.data_ptr(), stream)


def test_static_scratch_forward_matches_workspace_forward_twice(setup):
    lib, tables, expected = setup
    for _ in range(2):  # the second call starts from the first call's leftover scratch
        traces = torch.full_like(expected, float("nan"))
        rc = _call(lib, tables, traces)
        assert rc == 0, lib.load().fdtd_last_error().decode()
        torch.cuda.synchronize()
        assert _rel(traces, expected) <= 1e-6
        assert torch.equal(traces, expected)


def test_static_scratch_rejects_oversized_problem(setup):
    lib, tables, _ = setup
    from soundwavesimulation_gb300.engine import ProblemTables
    big = ProblemTables.__new__(ProblemTables)
    big.__dict__.update(tables.__dict__)
    prob = big.problem()
    prob.grid.ny = 2048
    prob.grid.nx = 2048
    prob.grid.pitch = 2048
    traces = torch.empty(1, device="cuda")
    rc = lib.load().fdtd_forward_plain_static(ctypes.byref(prob), traces.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream)
    assert rc == 3  # FDTD_ERR_WORKSPACE, rejected before any device work
    assert b"fixed" in lib.load().fdtd_last_error()


def test_static_scratch_rejects_bad_waveform_index(setup):
    """A source entry naming a waveform the table does not hold is refused with
    FDTD_ERR_INVALID before any device work: the traces stay untouched."""
    lib, tables, _ = setup
    from soundwavesimulation_gb300.engine import ProblemTables
    bad = ProblemTables.__new__(ProblemTables)
    bad.__dict__.update(tables.__dict__)
    bad._s_wave = tables._s_wave.copy()
    bad._s_wave[1, 0] = 5  # the table holds one waveform
    traces = torch.full((3, 20, 4), float("nan"), device="cuda")
    rc = _call(lib, bad, traces)
    torch.cuda.synchronize()
    assert rc == 1
    assert b"waveform index" in lib.load().fdtd_last_error()
    assert torch.isnan(traces).all()
