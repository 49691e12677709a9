"""GPU parity of the PML option (no reference counterpart; the reference has
first-order Mur edges only, fdtd2d/solver.py:90-124).

The checker is the float64 PML restatement (oracle/fdtd_oracle.c, pinned to the
NumPy restatement, an unbounded grid, the water line-source trace and central
differences in tests/test_pml_oracle.py). Budgets: traces rel-L2 <= 1e-5 and
gradient rel-L2 <= 1e-3 against float64; the fused kernel and the one-step PML
kernel run the same float32 arithmetic and agree bit for bit.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import c_oracle
from oracle import fdtd_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import _lib, engine
    return _lib, engine


def _problem(ny, nx, n_shots, nt, seed):
    rng = np.random.default_rng(seed)
    dx = 0.25e-3
    c = 1480.0 + 150.0 * rng.random((ny, nx))
    c[ny // 3: ny // 2, nx // 4: nx // 2] = 1750.0
    dt = orc.stable_dt(c.max(), dx, dx, 0.3)
    x, y = orc.axis_centers(nx, dx), orc.axis_centers(ny, dx)
    geo = orc.ring_geometry(24, 0.4 * min(nx, ny) * dx, x, y)
    tx = np.arange(n_shots) * (24 // n_shots)
    taps = [orc.bilinear_source_taps(geo, t) for t in tx]
    rows, cols, w = (np.stack([t[i] for t in taps]) for i in range(3))
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    t = np.arange(nt) * dt
    f0 = 3.0e5
    a = (np.pi * f0 * (t - 1.5 / f0)) ** 2
    wav = (1 - 2 * a) * np.exp(-a)
    return dict(c=c, dx=dx, dt=dt, geo=geo, tx=tx, src=(rows, cols, w), rx=rx, wav=wav, nt=nt, x=x, y=y)


def _plan(engine, medium, p, tuning=None, for_gradient=False, truth=False):
    rows, cols, w = p["src"]
    waves = torch.as_tensor(p["wav"][None], dtype=torch.float32, device="cuda")
    return engine.FusedPlan(medium, p["rx"], (rows, cols, w, np.zeros(rows.shape, dtype=np.int64)), waves, p["nt"],
                            tuning=tuning, for_gradient=for_gradient)


@pytest.mark.parametrize("ny,nx,P,tuning", [
    (150, 133, 20, {"rows_per_lane": 8, "warps": 16, "steps_per_launch": 12}),
    (171, 260, 30, {"rows_per_lane": 4, "warps": 16, "steps_per_launch": 9}),
    (200, 141, 12, {"rows_per_lane": 8, "warps": 12, "steps_per_launch": 15}),
    (129, 300, 25, {"rows_per_lane": 4, "warps": 16, "steps_per_launch": 7}),
])
def test_fused_pml_traces_vs_float64_and_one_step_kernel(eng, ny, nx, P, tuning):
    _lib, engine = eng
    p = _problem(ny, nx, 3, 260, seed=ny + nx)
    medium = engine.DeviceMedium(p["c"], p["dx"], p["dx"], p["dt"], "cuda", pml_cells=P)
    traces = _plan(engine, medium, p, tuning).forward()
    ref = c_oracle.forward_shots(p["c"], p["dx"], p["dx"], p["dt"], p["src"], p["rx"], p["wav"], p["nt"], pml=P)
    assert rel(traces.cpu().numpy(), ref) < 1e-5
    # the one-step PML kernel, one launch per step, gathers after every step
    tables = engine.ProblemTables(medium, p["rx"], (*p["src"], np.zeros(p["src"][0].shape, dtype=np.int64)),
                                  torch.as_tensor(p["wav"][None], dtype=torch.float32, device="cuda"), p["nt"])
    lib = _lib.load()
    S = len(p["tx"])
    f = [medium.new_field(S) for _ in range(3)]
    psi = [[medium.new_field(S) for _ in range(2)] for _ in range(2)]
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    srow, scol = dev(tables._s_row, torch.int32), dev(tables._s_col, torch.int32)
    sw, swave = dev(tables._s_w, torch.float32), dev(tables._s_wave, torch.int32)
    rc = dev(np.stack([tables._rx_row0, tables._rx_col0], 1), torch.int32)
    rw = dev(tables._rx_w, torch.float32)
    out = torch.empty_like(traces)
    grid = medium.grid()
    stream = torch.cuda.current_stream().cuda_stream
    io, ic, inx, ps = 0, 1, 2, 0
    for n in range(p["nt"]):
        _lib.check(lib.fdtd_step_pml(ctypes.byref(grid), S, f[io].data_ptr(), f[ic].data_ptr(), f[inx].data_ptr(),
                                     psi[ps][0].data_ptr(), psi[ps][1].data_ptr(), psi[ps ^ 1][0].data_ptr(),
                                     psi[ps ^ 1][1].data_ptr(), tables._s_row.shape[1], srow.data_ptr(),
                                     scol.data_ptr(), sw.data_ptr(), swave.data_ptr(), tables.waveforms.data_ptr(),
                                     p["nt"], n, None, 0, stream), "step_pml")
        _lib.check(lib.fdtd_gather(ctypes.byref(grid), S, f[inx].data_ptr(), len(p["rx"][0]), rc.data_ptr(),
                                   rw.data_ptr(), out[:, :, n:].data_ptr(), out.stride(0), out.stride(1), stream),
                   "gather")
        io, ic, inx, ps = ic, inx, io, ps ^ 1
    assert torch.equal(out, traces), float((out - traces).abs().max())


def test_pml_gradient_vs_float64(eng):
    _lib, engine = eng
    p = _problem(160, 150, 2, 300, seed=4)
    P = 20
    truth = engine.DeviceMedium(p["c"], p["dx"], p["dx"], p["dt"], "cuda", pml_cells=P)
    observed = _plan(engine, truth, p).forward()
    c0 = p["c"] * 1.015  # a start whose arrivals already differ: a well-posed misfit
    start = engine.DeviceMedium(c0, p["dx"], p["dx"], p["dt"], "cuda", pml_cells=P)
    plan = _plan(engine, start, p, {"ckpt_every": 48}, for_gradient=True)
    pred = plan.forward(save_checkpoints=True)
    mute = torch.as_tensor(p["tx"], dtype=torch.int32, device="cuda")
    res, misfit = engine.residual_misfit(pred, observed, mute)
    g = torch.zeros((start.ny, start.pitch), dtype=torch.float64, device="cuda")
    plan.adjoint(res, g)
    J64, g64 = c_oracle.gradient_shots(c0, p["dx"], p["dx"], p["dt"], p["src"], p["rx"], p["wav"], p["nt"],
                                       observed.cpu().numpy().astype(np.float64), p["tx"], ckpt_every=30, pml=P)
    mask = orc.interior_mask(p["x"], p["y"], 0.4 * 150 * p["dx"], 2 * p["dx"])
    gm = start.physical(g).cpu().numpy()
    assert abs(float(misfit.item()) - J64) / J64 < 1e-5
    assert rel(np.where(mask, gm, 0.0), np.where(mask, g64, 0.0)) < 1e-3


def test_pml_reflection_on_the_gpu(eng):
    """Water, one shot: the engine's PML trace against the same shot on a grid so
    large that no edge echo arrives (the float64 oracle), Mur for comparison."""
    _lib, engine = eng
    n, dx, nt = 120, 0.2e-3, 900
    c = np.full((n, n), 1500.0)
    dt = orc.stable_dt(1500.0, dx, dx, 0.3)
    x = orc.axis_centers(n, dx)
    geo = orc.ring_geometry(32, 0.45 * n * dx, x, x)
    f0 = 0.4e6
    t = np.arange(nt) * dt
    a = (np.pi * f0 * (t - 1.5 / f0)) ** 2
    wav = (1 - 2 * a) * np.exp(-a)
    rows, cols = geo["rows"][[0]][:, None], geo["cols"][[0]][:, None]
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    big = 300
    ref = c_oracle.forward_shots(np.pad(c, big, mode="edge"), dx, dx, dt, (rows + big, cols + big, np.ones(rows.shape)),
                                 (rx[0] + big, rx[1] + big, rx[2]), wav, nt)
    waves = torch.as_tensor(wav[None], dtype=torch.float32, device="cuda")
    out = {}
    for P in (0, 30):
        medium = engine.DeviceMedium(c, dx, dx, dt, "cuda", pml_cells=P)
        plan = engine.FusedPlan(medium, rx, (rows, cols, np.ones(rows.shape), np.zeros(rows.shape, dtype=np.int64)),
                                waves, nt)
        out[P] = rel(plan.forward().cpu().numpy(), ref)
    assert out[0] > 0.1 and out[30] < 1e-3, out


def test_fwi_driver_on_a_pml_solver(eng):
    """TorchLeastSquaresFWI with a PML solver: misfit and masked gradient against
    the float64 oracle (the reference's API with the layer as an option)."""
    from soundwavesimulation_gb300 import RingArray, axis_centers, fwi, interior_mask, stable_dt
    from soundwavesimulation_gb300 import torch_backend as tb
    n, dx, nt, S = 96, 0.4e-3, 260, 8
    rng = np.random.default_rng(2)
    c_true = 1500.0 + 60.0 * rng.random((n, n))
    c0 = np.full((n, n), 1520.0)
    dt = stable_dt(1700.0, dx, dx, cfl=0.3)
    x = axis_centers(n, dx)
    ring = RingArray(S, 0.4 * n * dx, x, x)
    t = np.arange(nt) * dt
    a = (np.pi * 2.5e5 * (t - 6e-6)) ** 2
    wav = (1 - 2 * a) * np.exp(-a)
    P = 16
    truth = tb.TorchFDTD2D(tb.TorchScalarWave2D(c_true, dx, device="cuda"), dt, pml_cells=P)
    sampler = tb.TorchRingSampler(ring, device="cuda")
    observed, _ = tb.simulate_shots_batch(truth, sampler, wav, ring.rows, ring.cols, nt)
    solver = tb.TorchFDTD2D(tb.TorchScalarWave2D(c0, dx, device="cuda"), dt, pml_cells=P)
    mask = interior_mask(x, x, 0.4 * n * dx, 3 * dx)
    problem = fwi.TorchLeastSquaresFWI(solver, sampler, ring, wav, nt, S, observed.clone(), mask, parallel_shots=S)
    J, g_c2 = problem.gradient_c2(1.0 / c0 ** 2, np.arange(S))
    src = (ring.rows[:, None], ring.cols[:, None], np.ones((S, 1)))
    J64, g64 = c_oracle.gradient_shots(c0, dx, dx, dt, src, ring.receiver_taps(), wav, nt,
                                       observed.cpu().numpy().astype(np.float64), np.arange(S), pml=P)
    assert abs(J - J64) / J64 < 1e-5
    assert rel(np.where(mask, g_c2, 0.0), np.where(mask, g64, 0.0)) < 1e-3
