"""GPU parity of the forward path: one-step kernels and the fused engine.

The oracle (float64 NumPy restatement of the reference, pinned to the
reference's own outputs in test_oracle_golden.py) is the checker. Tolerances:
traces rel-L2 <= 1e-5 against float64 (the required trace budget), one-step
kernels <= 1e-6; the fused engine and the one-step kernels run the same
float32 arithmetic and must agree bit for bit.
"""

import numpy as np
import pytest
import torch

from oracle import fdtd_oracle as orc

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
FIELD_TOL = 5e-5  # whole final field (the 1e-5 budget is for traces)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def tb():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import torch_backend
    return torch_backend


def geo_of(d):
    g = {k: d[k] for k in ("row0", "col0", "w00", "w10", "w01", "w11")}
    g["row1"] = g["row0"] + 1
    g["col1"] = g["col0"] + 1
    return g


def ring41_objects(tb, golden, tuning=None):
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("ring41")
    x = axis_centers(41, float(d["dx"]))
    model = tb.TorchScalarWave2D(d["c_true"], float(d["dx"]), device="cuda")
    solver = tb.TorchFDTD2D(model, float(d["dt"]))
    array = RingArray(6, 0.030, x, x)
    sampler = tb.TorchRingSampler(array, device="cuda")
    return d, solver, array, sampler


def test_one_step_kernels_nonsquare(tb, golden):
    """fdtd_step (forward and adjoint), gather, scatter and image vs the reference's single steps."""
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("steps_nonsquare")
    ny, nx = d["c"].shape
    dx, dy, dt = float(d["dx"]), float(d["dy"]), float(d["dt"])
    model = tb.TorchScalarWave2D(d["c"], dx, dy, device="cuda")
    solver = tb.TorchFDTD2D(model, dt)
    ring = RingArray(5, 0.0085, axis_centers(nx, dx), axis_centers(ny, dy))
    sampler = tb.TorchRingSampler(ring, device="cuda")
    batched = tb.TorchFDTD2DBatch(solver, 2)
    batched.set_sources(d["src_rows"], d["src_cols"])
    batched.u_old.copy_(torch.as_tensor(d["u_old0"]))
    batched.u.copy_(torch.as_tensor(d["u0"]))
    u, samples = batched.step_record(torch.tensor(float(d["src_value"]), device="cuda"), sampler)
    assert rel(u.cpu(), d["fwd_u"]) < 1e-6
    assert rel(samples.cpu(), d["fwd_samples"]) < 1e-6
    batched.u_old.copy_(torch.as_tensor(d["u_old0"]))
    batched.u.copy_(torch.as_tensor(d["u0"]))
    g = batched.adjoint_step_image(torch.as_tensor(d["resid"], device="cuda"), sampler,
                                   torch.as_tensor(d["fwd_field"], device="cuda"),
                                   torch.as_tensor(d["g_in"], device="cuda"), float(d["image_scale"]))
    assert rel(batched.u.cpu(), d["adj_u"]) < 1e-6
    assert rel(g.cpu(), d["g_out"]) < 1e-6
    solver.reset()
    solver._rot.view(solver._rot.io).copy_(torch.as_tensor(d["u_old0"][0]))
    solver._rot.view(solver._rot.ic).copy_(torch.as_tensor(d["u0"][0]))
    single = solver.inject_field_and_step(torch.as_tensor(d["fwd_field"][0]), adjoint=True)
    assert rel(single.cpu(), d["single_adj"]) < 1e-6


def test_fused_ring41_matches_reference(tb, golden):
    d, solver, array, sampler = ring41_objects(tb, golden)
    nt = int(d["n_steps"])
    traces, u = tb.simulate_shots_batch(solver, sampler, torch.as_tensor(d["pulse"]), array.rows,
                                        array.cols, nt)
    assert traces.shape == (6, 6, nt)
    assert rel(traces.cpu(), d["observed"]) < TRACE_TOL
    assert rel(u.cpu(), d["batched_u"]) < FIELD_TOL


def test_traces_written_into_pinned_host_out(tb, golden):
    """simulate_shots_batch(out=...): a pinned host tensor is written by the kernels
    directly (bit for bit the device result, no copy); a device tensor likewise;
    pageable host memory and wrong shapes are refused before any launch."""
    d, solver, array, sampler = ring41_objects(tb, golden)
    nt = int(d["n_steps"])
    pulse = torch.as_tensor(d["pulse"])
    ref, _ = tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt)
    ref = ref.clone()
    host = torch.full((6, 6, nt), float("nan"), dtype=torch.float32, pin_memory=True)
    got, _ = tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt, out=host)
    torch.cuda.synchronize()
    assert got.data_ptr() == host.data_ptr()
    assert torch.equal(host, ref.cpu())
    dev = torch.empty_like(ref)
    tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt, out=dev)
    assert torch.equal(dev, ref)
    with pytest.raises(ValueError):
        tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt,
                                out=torch.empty((6, 6, nt), dtype=torch.float32))
    with pytest.raises(ValueError):
        tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt,
                                out=torch.empty((6, 5, nt), dtype=torch.float32, pin_memory=True))


def test_single_shot_matches_reference(tb, golden):
    d, solver, array, sampler = ring41_objects(tb, golden)
    nt = int(d["n_steps"])
    pulse = torch.as_tensor(d["pulse"], device="cuda")
    fused, _ = tb.simulate_shot(solver, sampler, pulse, *array.inject_rows_cols(2), nt)
    stepped, snaps = tb.simulate_shot(solver, sampler, pulse, *array.inject_rows_cols(2), nt,
                                      snapshot_stride=50)
    assert len(snaps) == (nt + 49) // 50
    assert rel(fused.cpu(), d["observed"][2]) < TRACE_TOL
    assert torch.equal(fused, stepped)  # fused engine == one-step kernels, bit for bit


def test_fused_equals_per_step_bitwise(tb, golden):
    d, solver, array, sampler = ring41_objects(tb, golden)
    nt = int(d["n_steps"])
    pulse = torch.as_tensor(d["pulse"], device="cuda", dtype=torch.float32)
    traces, u = tb.simulate_shots_batch(solver, sampler, pulse, array.rows, array.cols, nt)
    u = u.clone()
    batched = tb.TorchFDTD2DBatch(solver, 6)
    batched.set_sources(array.rows, array.cols)
    batched.reset()
    steps = []
    zero = torch.zeros((), device="cuda")
    for n in range(nt):
        _, s = batched.step_record(pulse[n] if n < pulse.numel() else zero, sampler)
        steps.append(s)
    stepped = torch.stack(steps, dim=2)
    assert torch.equal(traces, stepped)
    assert torch.equal(u, batched.u)


def test_ellipse_traces_against_float64(tb, golden):
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("ellipses64")
    n = d["c"].shape[0]
    dx = float(d["dx"])
    x = axis_centers(n, dx)
    model = tb.TorchScalarWave2D(d["c"], dx, device="cuda")
    solver = tb.TorchFDTD2D(model, float(d["dt"]))
    ring = RingArray(16, 0.45 * n * dx, x, x)
    sampler = tb.TorchRingSampler(ring, device="cuda")
    tx = d["tx"]
    wav = torch.as_tensor(d["wavelet"], dtype=torch.float32)
    traces, _ = tb.simulate_shots_batch(solver, sampler, wav, ring.rows[tx], ring.cols[tx],
                                        int(d["n_steps"]), source_values=wav)
    assert rel(traces.cpu(), d["traces_f64"]) < TRACE_TOL


def _random_problem(ny, nx, n_shots, n_rx, nt, seed, per_shot=1):
    rng = np.random.default_rng(seed)
    c = rng.uniform(1400.0, 1700.0, size=(ny, nx))
    c[ny // 3: ny // 2, nx // 4: nx // 2] = 1900.0
    dx, dy = 1.0e-3, 1.3e-3
    dt = orc.stable_dt(2000.0, dx, dy, cfl=0.4)
    row0 = rng.integers(0, ny - 1, size=n_rx)
    col0 = rng.integers(0, nx - 1, size=n_rx)
    wx = rng.uniform(0, 1, n_rx)
    wy = rng.uniform(0, 1, n_rx)
    w = np.stack([(1 - wx) * (1 - wy), wx * (1 - wy), (1 - wx) * wy, wx * wy], 1)
    srow = rng.integers(1, ny - 1, size=(n_shots, per_shot))
    scol = rng.integers(1, nx - 1, size=(n_shots, per_shot))
    sw = rng.uniform(0.5, 1.5, size=(n_shots, per_shot))
    wave = np.ones((n_shots, per_shot), dtype=np.int64)
    t = np.arange(nt) * dt
    waves = np.stack([np.sin(2e5 * t) * np.exp(-((t - 3e-5) / 1e-5) ** 2),
                      np.cos(3e5 * t) * np.exp(-((t - 2e-5) / 8e-6) ** 2)])
    return dict(c=c, dx=dx, dy=dy, dt=dt, row0=row0, col0=col0, w=w, srow=srow, scol=scol, sw=sw,
                wave=wave, waves=waves)


def _oracle_forward(p, nt):
    ny, nx = p["c"].shape
    geo = {"row0": p["row0"], "col0": p["col0"], "row1": p["row0"] + 1, "col1": p["col0"] + 1,
           "w00": p["w"][:, 0], "w10": p["w"][:, 1], "w01": p["w"][:, 2], "w11": p["w"][:, 3]}
    fields = orc.point_sources((ny, nx), p["srow"], p["scol"], p["sw"])
    values = p["waves"][p["wave"][:, 0]]
    traces, _, _, _ = orc.simulate_shots_batch(p["c"], p["dx"], p["dy"], p["dt"], geo, fields, values, nt)
    return traces


@pytest.mark.parametrize("ny,nx,shots,nt,tuning", [
    (41, 37, 3, 90, {"steps_per_launch": 5}),
    (67, 130, 2, 61, {"steps_per_launch": 7, "rows_per_lane": 4, "warps": 16}),
    (150, 133, 2, 40, {"steps_per_launch": 12}),
    (257, 261, 1, 33, {"steps_per_launch": 16, "warps": 12}),
    (129, 128, 2, 25, {"steps_per_launch": 1}),
    (200, 140, 2, 37, {"steps_per_launch": 3, "rows_per_lane": 4, "warps": 10}),
    (300, 211, 2, 47, {"steps_per_launch": 11, "rows_per_lane": 8, "warps": 12}),
    (260, 300, 2, 41, {"steps_per_launch": 9, "rows_per_lane": 4, "warps": 32}),
])
def test_fused_engine_shapes_and_tunings(tb, ny, nx, shots, nt, tuning):
    """Odd sizes, several tiles, edge-straddling receivers, multi-node sources, every tuning family."""
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan
    p = _random_problem(ny, nx, shots, 24, nt, seed=ny * 7 + nx, per_shot=2)
    medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
    waves = torch.as_tensor(p["waves"], dtype=torch.float32, device="cuda")
    wave_idx = np.stack([p["wave"][:, 0], 1 - p["wave"][:, 0]], 1)
    plan = FusedPlan(medium, (p["row0"], p["col0"], p["w"]), (p["srow"], p["scol"], p["sw"], wave_idx),
                     waves, nt, tuning=tuning)
    traces = plan.forward().cpu().numpy()
    q = dict(p)
    geo = {"row0": p["row0"], "col0": p["col0"], "row1": p["row0"] + 1, "col1": p["col0"] + 1,
           "w00": p["w"][:, 0], "w10": p["w"][:, 1], "w01": p["w"][:, 2], "w11": p["w"][:, 3]}
    fields = np.zeros((shots, ny, nx))
    ref = np.zeros_like(traces, dtype=np.float64)
    # two waveforms per shot: superpose two oracle runs (the engine is linear in the sources)
    for k in range(2):
        fields = orc.point_sources((ny, nx), p["srow"][:, k:k + 1], p["scol"][:, k:k + 1], p["sw"][:, k:k + 1])
        values = p["waves"][wave_idx[:, k]]
        tr, _, _, _ = orc.simulate_shots_batch(p["c"], p["dx"], p["dy"], p["dt"], geo, fields, values, nt)
        ref += tr
    del q
    assert rel(traces, ref) < TRACE_TOL


@pytest.mark.parametrize("tuning", [{"steps_per_launch": 6, "rows_per_lane": 4, "warps": 16},
                                    {"steps_per_launch": 13}])
def test_fused_many_sources_per_shot(tb, tuning):
    """Focused-arc style shots: 40 injection nodes per shot with three waveforms
    (2DArcFDTD.py:203-228 fires every transmit element with its own delayed
    waveform), two entries sharing one node, nodes spread over several tiles."""
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan
    ny, nx, S, K, nt = 140, 170, 2, 40, 70
    p = _random_problem(ny, nx, S, 30, nt, seed=77, per_shot=K)
    rng = np.random.default_rng(5)
    wave_idx = rng.integers(0, 3, size=(S, K))
    p["srow"][:, 1] = p["srow"][:, 0]
    p["scol"][:, 1] = p["scol"][:, 0]
    waves = np.concatenate([p["waves"], -0.5 * p["waves"][:1]])
    medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
    plan = FusedPlan(medium, (p["row0"], p["col0"], p["w"]), (p["srow"], p["scol"], p["sw"], wave_idx),
                     torch.as_tensor(waves, dtype=torch.float32, device="cuda"), nt, tuning=tuning)
    traces = plan.forward().cpu().numpy()
    geo = {"row0": p["row0"], "col0": p["col0"], "row1": p["row0"] + 1, "col1": p["col0"] + 1,
           "w00": p["w"][:, 0], "w10": p["w"][:, 1], "w01": p["w"][:, 2], "w11": p["w"][:, 3]}
    ref = np.zeros(traces.shape)
    for k in range(3):  # the engine is linear in the sources: one oracle run per waveform
        fields = orc.point_sources((ny, nx), p["srow"], p["scol"], p["sw"] * (wave_idx == k))
        values = np.repeat(waves[k][None], S, axis=0)
        tr, _, _, _ = orc.simulate_shots_batch(p["c"], p["dx"], p["dy"], p["dt"], geo, fields, values, nt)
        ref += tr
    assert rel(traces, ref) < TRACE_TOL


def test_simulate_sources_arc_firing_matches_per_step_form(tb):
    """Focused firing of a 16-element transmit arc, each element with its own
    delayed chirp, recorded on a separate receive arc: the fused engine against
    the per-step dense-injection form (2DArcFDTD.py:203-228)."""
    from soundwavesimulation_gb300 import ArcArray, axis_centers, linear_chirp, stable_dt
    n, dx, nt = 96, 0.4e-3, 160
    x = axis_centers(n, dx)
    c = np.full((n, n), 1500.0)
    c[30:60, 40:70] = 1650.0
    dt = stable_dt(1650.0, dx, dx, cfl=0.4)
    tx = ArcArray(16, 0.4 * n * dx, 60.0, 180.0, x, x)
    rx = ArcArray(20, 0.4 * n * dx, 60.0, 0.0, x, x)
    model = tb.TorchScalarWave2D(c, dx, device="cuda")
    solver = tb.TorchFDTD2D(model, dt)
    sampler = tb.TorchRingSampler(rx, device="cuda")
    pulse = linear_chirp(dt, 60 * dt, 2e5, 6e5)
    values = np.zeros((tx.n_elements, nt))
    for k in range(tx.n_elements):
        d = 2 * k
        values[k, d:d + pulse.size] = pulse[:nt - d]
    fused, _ = tb.simulate_sources(solver, sampler, tx.rows, tx.cols, values, nt)
    fused = fused.cpu().numpy()
    stepped, snaps = tb.simulate_sources(solver, sampler, tx.rows, tx.cols, values, nt, snapshot_steps=(nt - 1,))
    assert rel(fused, stepped.cpu().numpy()) < 1e-6
    assert set(snaps) == {nt - 1}


def test_graph_replay_matches_eager_launches(tb):
    """The forward / adjoint launch sequences replayed as CUDA graphs give the bits
    of host-launched kernels, also after the output buffers change."""
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, residual_misfit
    ny, nx, S, nt = 150, 133, 3, 53
    p = _random_problem(ny, nx, S, 20, nt, seed=21)
    medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
    waves = torch.as_tensor(p["waves"], dtype=torch.float32, device="cuda")
    src = (p["srow"], p["scol"], p["sw"], p["wave"])
    rx = (p["row0"], p["col0"], p["w"])
    out = {}
    for eager in (1, 0):
        plan = FusedPlan(medium, rx, src, waves, nt, for_gradient=True,
                         tuning={"steps_per_launch": 6, "eager": eager})
        runs = []
        for _ in range(3):  # fresh output buffers every call: a new graph each time
            tr = plan.forward(save_checkpoints=True)
            res, _ = residual_misfit(tr, torch.zeros_like(tr), None)
            g = torch.zeros((ny, medium.pitch), dtype=torch.float64, device="cuda")
            plan.adjoint(res, g)
            runs.append((tr.clone(), g))
        trs = [r[0] for r in runs]
        assert all(torch.equal(trs[0], t) for t in trs[1:])
        out[eager] = runs[0]
    assert torch.equal(out[0][0], out[1][0])
    assert rel(out[0][1].cpu().numpy(), out[1][1].cpu().numpy()) < 1e-12


def test_graph_kept_across_in_place_medium_updates(tb):
    """A plan keeps its captured graph while the medium changes in place (same
    buffers) and sees the new values: traces and gradient equal a fresh plan's on
    the new medium, with the same output buffers (the graph replayed)."""
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, residual_misfit
    ny, nx, S, nt = 140, 121, 2, 47
    p = _random_problem(ny, nx, S, 20, nt, seed=5)
    waves = torch.as_tensor(p["waves"], dtype=torch.float32, device="cuda")
    src = (p["srow"], p["scol"], p["sw"], p["wave"])
    rx = (p["row0"], p["col0"], p["w"])
    tun = {"steps_per_launch": 6}
    medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
    plan = FusedPlan(medium, rx, src, waves, nt, tuning=tun, for_gradient=True)
    tr = torch.empty((S, len(p["row0"]), nt), dtype=torch.float32, device="cuda")
    res = torch.empty_like(tr)
    zero = torch.zeros_like(tr)
    g = torch.zeros((ny, medium.pitch), dtype=torch.float64, device="cuda")

    def gradient():  # the same buffers every time: both graphs are replayed
        plan.forward(tr, save_checkpoints=True)
        residual_misfit(tr, zero, None, residual=res)
        g.zero_()
        plan.adjoint(res, g)

    gradient()
    c2 = p["c"] * 1.03
    medium.set_c(c2)                       # in place: same coefficient buffers
    gradient()
    fresh_medium = DeviceMedium(c2, p["dx"], p["dy"], p["dt"], "cuda")
    fresh = FusedPlan(fresh_medium, rx, src, waves, nt, tuning=tun, for_gradient=True)
    tr2 = fresh.forward(save_checkpoints=True)
    res2, _ = residual_misfit(tr2.clone(), torch.zeros_like(tr2), None)
    g2 = torch.zeros_like(g)
    fresh.adjoint(res2, g2)
    assert torch.equal(tr, tr2)
    assert rel(g.cpu().numpy(), g2.cpu().numpy()) < 1e-12


@pytest.mark.parametrize("shape", [{"rows_per_lane": 8, "warps": 16}, {"rows_per_lane": 4, "warps": 32},
                                   {"rows_per_lane": 8, "warps": 16, "kept_segments": 1}])
def test_plan_group_matches_separate_plans(tb, shape):
    """Three grids of different sizes, step counts and temporal-block depths in shared
    launches: traces equal each plan run alone (bitwise), gradients to float64
    summation order; with every segment's stencil stream kept by the forward (the
    default at these sizes) and with one kept segment (the rest recomputed)."""
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, PlanGroup, residual_misfit
    cases = [(96, 90, 3, 47, 6), (150, 133, 2, 61, 9), (70, 201, 4, 33, 5)]
    plans, alone = [], []
    for i, (ny, nx, S, nt, T) in enumerate(cases):
        p = _random_problem(ny, nx, S, 20, nt, seed=60 + i)
        medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
        waves = torch.as_tensor(p["waves"], dtype=torch.float32, device="cuda")
        args = (medium, (p["row0"], p["col0"], p["w"]), (p["srow"], p["scol"], p["sw"], p["wave"]), waves, nt)
        tuning = dict(shape, steps_per_launch=T)
        plans.append(FusedPlan(*args, tuning=tuning, for_gradient=True))
        alone.append(FusedPlan(*args, tuning=tuning, for_gradient=True))
    group = PlanGroup(plans)
    traces = group.forward(save_checkpoints=True)
    grads = [torch.zeros((p.medium.ny, p.medium.pitch), dtype=torch.float64, device="cuda") for p in plans]
    group.adjoint([residual_misfit(t, torch.zeros_like(t), None)[0] for t in traces], grads)
    for plan, tr, g in zip(alone, traces, grads):
        ref = plan.forward(save_checkpoints=True)
        assert torch.equal(ref, tr)
        g_ref = torch.zeros_like(g)
        plan.adjoint(residual_misfit(ref, torch.zeros_like(ref), None)[0], g_ref)
        assert rel(g.cpu().numpy(), g_ref.cpu().numpy()) < 1e-12


@pytest.mark.parametrize("for_gradient", [False, True])
def test_library_autotuner_picks_a_working_shape(tb, for_gradient):
    """fdtd_autotune (the C-ABI launch-shape search) reports every shape it timed,
    returns the fastest of them, and the chosen shape reproduces the default
    shape's traces bit for bit."""
    from soundwavesimulation_gb300.autotune import autotune, clear_cache
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan
    p = _random_problem(200, 180, 3, 20, 60, seed=11, per_shot=1)
    medium = DeviceMedium(p["c"], p["dx"], p["dy"], p["dt"], "cuda")
    waves = torch.as_tensor(p["waves"], dtype=torch.float32, device="cuda")
    rx = (p["row0"], p["col0"], p["w"])
    src = (p["srow"], p["scol"], p["sw"], p["wave"])
    clear_cache()
    best = autotune(medium, rx, src, waves, 60, launches=2, repeats=1, for_gradient=for_gradient)
    assert best["rows_per_lane"] in (4, 8) and 6 <= best["steps_per_launch"] <= 23
    ref = FusedPlan(medium, rx, src, waves, 60).forward()
    got = FusedPlan(medium, rx, src, waves, 60, tuning=best).forward()
    assert torch.equal(ref, got)
