"""GPU parity of the FWI gradient: fused checkpointed adjoint vs the reference and the oracle.

Tolerances: gradient rel-L2 <= 1e-3 against float64 (the required budget; the
float32 engine lands near 1e-5), misfit rel 1e-5. The checkpointed gradient must
not depend on the checkpoint spacing beyond float32 summation order, and 16-bit
checkpoints must stay within 1e-3 of float32 storage.
"""

import numpy as np
import pytest
import torch

from oracle import fdtd_oracle as orc

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import fwi, torch_backend
    return torch_backend, fwi


def ring41_problem(mods, golden, **options):
    tb, fwi = mods
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("ring41")
    x = axis_centers(41, float(d["dx"]))
    model = tb.TorchScalarWave2D(d["c_true"], float(d["dx"]), device="cuda")
    solver = tb.TorchFDTD2D(model, float(d["dt"]))
    array = RingArray(6, 0.030, x, x)
    sampler = tb.TorchRingSampler(array, device="cuda")
    problem = fwi.TorchLeastSquaresFWI(
        solver, sampler, array, torch.as_tensor(d["pulse"]), int(d["n_steps"]), 6,
        torch.as_tensor(d["observed"]), d["mask"], c_min=1400.0, c_max=2000.0,
        c_background=1500.0, **options)
    return d, problem


@pytest.mark.parametrize("options", [{"parallel_shots": 6}, {"parallel_shots": 4},
                                     {"parallel_shots": 1}, {"ckpt_every": 12, "parallel_shots": 6}])
def test_ring41_gradient_matches_reference(mods, golden, options):
    d, problem = ring41_problem(mods, golden, **options)
    J, g = problem.misfit_and_grad(d["m0"])
    assert J == pytest.approx(float(d["misfit"]), rel=1e-5)
    assert rel(g, d["grad_m"]) < GRAD_TOL
    assert rel(g, d["grad_m"]) < 1e-4  # what float32 actually reaches on this problem


def test_ring41_unmasked_g_c2_and_misfit(mods, golden):
    d, problem = ring41_problem(mods, golden, parallel_shots=6)
    J, g_c2 = problem.gradient_c2(d["m0"], np.arange(6))
    assert rel(g_c2, d["g_c2"]) < 1e-4
    assert J == pytest.approx(float(d["residual_misfit"]), rel=1e-5)
    J2 = problem.misfit(d["m0"])
    assert J2 == pytest.approx(float(d["misfit"]), rel=1e-5)


def test_ellipse_gradient_vs_reference(mods, golden):
    tb, fwi = mods
    from soundwavesimulation_gb300 import RingArray, axis_centers
    d = golden("ellipses64")
    n = d["c"].shape[0]
    dx, dt, nt = float(d["dx"]), float(d["dt"]), int(d["n_steps"])
    x = axis_centers(n, dx)
    ring = RingArray(16, 0.45 * n * dx, x, x)
    geo = orc.ring_geometry(16, 0.45 * n * dx, x, x)
    obs, _, _, _ = orc.simulate_shots_batch(d["c"], dx, dx, dt, geo,
                                            orc.point_sources(d["c"].shape, ring.rows, ring.cols),
                                            d["wavelet"], nt)
    model = tb.TorchScalarWave2D(d["c"], dx, device="cuda")
    solver = tb.TorchFDTD2D(model, dt)
    sampler = tb.TorchRingSampler(ring, device="cuda")
    problem = fwi.TorchLeastSquaresFWI(solver, sampler, ring, d["wavelet"], nt, 16,
                                       torch.as_tensor(obs, dtype=torch.float32), d["mask"],
                                       parallel_shots=16, tuning={"steps_per_launch": 8})
    J, g_c2 = problem.gradient_c2(1.0 / d["c_start"] ** 2, d["tx"])
    assert rel(g_c2, d["g_c2_tx"]) < GRAD_TOL
    assert J == pytest.approx(float(d["misfit_tx"]), rel=1e-4)
    J_all, g_all = problem.misfit_and_grad(d["m_start"])
    assert rel(g_all, d["grad_m_all"]) < GRAD_TOL
    assert J_all == pytest.approx(float(d["misfit_all"]), rel=1e-4)


def test_checkpoint_spacing_and_16bit_storage(mods, golden):
    d, exact = ring41_problem(mods, golden, parallel_shots=6, tuning={"steps_per_launch": 4})
    _, g_ref = exact.gradient_c2(d["m0"], np.arange(6))
    for every in (4, 8, 40, 204):
        _, p = ring41_problem(mods, golden, parallel_shots=6, ckpt_every=every,
                              tuning={"steps_per_launch": 4})
        _, g = p.gradient_c2(d["m0"], np.arange(6))
        assert rel(g, g_ref) < 1e-6
    # float16 checkpoints (11-bit significand, power-of-two scale) keep the 1e-3
    # gradient budget; bfloat16 (8-bit significand) does not, and the engine warns
    _, p = ring41_problem(mods, golden, parallel_shots=6, wave_dtype=torch.float16, ckpt_every=20,
                          tuning={"steps_per_launch": 4})
    _, g = p.gradient_c2(d["m0"], np.arange(6))
    assert rel(g, g_ref) < 1e-3
    with pytest.warns(UserWarning, match="bfloat16"):
        _, p = ring41_problem(mods, golden, parallel_shots=6, wave_dtype=torch.bfloat16, ckpt_every=20,
                              tuning={"steps_per_launch": 4})
        _, g = p.gradient_c2(d["m0"], np.arange(6))
    assert float(np.sum(g * g_ref) / (np.linalg.norm(g) * np.linalg.norm(g_ref))) > 0.999


def _ellipse_gradient_case(nt=300):
    """150^2 ellipse medium, 3 shots of a 40-element ring, a start model with the
    inclusions halved: (true medium, start medium, ring, tx, sources, waveforms, nt)."""
    from soundwavesimulation_gb300.engine import DeviceMedium
    from soundwavesimulation_gb300.phantoms import random_ellipses
    from soundwavesimulation_gb300 import RingArray, axis_centers, stable_dt, ricker
    n, dx = 150, 0.35e-3
    c, _ = random_ellipses(n, dx, 5, seed=3)
    dt = stable_dt(float(c.max()), dx, dx, cfl=0.3)
    x = axis_centers(n, dx)
    ring = RingArray(40, 0.45 * n * dx, x, x)
    tx = np.array([0, 7, 13])
    rows, cols = ring.rows[tx][:, None], ring.cols[tx][:, None]
    src = (rows, cols, np.ones(rows.shape), np.zeros(rows.shape, dtype=np.int64))
    waves = torch.as_tensor(ricker(3e5, dt, nt)[None], dtype=torch.float32, device="cuda")
    true = DeviceMedium(c, dx, dx, dt, "cuda")
    start = DeviceMedium(np.where(c > 1500.0, 0.5 * (c + 1500.0), c), dx, dx, dt, "cuda")
    return true, start, ring, tx, src, waves, nt


@pytest.mark.parametrize("tuning", [{"steps_per_launch": 10},
                                    {"steps_per_launch": 10, "kept_segments": -1},
                                    {"steps_per_launch": 9, "rows_per_lane": 4, "warps": 32},
                                    {"steps_per_launch": 7, "rows_per_lane": 8, "warps": 12}])
def test_fused_gradient_equals_plain_form(mods, tuning):
    """Checkpointed fused gradient vs the plain per-shot full-history gradient, per launch
    shape; with every segment's stencil stream kept by the forward (the default at this
    size) and with every segment recomputed (kept_segments -1)."""
    from soundwavesimulation_gb300.engine import FusedPlan, ProblemTables, gradient_plain
    from soundwavesimulation_gb300.engine import residual_misfit
    true, start, ring, tx, src, waves, nt = _ellipse_gradient_case()
    n = start.ny
    observed = FusedPlan(true, ring.receiver_taps(), src, waves, nt).forward().clone()
    plan = FusedPlan(start, ring.receiver_taps(), src, waves, nt, for_gradient=True, tuning=tuning)
    traces = plan.forward(save_checkpoints=True)
    res, J = residual_misfit(traces, observed, tx)
    g = torch.zeros((n, start.pitch), dtype=torch.float64, device="cuda")
    plan.adjoint(res, g)
    Jp, gp = gradient_plain(ProblemTables(start, ring.receiver_taps(), src, waves, nt), observed, tx)
    assert float(J) == pytest.approx(float(Jp), rel=1e-6)
    assert rel(g.cpu(), gp.cpu()) < 1e-6


@pytest.mark.parametrize("store", [0, 1])
def test_kept_segments_leave_traces_and_gradient_unchanged(mods, store):
    """The forward keeps the stencil stream of the last kept_segments checkpoint
    segments (their recompute is skipped): traces are bit for bit those of the plain
    forward, and the gradient equals the all-recompute gradient to float64 summation
    order with float32 checkpoints (16-bit checkpoints: the kept segments image the
    exact stream, the recomputed ones the stream from rounded checkpoints)."""
    from soundwavesimulation_gb300.engine import FusedPlan, residual_misfit
    true, start, ring, tx, src, waves, nt = _ellipse_gradient_case(nt=290)
    observed = FusedPlan(true, ring.receiver_taps(), src, waves, nt).forward().clone()
    base = {"steps_per_launch": 10, "ckpt_every": 30, "ckpt_store": store}  # 10 segments, the last short
    ref_plan = FusedPlan(start, ring.receiver_taps(), src, waves, nt, for_gradient=True,
                         tuning={**base, "kept_segments": -1})
    assert ref_plan.tuning["kept_segments"] == -1
    ref_tr = ref_plan.forward(save_checkpoints=True).clone()
    res, _ = residual_misfit(ref_tr, observed, tx)
    g_ref = torch.zeros((start.ny, start.pitch), dtype=torch.float64, device="cuda")
    ref_plan.adjoint(res, g_ref)
    for kept in (1, 3, 10, 25):
        plan = FusedPlan(start, ring.receiver_taps(), src, waves, nt, for_gradient=True,
                         tuning={**base, "kept_segments": kept})
        assert plan.tuning["kept_segments"] == min(kept, 10)
        tr = plan.forward(save_checkpoints=True)
        assert torch.equal(tr, ref_tr)
        res_k, _ = residual_misfit(tr, observed, tx)
        g = torch.zeros_like(g_ref)
        plan.adjoint(res_k, g)
        assert rel(g.cpu(), g_ref.cpu()) < (1e-12 if store == 0 else 2e-3), kept
        # a second pass through the same plan (graph replay) gives the same gradient
        g2 = torch.zeros_like(g_ref)
        plan.forward(save_checkpoints=True)
        plan.adjoint(res_k, g2)
        assert rel(g2.cpu(), g.cpu()) < 1e-12


def _fd_problem(mods, n_shots):
    """80^2 ellipse medium, blurred start. The ring sits ~10 cells inside the Mur
    edges: the reference's adjoint reuses the forward Mur update, which is not its
    transpose, and with the ring 4 cells from the edge its own float64 gradient
    misses central differences by up to ~1e-3."""
    tb, fwi = mods
    from soundwavesimulation_gb300 import RingArray, axis_centers, interior_mask, m_from_c, stable_dt, ricker
    from soundwavesimulation_gb300.phantoms import blurred_start, random_ellipses
    n, dx, nt = 80, 0.64e-3, 240
    c_true, _ = random_ellipses(n, dx, 6, seed=9)
    dt = stable_dt(2000.0, dx, dx, cfl=0.3)
    x = axis_centers(n, dx)
    ring = RingArray(n_shots, 0.38 * n * dx, x, x)
    wav = ricker(2.0e5, dt, nt)
    mask = interior_mask(x, x, 0.38 * n * dx, margin_m=3 * dx)
    model = tb.TorchScalarWave2D(c_true, dx, device="cuda")
    solver = tb.TorchFDTD2D(model, dt)
    sampler = tb.TorchRingSampler(ring, device="cuda")
    observed, _ = tb.simulate_shots_batch(solver, sampler, wav, ring.rows, ring.cols, nt)
    problem = fwi.TorchLeastSquaresFWI(solver, sampler, ring, wav, nt, n_shots, observed.clone(), mask,
                                       parallel_shots=n_shots)
    m0 = problem.project(m_from_c(blurred_start(c_true, 1.5, mask)))
    return problem, m0, mask, ring, wav, observed.cpu().numpy().astype(np.float64), dx, dt, nt


def test_gradient_matches_float64_finite_differences(mods):
    """Central differences (eps = 1e-3 relative) of the float64 objective along 5 random
    directions against g . dm from the engine (config-3 style, small)."""
    problem, m0, mask, ring, wav, observed, dx, dt, nt = _fd_problem(mods, 8)
    _, g = problem.misfit_and_grad(m0)
    n = m0.shape[0]
    x = problem.array._x_axis
    geo = orc.ring_geometry(8, ring.radius_m, x, x)
    src = orc.point_sources((n, n), ring.rows, ring.cols)

    def J64(m):
        m = problem.project(m)
        tr, _, _, _ = orc.simulate_shots_batch(1.0 / np.sqrt(m), dx, dx, dt, geo, src, wav, nt)
        r = orc.residual_batch(tr, observed, np.arange(8))
        return 0.5 * float(np.sum(r * r))

    rng = np.random.default_rng(4)
    errors = []
    for _ in range(5):
        dm = np.where(mask, rng.standard_normal((n, n)), 0.0)
        dm *= np.linalg.norm(m0[mask]) / np.linalg.norm(dm[mask])
        eps = 1e-3
        fd = (J64(m0 + eps * dm) - J64(m0 - eps * dm)) / (2 * eps)
        directional = float(np.sum(g * dm))
        errors.append(abs(fd - directional) / abs(directional))
    assert max(errors) < 1e-3, errors


def test_gradient_finite_difference_all_gpu(mods):
    """The same check with the float32 engine on both sides: FP32 noise in J limits it to ~1e-2."""
    problem, m0, mask, *_ = _fd_problem(mods, 24)
    _, g = problem.misfit_and_grad(m0)
    rng = np.random.default_rng(5)
    errors = []
    for _ in range(5):
        # random directions with a share of the gradient, so g . dm is never near zero
        r = np.where(mask, rng.standard_normal(m0.shape), 0.0)
        dm = r / np.linalg.norm(r) + g / np.linalg.norm(g)
        dm *= np.linalg.norm(m0[mask]) / np.linalg.norm(dm[mask])
        eps = 1e-2
        fd = (problem.misfit(m0 + eps * dm) - problem.misfit(m0 - eps * dm)) / (2 * eps)
        errors.append(abs(fd - float(np.sum(g * dm))) / abs(float(np.sum(g * dm))))
    assert max(errors) < 5e-2, errors


def test_autograd_function_matches_misfit_and_grad(mods, golden):
    tb, fwi = mods
    d, problem = ring41_problem(mods, golden, parallel_shots=6)
    _, g_c2_ref = problem.gradient_c2(d["m0"], np.arange(6))
    m = torch.tensor(d["m0"], dtype=torch.float64, device="cuda", requires_grad=True)
    rows, cols = problem.array.rows, problem.array.cols
    traces = fwi.simulate_traces(m, problem.solver, problem.sampler, rows, cols,
                                 problem.source_values, problem.n_steps)
    observed = problem.observed
    r = traces - observed
    mute = torch.ones_like(r)
    mute[torch.arange(6), torch.arange(6)] = 0.0
    loss = 0.5 * torch.sum((r * mute).double() ** 2)
    loss.backward()
    g_expected = -g_c2_ref / d["m0"] ** 2
    assert rel(m.grad.cpu().numpy(), g_expected) < 1e-6
