"""Every benchmark configuration against float64 at its own grid size and step count.

The float64 side is the C oracle (oracle/fdtd_oracle.c, pinned to the reference's
own outputs and to the NumPy oracle in tests/test_oracle_golden.py), run on the
host cores for a subset of each configuration's shots. The GPU side is the
engine at the configuration's full size: grid, step count and launch shape are
the configuration's; only the number of shots compared is cut.

Budgets (the contract): traces rel-L2 <= 1e-5, misfit rel <= 1e-5, gradient
rel-L2 <= 1e-3 on the inversion mask, all against float64. The gradient is also
checked the way the reference checks its own (invert_ring.py:704-779): central
differences of the float64 objective along random in-mask directions scaled to
|m|, eps = 1e-3, against g . d. bfloat16 checkpoints are outside the 1e-3
gradient budget: the engine warns when they are chosen, and the test checks the
warning and that the gradient keeps its direction.

This file sorts after the other GPU tests and before test_zz_no_alloc.py. With
FDTD_PARITY_JSON set, the measured figures are written to that file.
"""

import json
import os
import warnings

import numpy as np
import pytest
import torch

from oracle import c_oracle

pytestmark = pytest.mark.gpu

BENCH_TUNING = {"rows_per_lane": 8, "warps": 16, "steps_per_launch": 15}
TRACE_BUDGET, GRAD_BUDGET = 1e-5, 1e-3
RESULTS = {}


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import engine, phantoms
    c_oracle.build()
    yield engine, phantoms
    path = os.environ.get("FDTD_PARITY_JSON")
    if path:
        with open(path, "w") as f:
            json.dump(RESULTS, f, indent=1, sort_keys=True)


def _sources(acq, shots):
    rows, cols, w, _ = acq.source_tables()
    return rows[shots], cols[shots], w[shots]


def _plan(engine, medium, acq, shots=None, for_gradient=False, tuning=None):
    rows, cols, w, wave = acq.source_tables()
    if shots is not None:
        rows, cols, w, wave = rows[shots], cols[shots], w[shots], wave[shots]
    waves = torch.as_tensor(acq.wavelet[None], dtype=torch.float32, device="cuda")
    return engine.FusedPlan(medium, acq.ring.receiver_taps(), (rows, cols, w, wave), waves, acq.n_steps,
                            tuning=dict(tuning or BENCH_TUNING), for_gradient=for_gradient)


def _mask(acq, margin_cells=3):
    from soundwavesimulation_gb300 import interior_mask
    return interior_mask(acq.x, acq.x, 0.45 * acq.n * acq.dx, margin_m=margin_cells * acq.dx)


def _gpu_gradient(engine, medium, acq, shots, observed, tuning=None):
    """Misfit and g_{c^2} (float64, (ny, nx)) of the fused engine for `shots`."""
    plan = _plan(engine, medium, acq, shots, for_gradient=True, tuning=tuning)
    pred = plan.forward(save_checkpoints=True)
    mute = torch.as_tensor(acq.tx[shots], dtype=torch.int32, device="cuda")
    res, misfit = engine.residual_misfit(pred, observed, mute)
    g = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device="cuda")
    plan.adjoint(res, g)
    torch.cuda.synchronize()
    out = float(misfit.item()), g[:, :medium.nx].cpu().numpy()
    del plan, pred, res, g
    torch.cuda.empty_cache()
    return out


def _fp64_objective(acq, shots, c, observed64):
    traces = c_oracle.forward_shots(c, acq.dx, acq.dx, acq.dt, _sources(acq, shots), acq.ring.receiver_taps(),
                                    acq.wavelet, acq.n_steps)
    return c_oracle.misfit(traces, observed64, acq.tx[shots])


def _directional_checks(acq, shots, m0, mask, observed64, g_m, n_dirs, seed, eps=1e-3):
    """Central differences of the float64 objective along random in-mask
    directions (the recipe of invert_ring.py:704-779) against g_m . d."""
    rng = np.random.default_rng(seed)
    errs = []
    for _ in range(n_dirs):
        d = np.zeros_like(m0)
        d[mask] = rng.standard_normal(int(mask.sum()))
        d *= np.linalg.norm(m0[mask]) / np.linalg.norm(d[mask])
        jp = _fp64_objective(acq, shots, 1.0 / np.sqrt(m0 + eps * d), observed64)
        jm = _fp64_objective(acq, shots, 1.0 / np.sqrt(m0 - eps * d), observed64)
        fd = (jp - jm) / (2.0 * eps)
        directional = float(np.sum(g_m[mask] * d[mask]))
        errs.append(abs(fd - directional) / abs(fd))
    return errs


def test_config2_bench_workload_traces_vs_fp64(eng):
    """The bench workload itself (512^2, 128 shots, 4000 steps, bilinear sources,
    the bench's launch shape): four shots around the ring against float64."""
    engine, phantoms = eng
    acq = phantoms.config(2)[0]
    medium = engine.DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, "cuda")
    traces = _plan(engine, medium, acq).forward().cpu().numpy()
    shots = np.array([0, 37, 74, 111])
    ref = c_oracle.forward_shots(acq.c, acq.dx, acq.dx, acq.dt, _sources(acq, shots), acq.ring.receiver_taps(),
                                 acq.wavelet, acq.n_steps)
    err = rel(traces[shots], ref)
    RESULTS["config2_traces_rel_l2"] = err
    RESULTS["config2_traces_rel_l2_per_shot"] = [rel(traces[s], r) for s, r in zip(shots, ref)]
    assert err <= TRACE_BUDGET, err


def test_config3_gradient_vs_fp64_and_directional_fd(eng):
    """512^2, 4000 steps, blurred (sigma 10 cells) start: the checkpointed float32
    gradient of four of the 64 shots against the float64 adjoint gradient, and
    against central differences of the float64 objective along 5 directions."""
    engine, phantoms = eng
    acq = phantoms.config(3)[0]
    shots = np.array([0, 16, 32, 48])
    mask = _mask(acq)
    truth = engine.DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, "cuda")
    observed = _plan(engine, truth, acq, shots).forward()
    c0 = phantoms.blurred_start(acq.c, 10.0, mask)
    m0 = 1.0 / c0 ** 2
    start = engine.DeviceMedium(c0, acq.dx, acq.dx, acq.dt, "cuda")
    J, g_c2 = _gpu_gradient(engine, start, acq, shots, observed)
    obs64 = observed.cpu().numpy().astype(np.float64)
    J64, g64_c2 = c_oracle.gradient_shots(c0, acq.dx, acq.dx, acq.dt, _sources(acq, shots),
                                          acq.ring.receiver_taps(), acq.wavelet, acq.n_steps, obs64,
                                          acq.tx[shots])
    g_m = np.where(mask, -g_c2 / m0 ** 2, 0.0)
    g64_m = np.where(mask, -g64_c2 / m0 ** 2, 0.0)
    RESULTS["config3_misfit_rel"] = abs(J - J64) / J64
    RESULTS["config3_gradient_rel_l2"] = rel(g_m, g64_m)
    fd = _directional_checks(acq, shots, m0, mask, obs64, g_m, 5, seed=3)
    fd64 = _directional_checks(acq, shots, m0, mask, obs64, g64_m, 2, seed=3)
    RESULTS["config3_directional_fd_rel"] = fd
    RESULTS["config3_directional_fd_rel_fp64_gradient"] = fd64
    assert abs(J - J64) / J64 <= TRACE_BUDGET
    assert rel(g_m, g64_m) <= GRAD_BUDGET, rel(g_m, g64_m)
    assert max(fd) <= GRAD_BUDGET, fd


def test_config4_uneven_batch_vs_fp64(eng):
    """The three grids of the uneven multiscale batch (256^2 / 384^2 / 512^2 at
    2000 / 3000 / 4000 steps) in shared launches: one shot per grid, traces and
    gradient (from a 4-cell blurred start) against float64."""
    engine, phantoms = eng
    acqs = phantoms.config(4)
    trace_errs, grad_errs = {}, {}
    plans, media, observed, starts = [], [], [], []
    for a in acqs:
        truth = engine.DeviceMedium(a.c, a.dx, a.dx, a.dt, "cuda")
        observed.append(_plan(engine, truth, a, np.array([0])).forward())
        c0 = phantoms.blurred_start(a.c, 4.0, _mask(a))
        starts.append(c0)
        media.append(engine.DeviceMedium(c0, a.dx, a.dx, a.dt, "cuda"))
        plans.append(_plan(engine, media[-1], a, np.array([0]), for_gradient=True))
    group = engine.PlanGroup(plans)
    preds = group.forward(save_checkpoints=True)
    residuals = []
    for a, p, o in zip(acqs, preds, observed):
        mute = torch.as_tensor(a.tx[:1], dtype=torch.int32, device="cuda")
        residuals.append(engine.residual_misfit(p.clone(), o, mute)[0])
    grads = [torch.zeros((m.ny, m.pitch), dtype=torch.float64, device="cuda") for m in media]
    group.adjoint(residuals, grads)
    torch.cuda.synchronize()
    for a, c0, p, o, g, m in zip(acqs, starts, preds, observed, grads, media):
        shots = np.array([0])
        ref = c_oracle.forward_shots(c0, a.dx, a.dx, a.dt, _sources(a, shots), a.ring.receiver_taps(), a.wavelet,
                                     a.n_steps)
        trace_errs[a.name] = rel(p.cpu().numpy(), ref)
        _, g64 = c_oracle.gradient_shots(c0, a.dx, a.dx, a.dt, _sources(a, shots), a.ring.receiver_taps(),
                                         a.wavelet, a.n_steps, o.cpu().numpy().astype(np.float64), a.tx[:1])
        mask = _mask(a)
        grad_errs[a.name] = rel(np.where(mask, g.cpu().numpy()[:, :m.nx], 0.0), np.where(mask, g64, 0.0))
    RESULTS["config4_traces_rel_l2"] = trace_errs
    RESULTS["config4_gradient_rel_l2"] = grad_errs
    assert max(trace_errs.values()) <= TRACE_BUDGET, trace_errs
    assert max(grad_errs.values()) <= GRAD_BUDGET, grad_errs


def test_config5_traces_and_checkpoint_precision_vs_fp64(eng):
    """1024^2, 6000 steps: traces of one shot against float64; the gradient of two
    of the 256 shots (20-cell blurred start) with float32, float16 and bfloat16
    checkpoints against the float64 adjoint gradient, float16 also by two
    directional differences of the float64 objective."""
    engine, phantoms = eng
    acq = phantoms.config(5)[0]
    shots = np.array([0, 128])
    mask = _mask(acq)
    truth = engine.DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, "cuda")
    observed = _plan(engine, truth, acq, shots).forward()
    ref = c_oracle.forward_shots(acq.c, acq.dx, acq.dx, acq.dt, _sources(acq, shots[:1]),
                                 acq.ring.receiver_taps(), acq.wavelet, acq.n_steps)
    RESULTS["config5_traces_rel_l2"] = rel(observed[:1].cpu().numpy(), ref)
    del truth
    c0 = phantoms.blurred_start(acq.c, 20.0, mask)
    m0 = 1.0 / c0 ** 2
    start = engine.DeviceMedium(c0, acq.dx, acq.dx, acq.dt, "cuda")
    obs64 = observed.cpu().numpy().astype(np.float64)
    J64, g64_c2 = c_oracle.gradient_shots(c0, acq.dx, acq.dx, acq.dt, _sources(acq, shots),
                                          acq.ring.receiver_taps(), acq.wavelet, acq.n_steps, obs64, acq.tx[shots])
    g64_m = np.where(mask, -g64_c2 / m0 ** 2, 0.0)
    errs, g_ms = {}, {}
    for name, store in (("f32", 0), ("f16", 1), ("bf16", 2)):
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("always")
            J, g_c2 = _gpu_gradient(engine, start, acq, shots, observed, tuning={**BENCH_TUNING, "ckpt_store": store})
        warned = any("bfloat16" in str(w.message) for w in caught)
        assert warned == (name == "bf16"), name
        g_ms[name] = np.where(mask, -g_c2 / m0 ** 2, 0.0)
        errs[name] = rel(g_ms[name], g64_m)
        if name == "f32":
            RESULTS["config5_misfit_rel"] = abs(J - J64) / J64
    RESULTS["config5_gradient_rel_l2"] = errs
    fd = _directional_checks(acq, shots, m0, mask, obs64, g_ms["f16"], 2, seed=5)
    RESULTS["config5_directional_fd_rel_f16"] = fd
    cos = float(np.sum(g_ms["bf16"] * g64_m) / (np.linalg.norm(g_ms["bf16"]) * np.linalg.norm(g64_m)))
    RESULTS["config5_bf16_cosine"] = cos
    assert RESULTS["config5_traces_rel_l2"] <= TRACE_BUDGET
    assert RESULTS["config5_misfit_rel"] <= TRACE_BUDGET
    assert errs["f32"] <= GRAD_BUDGET and errs["f16"] <= GRAD_BUDGET, errs
    assert max(fd) <= GRAD_BUDGET, fd
    assert cos > 0.999, cos
