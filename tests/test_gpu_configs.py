"""The benchmark configurations other than the bench line, at their full grid sizes
and step counts (shot counts cut where a property does not depend on them):

* configuration 1 (256^2, one shot, 2000 steps): fused traces vs the float64 oracle
  (rel-L2 1e-5);
* configuration 4 (256^2 / 384^2 / 512^2 at 96 / 96 / 64 shots and 2000 / 3000 / 4000
  steps): the three grids in shared launches equal each grid run alone (traces
  bitwise, gradients to float64 summation order);
* configuration 5 (1024^2, 6000 steps, 8 of the 256 shots): the gradient with
  float16 checkpoints within 1e-3 of float32 checkpoints, and the float32
  checkpointed gradient equal to the plain full-history form of one shot (1e-6).

Every configuration's error against float64 at full size is in
tests/test_zy_fullsize_fp64.py.
"""

import numpy as np
import pytest
import torch

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
    from soundwavesimulation_gb300 import engine, phantoms
    return engine, phantoms


def _plan(engine, acq, medium, n_shots=None, n_steps=None, **kw):
    sub = acq.subset(n_shots=n_shots, n_steps=n_steps) if (n_shots or n_steps) else acq
    waves = torch.as_tensor(sub.wavelet[None], dtype=torch.float32, device="cuda")
    return engine.FusedPlan(medium, sub.ring.receiver_taps(), sub.source_tables(), waves, sub.n_steps, **kw)


def test_config1_traces_vs_float64_oracle(eng):
    engine, phantoms = eng
    acq = phantoms.config(1)[0]
    medium = engine.DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, "cuda")
    traces = _plan(engine, acq, medium).forward().cpu().numpy()
    rows, cols, w, _ = acq.source_tables()
    geo = orc.ring_geometry(acq.n_elements, 0.45 * acq.n * acq.dx, acq.x, acq.x)
    ref, _, _, _ = orc.simulate_shots_batch(acq.c, acq.dx, acq.dx, acq.dt, geo,
                                            orc.point_sources(acq.c.shape, rows, cols, w), acq.wavelet,
                                            acq.n_steps)
    assert rel(traces, ref) < 1e-5


def test_config4_uneven_batch_in_shared_launches(eng):
    engine, phantoms = eng
    tuning = {"rows_per_lane": 8, "warps": 16, "steps_per_launch": 15}
    acqs = phantoms.config(4)
    media = [engine.DeviceMedium(a.c, a.dx, a.dx, a.dt, "cuda") for a in acqs]
    plans = [_plan(engine, a, m, tuning=tuning, for_gradient=True) for a, m in zip(acqs, media)]
    group = engine.PlanGroup(plans)
    traces = group.forward(save_checkpoints=True)
    residuals = [engine.residual_misfit(t, torch.zeros_like(t), None)[0] for t in traces]
    grads = [torch.zeros((m.ny, m.pitch), dtype=torch.float64, device="cuda") for m in media]
    group.adjoint(residuals, grads)
    for a, m, tr, g in zip(acqs, media, traces, grads):
        plan = _plan(engine, a, m, tuning=tuning, for_gradient=True)
        ref = plan.forward(save_checkpoints=True)
        assert torch.equal(ref, tr), a.name
        g_ref = torch.zeros_like(g)
        plan.adjoint(engine.residual_misfit(ref, torch.zeros_like(ref), None)[0], g_ref)
        assert rel(g.cpu().numpy(), g_ref.cpu().numpy()) < 1e-12, a.name
        del plan, ref, g_ref
    torch.cuda.empty_cache()


def test_config5_checkpoint_precision_and_plain_form(eng):
    engine, phantoms = eng
    acq = phantoms.config(5)[0]
    medium = engine.DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, "cuda")
    S = 8
    sub = acq.subset(n_shots=S)
    observed = _plan(engine, acq, medium, n_shots=S).forward()
    start = engine.DeviceMedium(np.where(acq.c > 1500.0, 0.5 * (acq.c + 1500.0), acq.c), acq.dx, acq.dx,
                                acq.dt, "cuda")
    grads = {}
    for store in (0, 1):  # float32, float16 checkpoints
        plan = _plan(engine, acq, start, n_shots=S, tuning={"ckpt_store": store}, for_gradient=True)
        tr = plan.forward(save_checkpoints=True)
        res, _ = engine.residual_misfit(tr, observed, torch.as_tensor(sub.tx, dtype=torch.int32, device="cuda"))
        g = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device="cuda")
        plan.adjoint(res, g)
        grads[store] = g.cpu().numpy()
        del plan, tr, res
        torch.cuda.empty_cache()
    # float16 (11-bit significand) meets the 1e-3 gradient budget at this size
    assert rel(grads[1], grads[0]) < 1e-3, rel(grads[1], grads[0])
    # one shot: checkpointed float32 gradient vs the plain full-history per-step form
    one = acq.subset(n_shots=1)
    waves = torch.as_tensor(one.wavelet[None], dtype=torch.float32, device="cuda")
    tables = engine.ProblemTables(start, one.ring.receiver_taps(), one.source_tables(), waves, one.n_steps)
    mute = torch.as_tensor(one.tx, dtype=torch.int32, device="cuda")
    _, gp = engine.gradient_plain(tables, observed[:1].contiguous(), mute)
    plan = _plan(engine, acq, start, n_shots=1, for_gradient=True)
    tr = plan.forward(save_checkpoints=True)
    res, _ = engine.residual_misfit(tr, observed[:1].contiguous(), mute)
    g1 = torch.zeros_like(gp)
    plan.adjoint(res, g1)
    assert rel(g1.cpu().numpy(), gp.cpu().numpy()) < 1e-6
