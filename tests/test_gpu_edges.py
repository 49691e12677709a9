"""Sources and receivers in the lanes holding the Mur edges.

Injection nodes (sources; in the adjoint, receiver taps) on and beside column
0, column nx-1 and the edge rows, for the three positions of column nx-1 inside
a lane's 4-column group that select the kernel's compact or general edge path.
Both must equal the plain per-step engine: the forward bit for bit, the
gradient to the float64 summation order.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import engine
    return engine


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _edge_problem(ny, nx, nt, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(1450.0, 1650.0, size=(ny, nx))
    dx = 0.5e-3
    dt = 0.3 * dx / 1650.0
    # shots: source beside the left edge, beside the right edge, on the right
    # edge column itself, and one inside
    srow = np.array([[ny // 2], [ny // 3], [2 * ny // 3], [ny // 2]])
    scol = np.array([[1], [nx - 2], [nx - 1], [nx // 2]])
    sw = np.ones(srow.shape)
    wave = np.zeros(srow.shape, dtype=np.int64)
    # receivers on and beside every edge plus a few inside (taps reach row0 + 1, col0 + 1)
    row0 = np.array([0, 1, ny // 2, ny // 3, ny - 2, ny - 3, 5, ny // 2, ny // 4, 3 * ny // 4])
    col0 = np.array([3, nx // 2, 0, 1, nx // 3, nx - 2, nx - 3, nx - 2, nx // 2, 2])
    wxy = rng.uniform(0.0, 1.0, size=(row0.size, 2))
    w = np.stack([(1 - wxy[:, 0]) * (1 - wxy[:, 1]), wxy[:, 0] * (1 - wxy[:, 1]),
                  (1 - wxy[:, 0]) * wxy[:, 1], wxy[:, 0] * wxy[:, 1]], 1)
    t = np.arange(nt) * dt
    waves = (np.sin(2.5e5 * t) * np.exp(-((t - 2.5e-5) / 8e-6) ** 2))[None]
    return c, dx, dt, (row0, col0, w), (srow, scol, sw, wave), waves


@pytest.mark.parametrize("ny,nx,tuning", [
    (150, 200, {"steps_per_launch": 9}),                                     # nx % 4 == 0
    (133, 203, {"steps_per_launch": 8, "rows_per_lane": 4, "warps": 16}),   # nx % 4 == 3
    (140, 261, {"steps_per_launch": 7, "rows_per_lane": 8, "warps": 12}),   # column nx-1 at c = 0
])
def test_edge_lane_injection_forward_and_gradient(eng, ny, nx, tuning):
    nt = 120
    c, dx, dt, rx, src, waves = _edge_problem(ny, nx, nt, seed=ny + nx)
    w = torch.as_tensor(waves, dtype=torch.float32, device="cuda")
    true = eng.DeviceMedium(c, dx, dx, dt, "cuda")
    plan = eng.FusedPlan(true, rx, src, w, nt, tuning=tuning)
    fused = plan.forward().clone()
    plain = eng.forward_plain(eng.ProblemTables(true, rx, src, w, nt))
    assert torch.equal(fused, plain)

    start = eng.DeviceMedium(np.full_like(c, 1550.0), dx, dx, dt, "cuda")
    gplan = eng.FusedPlan(start, rx, src, w, nt, for_gradient=True, tuning=tuning)
    traces = gplan.forward(save_checkpoints=True)
    res, J = eng.residual_misfit(traces, fused, None)
    g = torch.zeros((ny, start.pitch), dtype=torch.float64, device="cuda")
    gplan.adjoint(res, g)
    Jp, gp = eng.gradient_plain(eng.ProblemTables(start, rx, src, w, nt), fused, None)
    assert float(J) == pytest.approx(float(Jp), rel=1e-6)
    assert rel(g.cpu(), gp.cpu()) < 1e-6
