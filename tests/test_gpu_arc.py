"""GPU parity of the arc geometry paths against the reference's own outputs
(tests/golden/arcs.npz, written by tests/golden/make_golden.py):

* ``ArcLeastSquaresFWI`` (invert_arc.py:294-307): separate transmit / receive arcs,
  no muting; misfit rel 1e-5 and gradient rel-L2 1e-3 against the reference's
  float64 run (the ring tolerances);
* the observed-data precompute (invert_arc.py:317-337, invert_ring.py:1136-1160);
* the focused multi-element firing of 2DArcFDTD.py:203-228 (traces rel 1e-5).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import fwi, torch_backend, traces
    return torch_backend, fwi, traces


def _arc_setup(tb, d, prefix, n_tx, n_rx, c_key, dx_key, dt_key):
    from soundwavesimulation_gb300 import ArcArray, axis_centers
    c = d[c_key]
    n, dx = c.shape[0], float(d[dx_key])
    x = axis_centers(n, dx)
    radius = float(d[f"{prefix}radius"])
    tx = ArcArray(n_tx, radius, 60.0, float(d[f"{prefix}tx_center"]), x, x)
    rx = ArcArray(n_rx, radius, 60.0, float(d[f"{prefix}rx_center"]), x, x)
    np.testing.assert_array_equal(tx.rows, d[f"{prefix}tx_rows"])
    np.testing.assert_array_equal(rx.rows, d[f"{prefix}rx_rows"])
    model = tb.TorchScalarWave2D(c, dx, device="cuda")
    solver = tb.TorchFDTD2D(model, float(d[dt_key]))
    sampler = tb.TorchRingSampler(rx, device="cuda")
    return solver, sampler, tx, rx


def test_arc_fwi_gradient_matches_reference(mods, golden):
    tb, fwi, _ = mods
    d = golden("arcs")
    solver, sampler, tx, _ = _arc_setup(tb, d, "", 3, 5, "c", "dx", "dt")
    nt = int(d["n_steps"])
    problem = fwi.ArcLeastSquaresFWI(solver, sampler, tx, torch.as_tensor(d["pulse"]), nt, 3,
                                     torch.as_tensor(d["observed"]), d["mask"], c_min=1400.0, c_max=2000.0,
                                     c_background=1500.0)
    J, g = problem.misfit_and_grad(d["m0"])
    assert J == pytest.approx(float(d["value"]), rel=1e-5)
    assert rel(g, d["gradient"]) < 1e-3


def test_precompute_observed_matches_reference(mods, golden):
    tb, _, traces = mods
    d = golden("arcs")
    solver, sampler, tx, _ = _arc_setup(tb, d, "", 3, 5, "c", "dx", "dt")
    observed = traces.precompute_observed(solver, sampler, tx, torch.as_tensor(d["pulse"]), int(d["n_steps"]),
                                          parallel_shots=2)
    assert tuple(observed.shape) == d["observed"].shape
    assert rel(observed.cpu().numpy(), d["observed"]) < 1e-5


def test_focused_arc_firing_matches_reference(mods, golden):
    tb, _, _ = mods
    d = golden("arcs")
    solver, sampler, tx, _ = _arc_setup(tb, d, "focus_", 8, 6, "focus_c", "focus_dx", "focus_dt")
    out, _ = tb.simulate_sources(solver, sampler, tx.rows, tx.cols, d["focus_values"], int(d["focus_nt"]))
    assert rel(out.cpu().numpy(), d["focus_traces"]) < 1e-5


def test_resize_slowness_matches_reference(mods, golden):
    """Stage transfer of the multiscale driver (invert_ring.py:1048-1068) on the GPU."""
    from soundwavesimulation_gb300.multiscale import resize_slowness
    d = golden("multiscale")
    out = resize_slowness(d["m"], (d["sx"], d["sy"]), (d["tx"], d["ty"]), float(d["background"]))
    np.testing.assert_allclose(out, d["resized"], rtol=1e-13, atol=0.0)
    dev = resize_slowness(torch.as_tensor(d["m"], device="cuda"), (d["sx"], d["sy"]), (d["tx"], d["ty"]),
                          float(d["background"]))
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), out)
