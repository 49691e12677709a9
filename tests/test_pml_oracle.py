"""The float64 PML restatement (no reference counterpart; the reference has
first-order Mur edges only, fdtd2d/solver.py:90-124), on the CPU.

* the C oracle's PML equals the NumPy restatement (oracle/fdtd_oracle.py pml_step);
* reflections: a water shot with a 20 / 30 / 40-cell PML padded outside the grid
  against the same shot on a grid so large that no boundary echo arrives in the
  window (the PML's trace error is the reflection left), Mur for comparison;
* known answer: the water line-source trace of desmond/src/phase2_numerics.py:
  126-145 (exact 2-D Green's function convolved with the pulse); the PML trace
  departs from it exactly as the unbounded grid does (grid dispersion), Mur adds
  its echoes;
* the PML gradient (the adjoint with the same PML step) against central
  differences of the float64 objective along random in-mask directions.
"""

import numpy as np
import pytest

from oracle import c_oracle
from oracle import fdtd_oracle as orc


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def _water(n=120, dx=0.2e-3, nt=900, f0=0.4e6):
    c = np.full((n, n), 1500.0)
    dt = orc.stable_dt(1500.0, dx, dx, 0.3)
    x = orc.axis_centers(n, dx)
    geo = orc.ring_geometry(32, 0.45 * n * dx, x, x)

    def ricker(tt):
        a = (np.pi * f0 * (tt - 1.5 / f0)) ** 2
        return (1 - 2 * a) * np.exp(-a)

    wav = ricker(np.arange(nt) * dt)
    rows, cols = geo["rows"][[0]][:, None], geo["cols"][[0]][:, None]
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    return c, dx, dt, geo, (rows, cols, np.ones(rows.shape)), rx, wav, nt, ricker


def test_c_pml_equals_numpy_pml():
    rng = np.random.default_rng(1)
    ny, nx, dx, nt = 64, 59, 0.3e-3, 300
    c = 1500 + 80 * rng.random((ny, nx))
    dt = orc.stable_dt(c.max(), dx, dx, 0.3)
    geo = orc.ring_geometry(16, 0.4 * nx * dx, orc.axis_centers(nx, dx), orc.axis_centers(ny, dx))
    wav = np.sin(np.arange(nt) * 0.35) * np.exp(-((np.arange(nt) - 40) / 15.0) ** 2)
    taps = [orc.bilinear_source_taps(geo, t) for t in (0, 5)]
    rows, cols, w = (np.stack([t[i] for t in taps]) for i in range(3))
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    ref, _ = orc.simulate_pml(c, dx, dx, dt, geo, orc.point_sources((ny, nx), rows, cols, w), wav, nt, 12)
    out = c_oracle.forward_shots(c, dx, dx, dt, (rows, cols, w), rx, wav, nt, pml=12)
    assert rel(out, ref) < 1e-13


def test_pml_reflection_against_unbounded_grid_and_line_source():
    c, dx, dt, geo, src, rx, wav, nt, ricker = _water()
    big = 300  # no echo from the padded grid's edges reaches a receiver within nt steps
    rows, cols, w = src
    ref = c_oracle.forward_shots(np.pad(c, big, mode="edge"), dx, dx, dt, (rows + big, cols + big, w),
                                 (rx[0] + big, rx[1] + big, rx[2]), wav, nt)
    mur = c_oracle.forward_shots(c, dx, dx, dt, src, rx, wav, nt)
    errs = {P: rel(c_oracle.forward_shots(c, dx, dx, dt, src, rx, wav, nt, pml=P), ref) for P in (20, 30, 40)}
    assert rel(mur, ref) > 0.1                       # Mur: 14 % of the trace energy is echo
    assert errs[20] < 3e-3 and errs[30] < 1e-3 and errs[40] < 5e-4, errs
    assert errs[40] < errs[30] < errs[20]
    pml = c_oracle.forward_shots(c, dx, dx, dt, src, rx, wav, nt, pml=30)
    xs, ys = orc.axis_centers(120, dx)[geo["cols"][0]], orc.axis_centers(120, dx)[geo["rows"][0]]
    t = (np.arange(nt) + 1) * dt  # trace column n holds u at (n + 1) dt
    for j in (8, 16, 24):
        r = np.hypot(geo["x"][j] - xs, geo["y"][j] - ys)
        exact = orc.analytic_line_source(r, t, dx, dt, ricker)
        # the boundary adds nothing to the grid's own dispersion error with the PML
        assert abs(rel(pml[0, j], exact) - rel(ref[0, j], exact)) < 1e-3
        assert rel(mur[0, j], exact) > rel(ref[0, j], exact) + 0.05


def test_pml_gradient_against_central_differences():
    rng = np.random.default_rng(1)
    ny, nx, dx, nt, P = 64, 59, 0.3e-3, 400, 12
    c = 1500 + 80 * rng.random((ny, nx))
    dt = orc.stable_dt(c.max(), dx, dx, 0.3)
    x, y = orc.axis_centers(nx, dx), orc.axis_centers(ny, dx)
    geo = orc.ring_geometry(16, 0.4 * nx * dx, x, y)
    wav = np.sin(np.arange(nt) * 0.35) * np.exp(-((np.arange(nt) - 40) / 15.0) ** 2)
    tx = np.array([0, 5])
    taps = [orc.bilinear_source_taps(geo, t) for t in tx]
    src = tuple(np.stack([t[i] for t in taps]) for i in range(3))
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    c_true = c.copy()
    c_true[20:35, 20:30] += 60
    obs = c_oracle.forward_shots(c_true, dx, dx, dt, src, rx, wav, nt, pml=P)
    _, g = c_oracle.gradient_shots(c, dx, dx, dt, src, rx, wav, nt, obs, tx, ckpt_every=37, pml=P)
    m0 = 1 / c ** 2
    gm = -g / m0 ** 2
    mask = orc.interior_mask(x, y, 0.4 * nx * dx, 2 * dx)

    def J(mm):
        return c_oracle.misfit(c_oracle.forward_shots(1 / np.sqrt(mm), dx, dx, dt, src, rx, wav, nt, pml=P), obs, tx)

    for seed in range(3):
        r = np.random.default_rng(seed)
        d = np.where(mask, r.standard_normal(m0.shape), 0.0)
        d *= np.linalg.norm(m0[mask]) / np.linalg.norm(d[mask])
        fd = (J(m0 + 1e-3 * d) - J(m0 - 1e-3 * d)) / 2e-3
        assert abs(fd - np.sum(gm[mask] * d[mask])) / abs(fd) < 1e-3
