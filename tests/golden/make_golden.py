"""Generate the golden fixtures in this folder by running the reference itself.

Run in a container that has a checkout of the reference
(scjoshi/SoundWaveSimulation), giving its path as an argument or in the
``SWS_REFERENCE`` environment variable:

    python tests/golden/make_golden.py --reference PATH [--cases engine,optim]

``engine`` writes the engine fixtures (cases A-G below); ``optim`` writes
``optim.npz``: the reference's Tikhonov and total-variation regularisers
(fdtd2d/inversion/misfit.py:19-71) on a seeded model, and its projected Adam
(invert_ring.py:817-861) for one to three iterations on a fixed quadratic
objective.

The reference is imported read-only. Its drivers import matplotlib at module top
level (invert_ring.py:15), which is absent here, so a stub package that only
satisfies those imports is created in a temporary folder first; no plotting
code runs. Every case runs the reference's own torch engine on the CPU in
float64 (and float32 where named), then saves inputs and outputs as ``.npz``.
``torch.as_tensor`` shares memory with a float64 NumPy array, so every
medium handed to the reference is a copy (its ``set_c`` writes in place). The
fixtures are small (a few hundred KB in total) and are what the oracle is
pinned against (``tests/test_oracle_golden.py``); the GPU machine never runs this.
"""

from __future__ import annotations

import argparse
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def _install_matplotlib_stub() -> None:
    root = Path(tempfile.mkdtemp(prefix="mplstub_"))
    pkg = root / "matplotlib"
    pkg.mkdir()
    (pkg / "__init__.py").write_text("def use(*a, **k):\n    pass\n")
    for name in ("pyplot", "animation", "patches", "colors", "gridspec", "cm"):
        (pkg / f"{name}.py").write_text(
            "def __getattr__(name):\n"
            "    def _stub(*a, **k):\n"
            "        raise RuntimeError('plotting is not available')\n"
            "    return _stub\n"
        )
    sys.path.insert(0, str(root))


def ricker(f0, dt, n, t0=None):
    """Ricker wavelet sampled at ``k * dt`` with delay ``t0`` (default 1.5 / f0)."""
    t0 = 1.5 / f0 if t0 is None else t0
    a = (np.pi * f0 * (np.arange(n) * dt - t0)) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def ellipse_medium(n, dx, n_ellipses, seed, c0=1500.0, c_lo=1430.0, c_hi=1620.0):
    """Water plus seeded random ellipses (mask convention of fdtd2d/phantoms.py:27-35)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) - 0.5 * (n - 1)) * dx
    xx, yy = np.meshgrid(x, x, indexing="xy")
    L = n * dx
    c = np.full((n, n), c0)
    for _ in range(n_ellipses):
        x0, y0 = rng.uniform(-0.25 * L, 0.25 * L, size=2)
        a, b = rng.uniform(0.04 * L, 0.12 * L, size=2)
        phi = np.deg2rad(rng.uniform(0.0, 180.0))
        dxp, dyp = xx - x0, yy - y0
        xr = dxp * np.cos(phi) + dyp * np.sin(phi)
        yr = -dxp * np.sin(phi) + dyp * np.cos(phi)
        c[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] = rng.uniform(c_lo, c_hi)
    return c


def optimizer_cases() -> None:
    """optim.npz: the reference's regularisers and projected Adam on seeded inputs."""
    from fdtd2d.inversion import interior_mask, m_from_c
    from fdtd2d.inversion.misfit import tikhonov, total_variation
    from invert_ring import adam

    rng = np.random.default_rng(17)
    n, sp = 37, 1.5e-3
    x = (np.arange(n) - 0.5 * (n - 1)) * sp
    mask = interior_mask(x, x, 0.024, margin_m=sp)
    c = np.full((n, n), 1500.0)
    c[mask] = 1500.0 + 60.0 * rng.standard_normal(int(mask.sum()))
    m = m_from_c(c)
    alpha, tv, tv_eps = 3.0e10, 2.0e4, 1.0e-9
    tik_value, tik_grad = tikhonov(m.copy(), mask, alpha)
    tv_value, tv_grad = total_variation(m.copy(), mask, tv, tv_eps)
    # projected Adam on J(m) = 0.5 * sum(w * (m - target)^2) over the mask
    c_min, c_max, c_bg = 1400.0, 1700.0, 1500.0
    target = m_from_c(np.where(mask, 1500.0 + 80.0 * rng.standard_normal((n, n)), c_bg))
    weight = 1.0 + rng.random((n, n))

    def project(mm):
        out = np.clip(mm, 1.0 / c_max ** 2, 1.0 / c_min ** 2)
        out[~mask] = 1.0 / c_bg ** 2
        return out

    def misfit_and_grad(mm):
        r = np.where(mask, mm - target, 0.0)
        return 0.5 * float(np.sum(weight * r * r)), weight * r

    lr = 2.0e-9
    iterates = []
    for k in (1, 2, 3):
        m_k, _ = adam(m.copy(), misfit_and_grad, project, mask, lr, max_iter=k, verbose=False)
        iterates.append(m_k)
    np.savez_compressed(
        OUT / "optim.npz", m=m, mask=mask, alpha=alpha, tv=tv, tv_eps=tv_eps,
        tikhonov_value=tik_value, tikhonov_grad=tik_grad, tv_value=tv_value, tv_grad=tv_grad,
        adam_target=target, adam_weight=weight, adam_lr=lr, adam_c_min=c_min, adam_c_max=c_max,
        adam_c_background=c_bg, adam_iterates=np.stack(iterates),
    )


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SWS_REFERENCE"),
                    help="path of the reference checkout (default: $SWS_REFERENCE)")
    ap.add_argument("--cases", default="engine,optim")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give the reference checkout with --reference or SWS_REFERENCE")
    _install_matplotlib_stub()
    sys.path.insert(0, str(Path(args.reference).resolve()))
    cases = set(args.cases.split(","))
    if "optim" in cases:
        optimizer_cases()
    if "engine" in cases:
        engine_cases(Path(args.reference).resolve())
    for p in sorted(OUT.glob("*.npz")):
        print(f"{p.name}: {p.stat().st_size / 1024:.1f} KB")


def engine_cases(reference: Path) -> None:
    import torch
    from fdtd2d import ArcArray, RingArray, axis_centers, n_steps_for_crossing, stable_dt
    from fdtd2d.inversion import interior_mask, m_from_c, c_from_m
    from fdtd2d.torch_backend import (
        TorchFDTD2D, TorchFDTD2DBatch, TorchRingSampler, TorchScalarWave2D,
        linear_chirp, simulate_shot, simulate_shots_batch,
    )
    from invert_ring import TorchLeastSquaresFWI, forward_store_batch

    f64 = torch.float64
    geo_keys = ("rows", "cols", "_row0", "_col0", "_w00", "_w10", "_w01", "_w11")

    def geo_arrays(array, prefix=""):
        return {prefix + k.lstrip("_"): np.asarray(getattr(array, k)) for k in geo_keys}

    # --- A: the reference's own 41 x 41 test problem (tests/test_batching.py:20-48)
    N, SP, RAD = 41, 2.0e-3, 0.030
    x_m = axis_centers(N, SP)
    xx, yy = np.meshgrid(x_m, x_m, indexing="xy")
    c_true = np.full((N, N), 1500.0)
    c_true[xx**2 + yy**2 <= 0.012**2] = 1800.0
    dt = stable_dt(2000.0, SP, SP, cfl=0.45)
    pulse = linear_chirp(dt, 20.0e-6, 1.0e5, 2.5e5, device="cpu", dtype=f64)
    n_steps = max(n_steps_for_crossing(RAD, 1500.0, dt), pulse.numel() + 1)
    solver = TorchFDTD2D(TorchScalarWave2D(c_true.copy(), SP, device="cpu", dtype=f64), dt)
    array = RingArray(6, RAD, x_m, x_m)
    sampler = TorchRingSampler(array, device="cpu", dtype=f64)
    observed = torch.stack([
        simulate_shot(solver, sampler, pulse, *array.inject_rows_cols(tx), n_steps)[0]
        for tx in range(6)
    ])
    batched_traces, batched_u = simulate_shots_batch(
        solver, sampler, pulse, array.rows, array.cols, n_steps)
    mask = interior_mask(x_m, x_m, RAD, margin_m=2 * SP)
    problem = TorchLeastSquaresFWI(
        solver, sampler, array, pulse, n_steps, 6, observed, mask,
        c_min=1400.0, c_max=2000.0, c_background=1500.0, parallel_shots=6)
    rng = np.random.default_rng(0)
    m0 = np.full((N, N), m_from_c(1500.0))
    m0[mask] *= 1.0 + 0.02 * rng.standard_normal(int(mask.sum()))
    m0 = problem.project(m0)
    J, g_m = problem.misfit_and_grad(m0)
    # unmasked g_{c^2} through the same internals, all six shots
    problem.apply_medium(m0)
    batched = TorchFDTD2DBatch(solver, 6)
    sources = np.arange(6)
    pred, wave = forward_store_batch(solver, sampler, array, problem.source_values,
                                     sources, n_steps, batched)
    residual = problem._residual_batch(pred, observed[torch.as_tensor(sources)], sources)
    g_c2 = problem._adjoint_accumulate_batch(
        batched, wave, residual, torch.zeros((N, N), dtype=f64))
    np.savez_compressed(
        OUT / "ring41.npz",
        c_true=c_true, dx=SP, dy=SP, dt=dt, pulse=pulse.numpy(), n_steps=n_steps,
        observed=observed.numpy(), batched_traces=batched_traces.numpy(),
        batched_u=batched_u.numpy(), mask=mask, m0=m0, misfit=J, grad_m=g_m,
        c_m0=c_from_m(m0), g_c2=g_c2.numpy(),
        residual_misfit=0.5 * float(torch.sum(residual.square())),
        **geo_arrays(array),
    )

    # --- B: a reduced ellipse medium in the shape of the benchmark configs
    n, dx = 64, 0.8e-3
    L = n * dx
    c_b = ellipse_medium(n, dx, 6, seed=11)
    xb = axis_centers(n, dx)
    dt_b = stable_dt(float(c_b.max()), dx, dx, cfl=0.3)
    nt_b = 400
    wav = ricker(1.25e5, dt_b, nt_b)
    ring_b = RingArray(16, 0.45 * L, xb, xb)
    tx_b = np.array([0, 4, 8, 12])
    out_b = {"c": c_b, "dx": dx, "dt": dt_b, "n_steps": nt_b, "wavelet": wav,
             "tx": tx_b, **geo_arrays(ring_b)}
    for dtype, tag in ((f64, "f64"), (torch.float32, "f32")):
        sol = TorchFDTD2D(TorchScalarWave2D(c_b.copy(), dx, device="cpu", dtype=dtype), dt_b)
        smp = TorchRingSampler(ring_b, device="cpu", dtype=dtype)
        wt = torch.as_tensor(wav, dtype=dtype)
        tr, u_last = simulate_shots_batch(
            sol, smp, wt, ring_b.rows[tx_b], ring_b.cols[tx_b], nt_b, source_values=wt)
        out_b[f"traces_{tag}"] = tr.numpy()
        if tag == "f64":
            out_b["u_f64"] = u_last.numpy()
    # gradient at a blurred start model (invert_ring.py:1179-1184 convention)
    from scipy.ndimage import gaussian_filter
    sol = TorchFDTD2D(TorchScalarWave2D(c_b.copy(), dx, device="cpu", dtype=f64), dt_b)
    smp = TorchRingSampler(ring_b, device="cpu", dtype=f64)
    wt = torch.as_tensor(wav, dtype=f64)
    obs_all = torch.stack([
        simulate_shot(sol, smp, wt, *ring_b.inject_rows_cols(tx), nt_b)[0]
        for tx in range(16)
    ])
    mask_b = interior_mask(xb, xb, 0.45 * L, margin_m=2 * dx)
    prob_b = TorchLeastSquaresFWI(
        sol, smp, ring_b, wt, nt_b, 16, obs_all, mask_b,
        c_min=1400.0, c_max=2000.0, c_background=1500.0, parallel_shots=16)
    m_start = gaussian_filter(m_from_c(c_b), 1.25, mode="nearest")
    m_start[~mask_b] = m_from_c(1500.0)
    m_start = prob_b.project(m_start)
    J_b, g_b = prob_b.misfit_and_grad(m_start)
    prob_b.apply_medium(m_start)
    bat = TorchFDTD2DBatch(sol, len(tx_b))
    pred, wave = forward_store_batch(sol, smp, ring_b, prob_b.source_values, tx_b, nt_b, bat)
    res = prob_b._residual_batch(pred, obs_all[torch.as_tensor(tx_b)], tx_b)
    g_c2_b = prob_b._adjoint_accumulate_batch(bat, wave, res, torch.zeros((n, n), dtype=f64))
    out_b.update(
        mask=mask_b, m_start=m_start,
        c_start=c_from_m(m_start), misfit_all=J_b, grad_m_all=g_b,
        misfit_tx=0.5 * float(torch.sum(res.square())), g_c2_tx=g_c2_b.numpy(),
    )
    # --- C: bilinear (4-node) source, dense-field mode (desmond/src/phase2_numerics.py:107-118)
    tx = 3
    colf = (ring_b.x[tx] - xb[0]) / dx
    rowf = (ring_b.y[tx] - xb[0]) / dx
    c0i, r0i = int(np.floor(colf)), int(np.floor(rowf))
    wx, wy = colf - c0i, rowf - r0i
    field = torch.zeros((n, n), dtype=f64)
    for dr, dc, w in ((0, 0, (1 - wx) * (1 - wy)), (0, 1, wx * (1 - wy)),
                      (1, 0, (1 - wx) * wy), (1, 1, wx * wy)):
        field[r0i + dr, c0i + dc] = w
    sol.set_c(c_b)
    sol.reset()
    zero = torch.zeros((), dtype=f64)
    tr_bil = torch.empty((16, nt_b), dtype=f64)
    for k in range(nt_b):
        u = sol._step(zero, field * wt[k], 2)
        tr_bil[:, k] = smp.record(u)
    out_b.update(bilinear_tx=tx, bilinear_traces=tr_bil.numpy())
    np.savez_compressed(OUT / "ellipses64.npz", **out_b)

    # --- D: single step-level calls on a non-square grid with dx != dy
    ny, nx, dxd, dyd = 24, 20, 1.0e-3, 1.25e-3
    rng = np.random.default_rng(5)
    c_d = rng.uniform(1400.0, 2000.0, size=(ny, nx))
    dt_d = stable_dt(2000.0, dxd, dyd, cfl=0.4)
    xd = axis_centers(nx, dxd)
    yd = axis_centers(ny, dyd)
    ring_d = RingArray(5, 0.0085, xd, yd)
    sol_d = TorchFDTD2D(TorchScalarWave2D(c_d.copy(), dxd, dyd, device="cpu", dtype=f64), dt_d)
    smp_d = TorchRingSampler(ring_d, device="cpu", dtype=f64)
    bat_d = TorchFDTD2DBatch(sol_d, 2)
    u_old0 = rng.standard_normal((2, ny, nx))
    u0 = rng.standard_normal((2, ny, nx))
    fwd_field = rng.standard_normal((2, ny, nx))
    resid = rng.standard_normal((2, 5))
    g_in = rng.standard_normal((ny, nx))
    src_rows = np.array([3, 17])
    src_cols = np.array([1, 12])
    bat_d.set_sources(src_rows, src_cols)
    bat_d.u_old.copy_(torch.as_tensor(u_old0))
    bat_d.u.copy_(torch.as_tensor(u0))
    fwd_u, fwd_samples = bat_d.step_record(torch.tensor(0.75, dtype=f64), smp_d)
    fwd_u = fwd_u.clone()
    bat_d.u_old.copy_(torch.as_tensor(u_old0))
    bat_d.u.copy_(torch.as_tensor(u0))
    g_out = bat_d.adjoint_step_image(torch.as_tensor(resid), smp_d,
                                     torch.as_tensor(fwd_field), torch.as_tensor(g_in), 0.3)
    adj_u = bat_d.u.clone()
    sol_d.reset()
    sol_d.u_old.copy_(torch.as_tensor(u_old0[0]))
    sol_d.u.copy_(torch.as_tensor(u0[0]))
    single_adj = sol_d.inject_field_and_step(torch.as_tensor(fwd_field[0]), adjoint=True).clone()
    np.savez_compressed(
        OUT / "steps_nonsquare.npz",
        c=c_d, dx=dxd, dy=dyd, dt=dt_d, u_old0=u_old0, u0=u0, fwd_field=fwd_field,
        resid=resid, g_in=g_in, src_rows=src_rows, src_cols=src_cols, src_value=0.75,
        fwd_u=fwd_u.numpy(), fwd_samples=fwd_samples.numpy(), adj_u=adj_u.numpy(),
        g_out=g_out.numpy(), image_scale=0.3, single_adj=single_adj.numpy(),
        **geo_arrays(ring_d),
    )

    # --- E: ring and arc geometry at the benchmark grid sizes
    geo = {}
    for n_cells, h, n_el in ((256, 0.2e-3, 128), (512, 0.1e-3, 256), (1024, 0.05e-3, 512)):
        ax = axis_centers(n_cells, h)
        arr = RingArray(n_el, 0.45 * n_cells * h, ax, ax)
        geo.update(geo_arrays(arr, prefix=f"ring{n_cells}_"))
        geo[f"ring{n_cells}_meta"] = np.array([n_cells, h, n_el, 0.45 * n_cells * h])
    arc = ArcArray(16, 0.030, 120.0, 90.0, x_m, x_m)
    geo.update(geo_arrays(arc, prefix="arc41_"))
    geo["arc41_meta"] = np.array([41, SP, 16, 0.030, 120.0, 90.0])
    np.savez_compressed(OUT / "geometry.npz", **geo)

    # --- F: separate transmit / receive arcs (invert_arc.py, 2DArcFDTD.py) and the
    # trace file of 2DRingFDTD.py. The drivers are scripts; they load by path.
    import importlib.util

    def load_script(name, file):
        spec = importlib.util.spec_from_file_location(name, reference / file)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod

    arc_fwi = load_script("ref_invert_arc", "invert_arc.py")
    arc_cli = load_script("ref_arc_cli", "2DArcFDTD.py")
    ring_cli = load_script("ref_ring_cli", "2DRingFDTD.py")
    # F1: the arc gradient problem of run_arc_gradient_check (invert_arc.py:340-372), float64
    src_v = torch.zeros(n_steps, dtype=f64)
    src_v[:pulse.numel()].copy_(pulse)
    solver_f = TorchFDTD2D(TorchScalarWave2D(c_true.copy(), SP, device="cpu", dtype=f64), dt)
    tx_arc = ArcArray(3, RAD, 60.0, arc_fwi.TX_CENTER_DEG, x_m, x_m)
    rx_arc = ArcArray(5, RAD, 60.0, arc_fwi.RX_CENTER_DEG, x_m, x_m)
    sampler_f = TorchRingSampler(rx_arc, device="cpu", dtype=f64)
    observed_f = arc_fwi.simulate_observed(solver_f, sampler_f, tx_arc, pulse, src_v, n_steps,
                                           parallel_shots=3, batched_solvers={})
    mask_f = interior_mask(x_m, x_m, RAD, margin_m=2.0 * SP)
    problem_f = arc_fwi.ArcLeastSquaresFWI(solver_f, sampler_f, tx_arc, pulse, n_steps, 3, observed_f, mask_f,
                                           c_min=1400.0, c_max=2000.0, c_background=1500.0, shot_seed=0)
    rng_f = np.random.default_rng(0)
    m0_f = np.full((N, N), 1.0 / 1500.0 ** 2)
    m0_f[mask_f] *= 1.0 + 0.02 * rng_f.standard_normal(int(mask_f.sum()))
    m0_f = problem_f.project(m0_f)
    value_f, grad_f = problem_f.misfit_and_grad(m0_f.copy())
    # F2: focused firing of an 8-element transmit arc recorded on a 6-element receive arc
    n2, sp2, rad2, nt2 = 64, 1.0e-3, 0.025, 200
    x2 = axis_centers(n2, sp2)
    c2 = np.full((n2, n2), 1500.0)
    c2[np.add.outer(x2 ** 2, x2 ** 2) <= 0.008 ** 2] = 1650.0
    dt2 = stable_dt(1650.0, sp2, sp2, cfl=0.45)
    tx2 = ArcArray(8, rad2, 60.0, arc_cli.TX_CENTER_DEG, x2, x2)
    rx2 = ArcArray(6, rad2, 60.0, arc_cli.RX_CENTER_DEG, x2, x2)
    delays2, _ = arc_cli.focusing_delays(tx2, (0.0, 0.0), 1500.0)
    values2 = arc_cli.delayed_chirps(nt2, dt2, delays2, 40)
    solver2 = TorchFDTD2D(TorchScalarWave2D(c2.copy(), sp2, device="cpu", dtype=f64), dt2)
    sampler2 = TorchRingSampler(rx2, device="cpu", dtype=f64)
    traces2, _ = arc_cli.simulate(solver2, sampler2, tx2, values2, nt2, set())
    np.savez_compressed(
        OUT / "arcs.npz",
        c=c_true, dx=SP, dt=dt, pulse=pulse.numpy(), n_steps=n_steps, radius=RAD,
        tx_center=arc_fwi.TX_CENTER_DEG, rx_center=arc_fwi.RX_CENTER_DEG, observed=observed_f.numpy(),
        mask=mask_f, m0=m0_f, value=value_f, gradient=grad_f,
        focus_c=c2, focus_dx=sp2, focus_dt=dt2, focus_radius=rad2, focus_nt=nt2,
        focus_tx_center=arc_cli.TX_CENTER_DEG, focus_rx_center=arc_cli.RX_CENTER_DEG,
        focus_values=values2, focus_traces=traces2,
        **geo_arrays(tx_arc, prefix="tx_"), **geo_arrays(rx_arc, prefix="rx_"),
        **geo_arrays(tx2, prefix="focus_tx_"), **geo_arrays(rx2, prefix="focus_rx_"),
    )
    # F3: the trace file written by the forward CLI's save_traces (2DRingFDTD.py:291-327)
    ring6 = RingArray(6, RAD, x_m, x_m)
    tr_small = np.random.default_rng(3).standard_normal((6, 9)).astype(np.float32)
    ring_cli.save_traces(OUT / "trace_file.npz", tr_small, np.arange(9) * dt, ring6, 2,
                         np.linspace(0.0, 1.0, 5), dt, c_map=c_true[:4, :4], device="cuda:0",
                         dtype="float32", compiled=True, transmitter_indices=[2, 4])
    # --- G: multiscale stage transfer (invert_ring.py:1037-1068)
    from invert_ring import multiscale_stages, resize_slowness
    rng_g = np.random.default_rng(11)
    sx = axis_centers(41, 2.0e-3)
    tx_g = axis_centers(64, 1.4e-3) + 3.0e-3   # finer grid, shifted field of view
    ty_g = axis_centers(57, 1.6e-3) - 5.0e-3
    xx_g, yy_g = np.meshgrid(sx, sx, indexing="xy")
    m_g = 1.0 / (1500.0 + 80.0 * np.sin(90.0 * xx_g) * np.cos(70.0 * yy_g) + rng_g.normal(0, 2.0, xx_g.shape)) ** 2
    resized = resize_slowness(m_g, (sx, sx), (tx_g, ty_g), 1.0 / 1500.0 ** 2)
    np.savez_compressed(
        OUT / "multiscale.npz", m=m_g, sx=sx, sy=sx, tx=tx_g, ty=ty_g, background=1.0 / 1500.0 ** 2,
        resized=resized, stages_on=np.array(multiscale_stages(True)), stages_off=np.array(multiscale_stages(False)),
    )


if __name__ == "__main__":
    main()
