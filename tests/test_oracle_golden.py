"""Pin the NumPy oracle against outputs of the reference itself.

The fixtures in ``tests/golden`` were produced by running the reference's torch
engine in float64 (``tests/golden/make_golden.py``). Agreement here is at the
level of float64 rounding, so the oracle can stand in for the reference in the
GPU parity tests.
"""

import numpy as np
import pytest

from oracle import fdtd_oracle as orc


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def geo_from(d, prefix=""):
    g = {k: d[prefix + k] for k in ("row0", "col0", "w00", "w10", "w01", "w11")}
    g["row1"] = g["row0"] + 1
    g["col1"] = g["col0"] + 1
    return g


def test_ring41_single_and_batched_traces(golden):
    d = golden("ring41")
    geo = geo_from(d)
    shape = d["c_true"].shape
    src = orc.point_sources(shape, d["rows"], d["cols"])
    nt = int(d["n_steps"])
    traces, _, u, _ = orc.simulate_shots_batch(
        d["c_true"], float(d["dx"]), float(d["dy"]), float(d["dt"]), geo, src,
        np.pad(d["pulse"], (0, nt - d["pulse"].size)), nt)
    assert rel(traces, d["observed"]) < 1e-12
    assert rel(traces, d["batched_traces"]) < 1e-12
    assert rel(u, d["batched_u"]) < 1e-12


def test_ring41_gradient_and_misfit(golden):
    d = golden("ring41")
    geo = geo_from(d)
    shape = d["c_true"].shape
    nt = int(d["n_steps"])
    src = orc.point_sources(shape, d["rows"], d["cols"])
    values = np.pad(d["pulse"], (0, nt - d["pulse"].size))
    misfit, g_c2 = orc.misfit_and_gradient_c2(
        d["c_m0"], float(d["dx"]), float(d["dy"]), float(d["dt"]), geo, src, values, nt,
        d["observed"], np.arange(6))
    assert rel(g_c2, d["g_c2"]) < 1e-10
    assert misfit == pytest.approx(float(d["residual_misfit"]), rel=1e-12)
    assert misfit == pytest.approx(float(d["misfit"]), rel=1e-12)
    g_m = orc.gradient_m(g_c2, d["m0"], d["mask"])
    assert rel(g_m, d["grad_m"]) < 1e-10


def test_ellipse_traces_f64_and_reference_f32_drift(golden):
    d = golden("ellipses64")
    geo = geo_from(d)
    n = d["c"].shape[0]
    tx = d["tx"]
    src = orc.point_sources((n, n), d["rows"][tx], d["cols"][tx])
    nt = int(d["n_steps"])
    traces, _, u, _ = orc.simulate_shots_batch(
        d["c"], float(d["dx"]), float(d["dx"]), float(d["dt"]), geo, src, d["wavelet"], nt)
    assert rel(traces, d["traces_f64"]) < 1e-12
    assert rel(u, d["u_f64"]) < 1e-12
    # the reference's own float32 path sits well inside the 1e-5 trace budget
    assert rel(d["traces_f32"], d["traces_f64"]) < 1e-5


def test_ellipse_gradient(golden):
    d = golden("ellipses64")
    geo = geo_from(d)
    n = d["c"].shape[0]
    tx = d["tx"]
    nt = int(d["n_steps"])
    dx, dt = float(d["dx"]), float(d["dt"])
    src = orc.point_sources((n, n), d["rows"][tx], d["cols"][tx])
    observed, _, _, _ = orc.simulate_shots_batch(d["c"], dx, dx, dt, geo, src, d["wavelet"], nt)
    misfit, g_c2 = orc.misfit_and_gradient_c2(
        d["c_start"], dx, dx, dt, geo, src, d["wavelet"], nt, observed, tx)
    assert rel(g_c2, d["g_c2_tx"]) < 1e-9
    assert misfit == pytest.approx(float(d["misfit_tx"]), rel=1e-10)


def test_bilinear_source(golden):
    d = golden("ellipses64")
    geo = geo_from(d)
    n = d["c"].shape[0]
    tx = int(d["bilinear_tx"])
    full = orc.ring_geometry(16, 0.45 * n * float(d["dx"]), orc.axis_centers(n, float(d["dx"])),
                             orc.axis_centers(n, float(d["dx"])))
    rows, cols, w = orc.bilinear_source_taps(full, tx)
    src = orc.point_sources((n, n), rows[None], cols[None], w[None])
    nt = int(d["n_steps"])
    traces, _, _, _ = orc.simulate_shots_batch(
        d["c"], float(d["dx"]), float(d["dx"]), float(d["dt"]), geo, src, d["wavelet"], nt)
    assert rel(traces[0], d["bilinear_traces"]) < 1e-12


def test_step_level_nonsquare(golden):
    d = golden("steps_nonsquare")
    geo = geo_from(d)
    dx, dy, dt = float(d["dx"]), float(d["dy"]), float(d["dt"])
    c = d["c"]
    k = orc.mur_coefficients(c, dt, dx, dy)
    c2 = c * c
    src = orc.point_sources(c.shape, d["src_rows"], d["src_cols"]) * float(d["src_value"])
    fwd = orc.forward_step(d["u_old0"], d["u0"], c2, dt * dt, dx, dy, k, src)
    assert rel(fwd, d["fwd_u"]) < 1e-13
    assert rel(orc.gather(fwd, geo), d["fwd_samples"]) < 1e-13
    adj = orc.adjoint_step(d["u_old0"], d["u0"], c2, dt * dt, dx, dy, k,
                           orc.scatter(d["resid"], geo, c.shape))
    assert rel(adj, d["adj_u"]) < 1e-13
    g = d["g_in"] + float(d["image_scale"]) * np.sum(adj * orc.laplacian(d["fwd_field"], dx, dy), 0)
    assert rel(g, d["g_out"]) < 1e-13
    single = orc.adjoint_step(d["u_old0"][0], d["u0"][0], c2, dt * dt, dx, dy, k, d["fwd_field"][0])
    assert rel(single, d["single_adj"]) < 1e-13


@pytest.mark.parametrize("n_cells", [256, 512, 1024])
def test_ring_geometry(golden, n_cells):
    d = golden("geometry")
    n, h, n_el, radius = d[f"ring{n_cells}_meta"]
    ax = orc.axis_centers(int(n), h)
    g = orc.ring_geometry(int(n_el), radius, ax, ax)
    for key in ("rows", "cols", "row0", "col0"):
        np.testing.assert_array_equal(g[key], d[f"ring{n_cells}_{key}"])
    for key in ("w00", "w10", "w01", "w11"):
        np.testing.assert_allclose(g[key], d[f"ring{n_cells}_{key}"], rtol=0, atol=1e-14)


def test_arc_geometry(golden):
    d = golden("geometry")
    n, h, n_el, radius, span, center = d["arc41_meta"]
    ax = orc.axis_centers(int(n), h)
    g = orc.arc_geometry(int(n_el), radius, span, center, ax, ax)
    for key in ("rows", "cols", "row0", "col0"):
        np.testing.assert_array_equal(g[key], d[f"arc41_{key}"])
    for key in ("w00", "w10", "w01", "w11"):
        np.testing.assert_allclose(g[key], d[f"arc41_{key}"], rtol=0, atol=1e-14)


def _arc_pair(d, prefix, n_tx, n_rx, n, dx):
    ax = orc.axis_centers(n, dx)
    radius = float(d[f"{prefix}radius"])
    tx = orc.arc_geometry(n_tx, radius, 60.0, float(d[f"{prefix}tx_center"]), ax, ax)
    rx = orc.arc_geometry(n_rx, radius, 60.0, float(d[f"{prefix}rx_center"]), ax, ax)
    for key in ("rows", "cols", "row0", "col0"):
        np.testing.assert_array_equal(tx[key], d[f"{prefix}tx_{key}"])
        np.testing.assert_array_equal(rx[key], d[f"{prefix}rx_{key}"])
    return tx, rx


def test_arc_focused_firing(golden):
    """2DArcFDTD.py:203-228: eight transmit elements fire at once, each with its own
    delayed chirp; the oracle superposes one run per element (linearity)."""
    d = golden("arcs")
    n, dx, nt = d["focus_c"].shape[0], float(d["focus_dx"]), int(d["focus_nt"])
    tx, rx = _arc_pair(d, "focus_", 8, 6, n, dx)
    fields = orc.point_sources((n, n), tx["rows"], tx["cols"])
    traces, _, _, _ = orc.simulate_shots_batch(d["focus_c"], dx, dx, float(d["focus_dt"]), rx, fields,
                                               d["focus_values"], nt)
    assert rel(traces.sum(0), d["focus_traces"]) < 1e-10


def test_arc_gradient_without_muting(golden):
    """ArcLeastSquaresFWI.misfit_and_grad (invert_arc.py:294-307): three transmit
    elements, five receivers on a separate arc, the full residual kept."""
    d = golden("arcs")
    n, dx, nt = d["c"].shape[0], float(d["dx"]), int(d["n_steps"])
    tx, rx = _arc_pair(d, "", 3, 5, n, dx)
    values = np.zeros(nt)
    values[:d["pulse"].size] = d["pulse"]
    src = orc.point_sources((n, n), tx["rows"], tx["cols"])
    m0 = d["m0"]
    J, g_c2 = orc.misfit_and_gradient_c2(1.0 / np.sqrt(m0), dx, dx, float(d["dt"]), rx, src, values, nt,
                                         d["observed"], np.full(3, -1))
    assert J == pytest.approx(float(d["value"]), rel=1e-10)
    assert rel(orc.gradient_m(g_c2, m0, d["mask"]), d["gradient"]) < 1e-9


def test_resize_slowness(golden):
    """invert_ring.py:1048-1068 (torch grid_sample, bicubic, border, corners aligned)."""
    d = golden("multiscale")
    out = orc.resize_slowness(d["m"], (d["sx"], d["sy"]), (d["tx"], d["ty"]), float(d["background"]))
    np.testing.assert_allclose(out, d["resized"], rtol=1e-13, atol=0.0)
    assert (out == float(d["background"])).any() and (out != float(d["background"])).any()


def test_multiscale_stage_ladder(golden):
    from soundwavesimulation_gb300.multiscale import multiscale_stages
    d = golden("multiscale")
    np.testing.assert_array_equal(np.array(multiscale_stages(True)), d["stages_on"])
    np.testing.assert_array_equal(np.array(multiscale_stages(False)), d["stages_off"])


def test_regularisers_and_adam_match_reference(golden):
    """optim.npz holds the reference's tikhonov / total_variation
    (fdtd2d/inversion/misfit.py:19-71) on a seeded model and the iterates of its
    projected adam (invert_ring.py:817-861) on a fixed quadratic objective."""
    g = golden("optim")
    mask = g["mask"]
    v, gr = orc.tikhonov(g["m"], mask, float(g["alpha"]))
    assert v == pytest.approx(float(g["tikhonov_value"]), rel=1e-14)
    np.testing.assert_allclose(gr, g["tikhonov_grad"], rtol=0, atol=1e-14 * np.abs(g["tikhonov_grad"]).max())
    v, gr = orc.total_variation(g["m"], mask, float(g["tv"]), float(g["tv_eps"]))
    assert v == pytest.approx(float(g["tv_value"]), rel=1e-14)
    np.testing.assert_allclose(gr, g["tv_grad"], rtol=0, atol=1e-14 * np.abs(g["tv_grad"]).max())
    lo, hi, bg = 1.0 / float(g["adam_c_max"]) ** 2, 1.0 / float(g["adam_c_min"]) ** 2, 1.0 / float(
        g["adam_c_background"]) ** 2

    def project(mm):
        out = np.clip(mm, lo, hi)
        out[~mask] = bg
        return out

    def objective(mm):
        r = np.where(mask, mm - g["adam_target"], 0.0)
        return 0.5 * float(np.sum(g["adam_weight"] * r * r)), g["adam_weight"] * r

    its = orc.projected_adam(g["m"], objective, project, mask, float(g["adam_lr"]), 3)
    for k, (mine, ref) in enumerate(zip(its, g["adam_iterates"])):
        np.testing.assert_allclose(mine, ref, rtol=1e-14, atol=0, err_msg=f"iteration {k + 1}")


def _c_receivers(d, prefix=""):
    w = np.stack([d[prefix + k] for k in ("w00", "w10", "w01", "w11")], axis=1)
    return d[prefix + "row0"], d[prefix + "col0"], w


def test_c_oracle_matches_reference_ring41(golden):
    """The float64 C oracle (oracle/fdtd_oracle.c) reproduces the reference's
    traces, misfit and g_{c^2} of its own 41^2 problem, at any checkpoint spacing."""
    from oracle import c_oracle
    d = golden("ring41")
    nt = int(d["n_steps"])
    dx, dy, dt = float(d["dx"]), float(d["dy"]), float(d["dt"])
    rows, cols = d["rows"][:, None], d["cols"][:, None]
    src = (rows, cols, np.ones(rows.shape))
    values = np.pad(d["pulse"], (0, nt - d["pulse"].size))
    traces = c_oracle.forward_shots(d["c_true"], dx, dy, dt, src, _c_receivers(d), values, nt)
    assert rel(traces, d["batched_traces"]) < 1e-12
    for ckpt in (None, 5, nt):
        J, g = c_oracle.gradient_shots(d["c_m0"], dx, dy, dt, src, _c_receivers(d), values, nt, d["observed"],
                                       np.arange(6), ckpt_every=ckpt)
        assert J == pytest.approx(float(d["residual_misfit"]), rel=1e-12)
        assert rel(g, d["g_c2"]) < 1e-10


def test_c_oracle_matches_numpy_oracle_bilinear_nonsquare():
    """Non-square grid, dx != dy, 4-node bilinear sources: C and NumPy oracles agree."""
    from oracle import c_oracle
    rng = np.random.default_rng(9)
    ny, nx, dx, dy, nt = 53, 47, 0.6e-3, 0.5e-3, 180
    c = 1500.0 + 120.0 * rng.random((ny, nx))
    dt = orc.stable_dt(c.max(), dx, dy, 0.35)
    geo = orc.ring_geometry(10, 0.011, orc.axis_centers(nx, dx), orc.axis_centers(ny, dy))
    taps = [orc.bilinear_source_taps(geo, t) for t in (0, 3, 7)]
    rows, cols, w = (np.stack([t[i] for t in taps]) for i in range(3))
    wav = np.sin(np.arange(nt) * 0.3) * np.exp(-((np.arange(nt) - 30) / 12.0) ** 2)
    fields = orc.point_sources((ny, nx), rows, cols, w)
    ref, *_ = orc.simulate_shots_batch(c, dx, dy, dt, geo, fields, wav, nt)
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    out = c_oracle.forward_shots(c, dx, dy, dt, (rows, cols, w), rx, wav, nt)
    assert rel(out, ref) < 1e-13
    obs = ref * 0.9 + 0.01 * rng.standard_normal(ref.shape) * np.abs(ref).max()
    J_ref, g_ref = orc.misfit_and_gradient_c2(c * 0.98, dx, dy, dt, geo, fields, wav, nt, obs, np.array([0, 3, -1]))
    J, g = c_oracle.gradient_shots(c * 0.98, dx, dy, dt, (rows, cols, w), rx, wav, nt, obs, np.array([0, 3, -1]),
                                   ckpt_every=13)
    assert J == pytest.approx(J_ref, rel=1e-13)
    assert rel(g, g_ref) < 1e-12
