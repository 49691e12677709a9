"""NumPy restatement of the reference fdtd2d engine: TEST INFRASTRUCTURE ONLY.

This module is the oracle that the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use to check the CUDA engine in
``soundwavesimulation_gb300``. The product never imports, links or runs it.

Every function restates one piece of the reference (scjoshi/SoundWaveSimulation)
and cites the file:line it follows. Arithmetic runs in the dtype of the inputs
(float64 by default), vectorised over a leading shot axis where the reference
batches shots. Parity of this restatement with the reference itself is pinned by
``tests/golden/*.npz`` (produced by running the reference, see
``tests/golden/make_golden.py``) and checked in ``tests/test_oracle_golden.py``.

Array conventions follow the reference: fields are ``(shots, ny, nx)`` with
row = y and column = x; traces are ``(shots, receivers, steps)``.
"""

from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------------------
# Grid helpers (fdtd2d/experiment.py)
# ---------------------------------------------------------------------------

def axis_centers(n, spacing):
    """Cell-centre axis, origin at the grid centre (fdtd2d/experiment.py:6-8)."""
    return (np.arange(n) - 0.5 * (n - 1)) * spacing


def stable_dt(c_max, dx, dy, cfl=0.45):
    """CFL time step (fdtd2d/experiment.py:11-13)."""
    return cfl / (c_max * np.sqrt(1.0 / dx**2 + 1.0 / dy**2))


def n_steps_for_crossing(radius_m, c_min, dt, extras=1.6):
    """Steps to cross the ring diameter with margin (fdtd2d/experiment.py:16-18)."""
    return int(np.ceil(extras * (2.0 * radius_m / c_min) / dt))


# ---------------------------------------------------------------------------
# Ring geometry (fdtd2d/array.py)
# ---------------------------------------------------------------------------

def ring_geometry(n_elements, radius_m, x_m, y_m, center=(0.0, 0.0)):
    """Element positions, nearest nodes and bilinear taps of a ring.

    Restates RingArray.__init__ / _nearest_indices / _init_bilinear
    (fdtd2d/array.py:14-33 and 60-76). Returns a dict of arrays.
    """
    theta = 2.0 * np.pi * np.arange(n_elements) / n_elements
    x = center[0] + radius_m * np.cos(theta)
    y = center[1] + radius_m * np.sin(theta)
    return _geometry_from_points(x, y, np.asarray(x_m, float), np.asarray(y_m, float))


def arc_geometry(n_elements, radius_m, span_deg, center_deg, x_m, y_m, center=(0.0, 0.0)):
    """Elements equally spaced on an arc (ArcArray.__init__, fdtd2d/array.py:126-150)."""
    half = 0.5 * np.deg2rad(span_deg)
    theta = np.deg2rad(center_deg) + np.linspace(-half, half, n_elements)
    x = center[0] + radius_m * np.cos(theta)
    y = center[1] + radius_m * np.sin(theta)
    return _geometry_from_points(x, y, np.asarray(x_m, float), np.asarray(y_m, float))


def _geometry_from_points(x, y, x_axis, y_axis):
    dx = x_axis[1] - x_axis[0]
    dy = y_axis[1] - y_axis[0]
    cols = np.rint((x - x_axis[0]) / dx).astype(np.int64)  # array.py:28-33
    rows = np.rint((y - y_axis[0]) / dy).astype(np.int64)
    colf = (x - x_axis[0]) / dx  # array.py:60-76
    rowf = (y - y_axis[0]) / dy
    col0 = np.floor(colf).astype(np.int64)
    row0 = np.floor(rowf).astype(np.int64)
    wx = colf - col0
    wy = rowf - row0
    return {
        "x": x, "y": y, "rows": rows, "cols": cols,
        "row0": row0, "col0": col0, "row1": row0 + 1, "col1": col0 + 1,
        "w00": (1.0 - wx) * (1.0 - wy), "w10": wx * (1.0 - wy),
        "w01": (1.0 - wx) * wy, "w11": wx * wy,
    }


# ---------------------------------------------------------------------------
# Source waveform (fdtd2d/torch_backend.py:80-102)
# ---------------------------------------------------------------------------

def linear_chirp(dt, duration_s, f_start_hz, f_end_hz):
    """Hann-windowed linear chirp as the torch backend builds it.

    Restates torch_backend.linear_chirp (fdtd2d/torch_backend.py:80-102): the
    sweep rate uses ``(n_pulse - 1) * dt`` and the Hann window ``n_pulse - 1``.
    """
    n_pulse = max(int(round(duration_s / dt)), 2)
    t = np.arange(n_pulse) * dt
    sweep = (f_end_hz - f_start_hz) / float((n_pulse - 1) * dt)
    phase = 2.0 * np.pi * (f_start_hz * t + 0.5 * sweep * t * t)
    window = 0.5 - 0.5 * np.cos(2.0 * np.pi * np.arange(n_pulse) / (n_pulse - 1))
    return window * np.sin(phase)


# ---------------------------------------------------------------------------
# Stencil, Mur edges, one leapfrog step (fdtd2d/torch_backend.py)
# ---------------------------------------------------------------------------

def laplacian(u, dx, dy):
    """5-point Laplacian with zero padding, evaluated at every node.

    Restates the 3x3 conv2d kernel with ``padding=1`` (fdtd2d/torch_backend.py:
    122-132 and 170-174). Works on ``(..., ny, nx)``.
    """
    inv_dx2 = 1.0 / dx**2
    inv_dy2 = 1.0 / dy**2
    p = np.zeros(u.shape[:-2] + (u.shape[-2] + 2, u.shape[-1] + 2), dtype=u.dtype)
    p[..., 1:-1, 1:-1] = u
    return (
        (p[..., 1:-1, :-2] + p[..., 1:-1, 2:]) * inv_dx2
        + (p[..., :-2, 1:-1] + p[..., 2:, 1:-1]) * inv_dy2
        - 2.0 * (inv_dx2 + inv_dy2) * u
    )


def mur_coefficients(c, dt, dx, dy):
    """First-order Mur coefficients (fdtd2d/torch_backend.py:264-275)."""
    c = np.asarray(c)
    k = {
        "left": (c[1:-1, 0] * dt - dx) / (c[1:-1, 0] * dt + dx),
        "right": (c[1:-1, -1] * dt - dx) / (c[1:-1, -1] * dt + dx),
        "bottom": (c[0, 1:-1] * dt - dy) / (c[0, 1:-1] * dt + dy),
        "top": (c[-1, 1:-1] * dt - dy) / (c[-1, 1:-1] * dt + dy),
    }
    corners = np.array([c[0, 0], c[0, -1], c[-1, 0], c[-1, -1]])
    k["corner_kx"] = (corners * dt - dx) / (corners * dt + dx)
    k["corner_ky"] = (corners * dt - dy) / (corners * dt + dy)
    return k


_CORNERS = ((0, 0, 1, 1), (0, -1, 1, -2), (-1, 0, -2, 1), (-1, -1, -2, -2))


def apply_mur(u, u_next, k):
    """Mur edges, then corners from the already updated edges, in place.

    Restates _apply_mur_batch (fdtd2d/torch_backend.py:477-490), which is the
    batched form of the single-shot update at 212-232 and of the NumPy
    FDTD2D._apply_mur / _mur_corner (fdtd2d/solver.py:90-124). Works on
    ``(..., ny, nx)``.
    """
    u_next[..., 1:-1, 0] = u[..., 1:-1, 1] + k["left"] * (u_next[..., 1:-1, 1] - u[..., 1:-1, 0])
    u_next[..., 1:-1, -1] = u[..., 1:-1, -2] + k["right"] * (u_next[..., 1:-1, -2] - u[..., 1:-1, -1])
    u_next[..., 0, 1:-1] = u[..., 1, 1:-1] + k["bottom"] * (u_next[..., 1, 1:-1] - u[..., 0, 1:-1])
    u_next[..., -1, 1:-1] = u[..., -2, 1:-1] + k["top"] * (u_next[..., -2, 1:-1] - u[..., -1, 1:-1])
    vals = []
    for i, (r, c, ri, ci) in enumerate(_CORNERS):
        cu = u[..., r, c]
        from_x = u[..., r, ci] + k["corner_kx"][i] * (u_next[..., r, ci] - cu)
        from_y = u[..., ri, c] + k["corner_ky"][i] * (u_next[..., ri, c] - cu)
        vals.append(0.5 * (from_x + from_y))
    for (r, c, _, _), v in zip(_CORNERS, vals):
        u_next[..., r, c] = v
    return u_next


def forward_step(u_old, u, c2, dt2, dx, dy, k, source=None):
    """One forward leapfrog step ``u+ = 2u - u- + dt^2 c^2 lap(u) + s``, then Mur.

    Restates _advance_field / _advance_field_batch (fdtd2d/torch_backend.py:
    177-233 and 493-522): the soft source is added to ``u+`` before the Mur
    edges overwrite the boundary. ``source`` is None or an array broadcastable
    to ``u`` (a dense field holding the nearest-node or bilinear injection).
    """
    u_next = 2.0 * u - u_old + dt2 * c2 * laplacian(u, dx, dy)
    if source is not None:
        u_next = u_next + source
    return apply_mur(u, u_next, k)


def adjoint_step(l_old, l, c2, dt2, dx, dy, k, source=None):
    """Adjoint step ``l+ = 2l - l- + dt^2 lap(c^2 l) + s``, then the forward Mur.

    Restates _advance_adjoint_field_batch (fdtd2d/torch_backend.py:525-537) and
    the single-shot adjoint branch of _advance_field (201-205): the adjoint
    reuses the forward Mur update, which is not its exact transpose
    (fdtd2d/inversion/gradient.py:9-11).
    """
    l_next = 2.0 * l - l_old + dt2 * laplacian(c2 * l, dx, dy)
    if source is not None:
        l_next = l_next + source
    return apply_mur(l, l_next, k)


# ---------------------------------------------------------------------------
# Receivers and sources
# ---------------------------------------------------------------------------

def gather(fields, geo):
    """Bilinear receiver samples ``(..., R)`` (fdtd2d/torch_backend.py:540-548)."""
    return (
        fields[..., geo["row0"], geo["col0"]] * geo["w00"]
        + fields[..., geo["row0"], geo["col1"]] * geo["w10"]
        + fields[..., geo["row1"], geo["col0"]] * geo["w01"]
        + fields[..., geo["row1"], geo["col1"]] * geo["w11"]
    )


def scatter(residual, geo, shape):
    """Transpose of ``gather``: ``(S, R)`` residuals onto ``(S, ny, nx)``.

    Restates _adjoint_inject_batch's four accumulating index_put_ calls
    (fdtd2d/torch_backend.py:571-577) and RingArray.record_adjoint
    (fdtd2d/array.py:87-105).
    """
    residual = np.asarray(residual)
    out = np.zeros((residual.shape[0],) + tuple(shape), dtype=residual.dtype)
    for s in range(residual.shape[0]):
        for rows, cols, w in (("row0", "col0", "w00"), ("row0", "col1", "w10"),
                              ("row1", "col0", "w01"), ("row1", "col1", "w11")):
            np.add.at(out[s], (geo[rows], geo[cols]), residual[s] * geo[w])
    return out


def point_sources(shape, rows, cols, weights=None):
    """Dense per-shot injection fields with one or more weighted nodes per shot.

    Nearest-node injection (fdtd2d/torch_backend.py:517, ``u_next[b, row_b,
    col_b] += value``) is one node of weight 1 per shot. The bilinear source of
    desmond/src/phase2_numerics.py:107-118 is four nodes per shot with the
    bilinear weights, added as a dense field (torch_backend.py:209-210).
    ``rows``/``cols``/``weights`` are ``(S,)`` or ``(S, K)``.
    """
    rows = np.atleast_1d(np.asarray(rows))
    cols = np.atleast_1d(np.asarray(cols))
    if rows.ndim == 1:
        rows = rows[:, None]
        cols = cols[:, None]
    if weights is None:
        weights = np.ones(rows.shape)
    weights = np.asarray(weights, dtype=float).reshape(rows.shape)
    field = np.zeros((rows.shape[0],) + tuple(shape))
    for s in range(rows.shape[0]):
        np.add.at(field[s], (rows[s], cols[s]), weights[s])
    return field


def bilinear_source_taps(geo, tx):
    """Rows, columns and weights of the 4-node bilinear source of element ``tx``.

    Restates desmond/src/phase2_numerics.py:107-118, which spreads the point
    source over the four surrounding nodes with the receiver weights.
    """
    rows = [geo["row0"][tx], geo["row0"][tx], geo["row1"][tx], geo["row1"][tx]]
    cols = [geo["col0"][tx], geo["col1"][tx], geo["col0"][tx], geo["col1"][tx]]
    w = [geo["w00"][tx], geo["w10"][tx], geo["w01"][tx], geo["w11"][tx]]
    return np.array(rows), np.array(cols), np.array(w)


# ---------------------------------------------------------------------------
# Batched drivers (fdtd2d/torch_backend.py:736-770, invert_ring.py:422-455)
# ---------------------------------------------------------------------------

def simulate_shots_batch(c, dx, dy, dt, geo, source_fields, source_values, n_steps,
                         store=False, dtype=np.float64):
    """Batched forward run; returns traces ``(S, R, n_steps)`` and the final state.

    Restates simulate_shots_batch (fdtd2d/torch_backend.py:736-770): every step
    injects ``source_values[step] * source_fields`` (per-shot dense fields), applies
    Mur and samples the receivers from the new field. ``source_values`` is
    ``(n_steps,)`` (one waveform shared by all shots, as in the reference) or
    ``(S, n_steps)``. With ``store=True`` also returns every field after every step
    ``(n_steps, S, ny, nx)`` as forward_store_batch does with ``store_every=1``
    (invert_ring.py:422-455).
    """
    c = np.asarray(c, dtype=dtype)
    c2 = c * c
    dt2 = dtype(dt) * dtype(dt)
    k = mur_coefficients(c, dtype(dt), dtype(dx), dtype(dy))
    source_fields = np.asarray(source_fields, dtype=dtype)
    n_shots = source_fields.shape[0]
    values = np.asarray(source_values, dtype=dtype)
    if values.ndim == 1:
        values = np.broadcast_to(values, (n_shots, values.shape[0]))
    u_old = np.zeros((n_shots,) + c.shape, dtype=dtype)
    u = np.zeros_like(u_old)
    n_rx = len(geo["row0"])
    traces = np.zeros((n_shots, n_rx, n_steps), dtype=dtype)
    wave = np.zeros((n_steps,) + u.shape, dtype=dtype) if store else None
    for step in range(n_steps):
        src = source_fields * values[:, step, None, None] if step < values.shape[1] else None
        u_next = forward_step(u_old, u, c2, dt2, dx, dy, k, src)
        u_old, u = u, u_next
        traces[:, :, step] = gather(u, geo)
        if store:
            wave[step] = u
    return traces, u_old, u, wave


def residual_batch(predicted, observed, mute):
    """Residual with each shot's transmitter channel zeroed.

    Restates TorchLeastSquaresFWI._residual_batch (invert_ring.py:603-609) and
    fdtd2d/inversion/misfit.py:6-16. ``mute`` holds one channel per shot, or -1
    for no muting (the arc geometry, invert_arc.py:294-307).
    """
    residual = np.array(predicted - observed, copy=True)
    for s, ch in enumerate(np.asarray(mute)):
        if ch >= 0:
            residual[s, ch] = 0.0
    return residual


def adjoint_gradient_c2(c, dx, dy, dt, geo, wave, residual, dtype=np.float64):
    """Summed-over-shots gradient with respect to c^2 by the reverse-time loop.

    Restates _adjoint_accumulate_batch with ``store_every = 1`` (invert_ring.py:
    683-701) and the fused adjoint_step_image / adjoint_step_residual steps
    (fdtd2d/torch_backend.py:563-598): at loop index n the residual column n is
    scattered and injected, the adjoint field steps, and for n >= 1
    ``g += dt^2 * sum_shots(l+ * lap(wave[n-1]))`` with the zero-padded Laplacian.
    ``wave`` is ``(n_steps, S, ny, nx)``, ``residual`` ``(S, R, n_steps)``.
    ``dtype`` float32 runs the fields in single precision (the reference's
    float32 path) with the gradient still summed in float64.
    """
    c = np.asarray(c, dtype=dtype)
    c2 = c * c
    dt2 = dtype(dt) * dtype(dt)
    k = mur_coefficients(c, dtype(dt), dtype(dx), dtype(dy))
    n_steps = residual.shape[2]
    n_shots = residual.shape[0]
    residual = np.asarray(residual, dtype=dtype)
    geo = {key: (np.asarray(v, dtype=dtype) if key.startswith("w") else v) for key, v in geo.items()}
    l_old = np.zeros((n_shots,) + c.shape, dtype=dtype)
    lam = np.zeros_like(l_old)
    g = np.zeros(c.shape)
    for n in range(n_steps - 1, -1, -1):
        src = scatter(residual[:, :, n], geo, c.shape)
        l_next = adjoint_step(l_old, lam, c2, dt2, dx, dy, k, src)
        l_old, lam = lam, l_next
        if n > 0:
            g += dt2 * np.sum(lam * laplacian(wave[n - 1], dx, dy), axis=0)
    return g


def misfit_and_gradient_c2(c, dx, dy, dt, geo, source_fields, source_values, n_steps,
                           observed, mute, dtype=np.float64):
    """Misfit ``0.5 * sum(residual^2)`` and the unmasked ``g_{c^2}``.

    The device part of TorchLeastSquaresFWI.misfit_and_grad (invert_ring.py:
    634-656) for fixed shots with ``store_every = 1``, in ``dtype`` (float64 by
    default).
    """
    geo_d = {key: (np.asarray(v, dtype=dtype) if key.startswith("w") else v) for key, v in geo.items()}
    traces, _, _, wave = simulate_shots_batch(
        c, dx, dy, dt, geo_d, source_fields, source_values, n_steps, store=True, dtype=dtype)
    residual = residual_batch(traces, np.asarray(observed, dtype=dtype), mute)
    misfit = 0.5 * float(np.sum(residual.astype(np.float64) ** 2))
    return misfit, adjoint_gradient_c2(c, dx, dy, dt, geo, wave, residual, dtype=dtype)


def gradient_m(g_c2, m, mask=None):
    """Chain rule to slowness squared ``g_m = -g_{c^2} / m^2``, zero off the mask.

    Restates invert_ring.py:657-659 (without the regularisation terms).
    """
    g = -np.asarray(g_c2, dtype=float) / (np.asarray(m, float) ** 2)
    if mask is not None:
        g = np.where(mask, g, 0.0)
    return g


def interior_mask(x_m, y_m, radius_m, margin_m, center=(0.0, 0.0)):
    """Pixels strictly inside ``radius - margin`` (fdtd2d/inversion/medium.py:28-40)."""
    x, y = np.meshgrid(x_m, y_m, indexing="xy")
    r = float(radius_m) - float(margin_m)
    return (x - center[0]) ** 2 + (y - center[1]) ** 2 < r * r


def resize_slowness(m, source_axes, target_axes, background_m):
    """Bicubic transfer of m between grid levels (invert_ring.py:1048-1068).

    The reference calls ``torch.nn.functional.grid_sample`` (PyTorch, bicubic,
    ``padding_mode="border"``, ``align_corners=True``) in float64. Restated here
    from that operator's published definition: Keys' cubic convolution with
    a = -0.75 on the 4 x 4 neighbours, along x first, then y, neighbour indices
    clamped into the grid; points outside the source grid get ``background_m``.
    """
    m = np.asarray(m, dtype=float)
    sx, sy = (np.asarray(a, dtype=float) for a in source_axes)
    tx, ty = (np.asarray(a, dtype=float) for a in target_axes)
    u = 2.0 * (tx - sx[0]) / (sx[-1] - sx[0]) - 1.0
    v = 2.0 * (ty - sy[0]) / (sy[-1] - sy[0]) - 1.0
    vv, uu = np.meshgrid(v, u, indexing="ij")
    ny, nx = m.shape
    fx = ((uu + 1.0) / 2.0) * (nx - 1)
    fy = ((vv + 1.0) / 2.0) * (ny - 1)
    x0, y0 = np.floor(fx), np.floor(fy)
    tx_, ty_ = fx - x0, fy - y0
    a = -0.75

    def near(x):
        return ((a + 2.0) * x - (a + 3.0)) * x * x + 1.0

    def far(x):
        return ((a * x - 5.0 * a) * x + 8.0 * a) * x - 4.0 * a

    def weights(t):
        s = 1.0 - t
        return far(t + 1.0), near(t), near(s), far(s + 1.0)

    ix, iy = x0.astype(np.int64), y0.astype(np.int64)
    wx, wy = weights(tx_), weights(ty_)
    out = np.zeros(uu.shape)
    for r in range(4):
        yy = np.clip(iy - 1 + r, 0, ny - 1)
        row = np.zeros(uu.shape)
        for q in range(4):
            xx = np.clip(ix - 1 + q, 0, nx - 1)
            row = row + m[yy, xx] * wx[q]
        out = out + row * wy[r]
    out[(np.abs(uu) > 1.0) | (np.abs(vv) > 1.0)] = background_m
    return out


# ---------------------------------------------------------------------------
# Regularisers and projected Adam (fdtd2d/inversion/misfit.py, invert_ring.py)
# ---------------------------------------------------------------------------

def _mask_pairs(mask, axis):
    """Forward-difference pairs along ``axis`` whose two pixels are both inside."""
    if axis == 1:
        return mask[:, 1:] & mask[:, :-1]
    return mask[1:, :] & mask[:-1, :]


def tikhonov(m, mask, alpha):
    """Value and gradient of 0.5 * alpha * sum of squared in-mask forward differences.

    Restates fdtd2d/inversion/misfit.py:19-44: a difference counts only when
    both its pixels lie in the mask; the gradient is zero outside the mask.
    """
    m = np.asarray(m, dtype=float)
    mask = np.asarray(mask, dtype=bool)
    grad = np.zeros_like(m)
    if alpha <= 0.0:
        return 0.0, grad
    total = 0.0
    for axis in (1, 0):
        pairs = _mask_pairs(mask, axis)
        diff = np.diff(m, axis=axis)
        total += 0.5 * alpha * float(np.sum(diff[pairs] ** 2))
        flux = np.where(pairs, alpha * diff, 0.0)
        hi = (slice(None), slice(1, None)) if axis == 1 else (slice(1, None), slice(None))
        lo = (slice(None), slice(None, -1)) if axis == 1 else (slice(None, -1), slice(None))
        grad[hi] += flux
        grad[lo] -= flux
    grad[~mask] = 0.0
    return total, grad


def total_variation(m, mask, alpha, eps):
    """Value and gradient of alpha * sum(sqrt(|grad m|^2 + eps^2) - eps).

    Restates fdtd2d/inversion/misfit.py:47-71: in-mask forward differences
    (zero where a pair leaves the mask, and in the last row / column), the
    smoothed norm per pixel, and the gradient zeroed outside the mask.
    """
    m = np.asarray(m, dtype=float)
    mask = np.asarray(mask, dtype=bool)
    grad = np.zeros_like(m)
    if alpha <= 0.0:
        return 0.0, grad
    ddx = np.zeros_like(m)
    ddy = np.zeros_like(m)
    ddx[:, :-1] = np.where(_mask_pairs(mask, 1), np.diff(m, axis=1), 0.0)
    ddy[:-1, :] = np.where(_mask_pairs(mask, 0), np.diff(m, axis=0), 0.0)
    norm = np.sqrt(ddx * ddx + ddy * ddy + eps * eps)
    value = alpha * float(np.sum(norm - eps))
    qx = alpha * ddx / norm
    qy = alpha * ddy / norm
    grad -= qx + qy
    grad[:, 1:] += qx[:, :-1]
    grad[1:, :] += qy[:-1, :]
    grad[~mask] = 0.0
    return value, grad


def projected_adam(m0, misfit_and_grad, project, mask, learning_rate, iterations,
                   beta1=0.9, beta2=0.999, epsilon=1e-30):
    """The iterates of projected Adam (invert_ring.py:817-861).

    Moments update on the mask only; the bias-corrected step
    ``lr * m_hat / (sqrt(v_hat) + eps)`` is applied on the mask and the result
    projected. Returns the model after each of ``iterations`` steps.
    """
    mask = np.asarray(mask, dtype=bool)
    m = project(np.asarray(m0, dtype=float))
    _, g = misfit_and_grad(m)
    first = np.zeros_like(m)
    second = np.zeros_like(m)
    out = []
    for k in range(1, iterations + 1):
        first[mask] = beta1 * first[mask] + (1.0 - beta1) * g[mask]
        second[mask] = beta2 * second[mask] + (1.0 - beta2) * g[mask] ** 2
        step = np.zeros_like(m)
        step[mask] = learning_rate * (first[mask] / (1.0 - beta1 ** k)) / (
            np.sqrt(second[mask] / (1.0 - beta2 ** k)) + epsilon)
        m = project(m - step)
        _, g = misfit_and_grad(m)
        out.append(m.copy())
    return out


# ---------------------------------------------------------------------------
# PML absorbing layer (no reference counterpart: the reference has first-order
# Mur edges only, fdtd2d/solver.py:90-124). An own float64 restatement of the
# engine's PML, checked against a larger grid and the water line-source trace
# of desmond/src/phase2_numerics.py:126-145.
# ---------------------------------------------------------------------------

def pml_sigma_max(cells, h, c_ref, reflection=1e-5, order=2):
    """Peak damping of a graded layer of ``cells`` cells: (order+1) c ln(1/R) / (2 L)."""
    return (order + 1) * c_ref * np.log(1.0 / reflection) / (2.0 * cells * h)


def pml_profile(n, cells, h, sigma_max, order=2):
    """Damping at cell centres ``sc[i]`` and at left faces ``sf[i]`` (face i - 1/2) of a
    padded axis of n cells whose first and last ``cells`` cells form the layer.

    Depth is measured from the layer's inner face (coordinate cells - 1/2 on the
    low side, n - cells - 1/2 on the high side, cell i at coordinate i), in units
    of the layer thickness: sigma = sigma_max * (depth / cells)^order.
    """
    def sigma(x):
        lo = np.maximum(0.0, (cells - 0.5) - x)
        hi = np.maximum(0.0, x - (n - cells - 0.5))
        return sigma_max * (np.maximum(lo, hi) / cells) ** order
    i = np.arange(n, dtype=float)
    if cells <= 0:
        return np.zeros(n), np.zeros(n)
    return sigma(i), sigma(i - 0.5)


def pml_coefficients(c, dt, dx, dy, cells, reflection=1e-5):
    """Everything the PML update needs, in float64, for a padded medium c (ny, nx)."""
    c = np.asarray(c, dtype=float)
    ny, nx = c.shape
    smax_x = pml_sigma_max(cells, dx, float(c.max()), reflection)
    smax_y = pml_sigma_max(cells, dy, float(c.max()), reflection)
    sxc, sxf = pml_profile(nx, cells, dx, smax_x)
    syc, syf = pml_profile(ny, cells, dy, smax_y)
    a = 0.5 * dt * (sxc[None, :] + syc[:, None])
    q = 1.0 / (1.0 + a)
    return {
        "sxc": sxc, "sxf": sxf, "syc": syc, "syf": syf,
        "ax": (1.0 - 0.5 * dt * sxf) / (1.0 + 0.5 * dt * sxf),   # face decay of psi_x
        "bx": dt / (dx * dx * (1.0 + 0.5 * dt * sxf)),           # face forcing scale of psi_x
        "ay": (1.0 - 0.5 * dt * syf) / (1.0 + 0.5 * dt * syf),
        "by": dt / (dy * dy * (1.0 + 0.5 * dt * syf)),
        "q": q, "A": q * (2.0 - dt * dt * sxc[None, :] * syc[:, None]), "M": (1.0 - a) * q,
    }


def pml_step(u_old, u, psx, psy, coef, dx, dy, p, source=None):
    """One leapfrog step with the PML; returns (u_next, psx_next, psy_next).

    The second-order PML (stretched coordinates s = 1 + sigma / (i omega) per axis,
    multiplied through by s_x s_y):
      u_tt + (sx + sy) u_t + sx sy u = c^2 (lap u + d/dx phi_x + d/dy phi_y),
      phi_x_t = -sx phi_x + (sy - sx) du/dx,  phi_y_t = -sy phi_y + (sx - sy) du/dy,
    with phi on the cell faces at half steps (trapezoidal decay), stored as
    psi = phi / h. Here psx[..., j, i] lives on the face between cells i-1 and i
    and psy[..., j, i] on the face between rows j-1 and j; beyond the grid u and
    psi are zero (a rigid outer wall behind the layer). ``coef`` is (c dt)^2;
    the update is u+ = q coef (lap u + div psi) + A u - M u- (+ sources) with
    q = 1 / (1 + a), A = q (2 - dt^2 sx sy), M = (1 - a) q, a = dt (sx + sy) / 2,
    which is the plain leapfrog where sigma = 0.
    """
    zx = np.zeros(u.shape[:-1] + (1,))
    zy = np.zeros(u.shape[:-2] + (1, u.shape[-1]))
    dux = np.diff(np.concatenate([zx, u], axis=-1), axis=-1)      # u_i - u_{i-1}
    duy = np.diff(np.concatenate([zy, u], axis=-2), axis=-2)      # u_j - u_{j-1}
    psx_n = p["ax"][None, :] * psx + (p["syc"][:, None] - p["sxf"][None, :]) * p["bx"][None, :] * dux
    psy_n = p["ay"][:, None] * psy + (p["sxc"][None, :] - p["syf"][:, None]) * p["by"][:, None] * duy
    div = (np.diff(np.concatenate([psx_n, zx], axis=-1), axis=-1)
           + np.diff(np.concatenate([psy_n, zy], axis=-2), axis=-2))
    u_next = (p["q"] * coef) * (laplacian(u, dx, dy) + div) + (p["A"] * u - p["M"] * u_old)
    if source is not None:
        u_next = u_next + source
    return u_next, psx_n, psy_n


def pad_medium(c, cells):
    """The medium extended by ``cells`` cells on every side with its edge values."""
    return np.pad(np.asarray(c, dtype=float), cells, mode="edge")


def simulate_pml(c, dx, dy, dt, geo, source_fields, source_values, n_steps, cells, reflection=1e-5):
    """Batched forward with the PML padded outside the grid: traces (S, R, n_steps)
    at the receivers of ``geo`` (physical-grid indices), and the final physical field."""
    cp = pad_medium(c, cells)
    p = pml_coefficients(cp, dt, dx, dy, cells, reflection)
    coef = (cp * dt) ** 2
    fields = np.asarray(source_fields, dtype=float)
    S = fields.shape[0]
    fp = np.zeros((S,) + cp.shape)
    fp[:, cells:cells + c.shape[0], cells:cells + c.shape[1]] = fields
    values = np.asarray(source_values, dtype=float)
    if values.ndim == 1:
        values = np.broadcast_to(values, (S, values.shape[0]))
    u_old = np.zeros((S,) + cp.shape)
    u = np.zeros_like(u_old)
    psx = np.zeros_like(u)
    psy = np.zeros_like(u)
    g = dict(geo)
    for k in ("row0", "row1", "col0", "col1"):
        g[k] = np.asarray(geo[k]) + cells
    traces = np.zeros((S, len(geo["row0"]), n_steps))
    for step in range(n_steps):
        src = fp * values[:, step, None, None] if step < values.shape[1] else None
        u_next, psx, psy = pml_step(u_old, u, psx, psy, coef, dx, dy, p, src)
        u_old, u = u, u_next
        traces[:, :, step] = gather(u, g)
    return traces, u[:, cells:cells + c.shape[0], cells:cells + c.shape[1]]


def analytic_line_source(r, t, h, dt_sim, pulse, c=1500.0, dt_a=None):
    """Exact 2-D response at distance r to the solver's point source (u += pulse(t_n)
    per step), as desmond/src/phase2_numerics.py:126-145 computes it: the source is
    the forcing pulse(t) h^2 / dt^2 at a point, and the 2-D Green's function
    H(t - r/c) / (2 pi c^2 sqrt(t^2 - r^2/c^2)) is integrated exactly over each fine
    time step and convolved with the pulse. ``pulse`` is a callable of time."""
    dt_a = dt_sim / 20.0 if dt_a is None else dt_a
    T = r / c
    ta = np.arange(0, t[-1] + dt_a, dt_a)
    lo = np.maximum(ta, T)
    hi = np.maximum(ta + dt_a, T)
    G = np.arccosh(hi / T) - np.arccosh(lo / T)
    s = pulse(ta + 0.5 * dt_a)
    n = ta.size
    m = 1 << int(np.ceil(np.log2(2 * n)))
    u = np.fft.irfft(np.fft.rfft(s, m) * np.fft.rfft(G, m), m)[:n] / (2 * np.pi * c ** 2)
    u *= h ** 2 / dt_sim ** 2
    return np.interp(t, ta + dt_a, u)


# ---------------------------------------------------------------------------
# Variable density (no reference counterpart in 2-D: the reference propagates
# with constant density, FWI_Technical_Note.tex:56-59, and only plans the
# conservative form at fdtd2d/wave.py:61-63). The 1-D solver of
# 1DWaveSimulation.py:116-143 gives the discretisation: u_tt = rho c^2
# d/dx((1/rho) du/dx) with 1/rho on the faces as 2 / (rho_a + rho_b). Own float64
# restatement in 2-D; at constant rho it is the reference's stencil.
# ---------------------------------------------------------------------------

def density_faces(rho):
    """Face coefficients b = 1/rho: bx (ny, nx + 1) on the faces between columns
    x-1 and x (x = 0..nx; the outer faces take the edge cell's own rho) and by
    (ny + 1, nx) between rows."""
    r = np.asarray(rho, dtype=float)
    rx = np.concatenate([r[:, :1], r, r[:, -1:]], axis=1)
    ry = np.concatenate([r[:1, :], r, r[-1:, :]], axis=0)
    return 2.0 / (rx[:, 1:] + rx[:, :-1]), 2.0 / (ry[1:, :] + ry[:-1, :])


def density_operator(u, bx, by, dx, dy):
    """D(b, u) = d/dx(b du/dx) + d/dy(b du/dy) on faces, zero beyond the grid."""
    zx = np.zeros(u.shape[:-1] + (1,))
    zy = np.zeros(u.shape[:-2] + (1, u.shape[-1]))
    fx = bx * np.diff(np.concatenate([zx, u, zx], axis=-1), axis=-1) / (dx * dx)   # (.., ny, nx + 1)
    fy = by * np.diff(np.concatenate([zy, u, zy], axis=-2), axis=-2) / (dy * dy)   # (.., ny + 1, nx)
    return np.diff(fx, axis=-1) + np.diff(fy, axis=-2)


def simulate_density(c, rho, dx, dy, dt, geo, source_fields, source_values, n_steps, store=False):
    """Batched forward u+ = 2u - u- + dt^2 rho c^2 D(1/rho, u) + s with the
    reference's Mur edges (the local sound speed, fdtd2d/solver.py:90-124):
    traces (S, R, n_steps), and with ``store`` every field (n_steps, S, ny, nx)."""
    c = np.asarray(c, dtype=float)
    rho = np.asarray(rho, dtype=float)
    kap = dt * dt * rho * c * c
    bx, by = density_faces(rho)
    k = mur_coefficients(c, dt, dx, dy)
    fields = np.asarray(source_fields, dtype=float)
    S = fields.shape[0]
    values = np.asarray(source_values, dtype=float)
    if values.ndim == 1:
        values = np.broadcast_to(values, (S, values.shape[0]))
    u_old = np.zeros((S,) + c.shape)
    u = np.zeros_like(u_old)
    traces = np.zeros((S, len(geo["row0"]), n_steps))
    wave = np.zeros((n_steps,) + u.shape) if store else None
    for step in range(n_steps):
        u_next = 2.0 * u - u_old + kap * density_operator(u, bx, by, dx, dy)
        if step < values.shape[1]:
            u_next = u_next + fields * values[:, step, None, None]
        u_next = apply_mur(u, u_next, k)
        u_old, u = u, u_next
        traces[:, :, step] = gather(u, geo)
        if store:
            wave[step] = u
    return traces, wave


def density_gradient(c, rho, dx, dy, dt, geo, source_fields, source_values, n_steps, observed, mute):
    """Misfit and the gradients with respect to kappa = rho c^2 (per cell) and to
    the face coefficients bx, by, by the reverse-time loop of
    adjoint_gradient_c2 with the density operator: l+ = 2l - l- + D(b, dt^2 kappa l)
    + scatter(residual), the forward Mur, and for n >= 1
      g_kappa += dt^2 l+ D(b, u^{n-1}),
      g_bx(face x-1|x) += dt^2 (dt^2... per face: (l+_{x-1} kappa_{x-1} - l+_x kappa_x)
                          (u_x - u_{x-1}) / dx^2, and the same for by,
    the same pairing of adjoint and forward fields as the reference's imaging
    (invert_ring.py:683-701). Returns (misfit, g_kappa, g_bx, g_by)."""
    c = np.asarray(c, dtype=float)
    rho = np.asarray(rho, dtype=float)
    kap = rho * c * c
    bx, by = density_faces(rho)
    k = mur_coefficients(c, dt, dx, dy)
    traces, wave = simulate_density(c, rho, dx, dy, dt, geo, source_fields, source_values, n_steps, store=True)
    residual = residual_batch(traces, np.asarray(observed, dtype=float), mute)
    misfit = 0.5 * float(np.sum(residual ** 2))
    S = residual.shape[0]
    l_old = np.zeros((S,) + c.shape)
    lam = np.zeros_like(l_old)
    gk = np.zeros(c.shape)
    gbx = np.zeros(bx.shape)
    gby = np.zeros(by.shape)
    dt2 = dt * dt
    zx = np.zeros((S, c.shape[0], 1))
    zy = np.zeros((S, 1, c.shape[1]))
    for n in range(n_steps - 1, -1, -1):
        src = scatter(residual[:, :, n], geo, c.shape)
        l_next = 2.0 * lam - l_old + density_operator(dt2 * kap * lam, bx, by, dx, dy) + src
        l_next = apply_mur(lam, l_next, k)
        l_old, lam = lam, l_next
        if n > 0:
            u = wave[n - 1]
            gk += dt2 * np.sum(lam * density_operator(u, bx, by, dx, dy), axis=0)
            w = lam * kap
            wx = np.concatenate([zx, w, zx], axis=-1)
            ux = np.concatenate([zx, u, zx], axis=-1)
            gbx += dt2 * np.sum(-np.diff(wx, axis=-1) * np.diff(ux, axis=-1), axis=0) / (dx * dx)
            wy = np.concatenate([zy, w, zy], axis=-2)
            uy = np.concatenate([zy, u, zy], axis=-2)
            gby += dt2 * np.sum(-np.diff(wy, axis=-2) * np.diff(uy, axis=-2), axis=0) / (dy * dy)
    return misfit, gk, gbx, gby


def density_chain_rule(m, rho, g_kappa, g_bx, g_by):
    """g_m and g_rho from the kappa and face gradients, with kappa = rho / m and
    b = 2 / (rho_a + rho_b) (an outer face: 1 / rho of its edge cell)."""
    m = np.asarray(m, dtype=float)
    rho = np.asarray(rho, dtype=float)
    bx, by = density_faces(rho)
    g_m = -g_kappa * rho / (m * m)
    g_rho = g_kappa / m
    # interior faces: db/drho_a = -b^2 / 2 for both cells; outer faces: -b^2
    hx = -0.5 * g_bx * bx * bx
    hy = -0.5 * g_by * by * by
    g_rho = g_rho + hx[:, :-1] + hx[:, 1:] + hy[:-1, :] + hy[1:, :]
    g_rho[:, 0] += hx[:, 0]
    g_rho[:, -1] += hx[:, -1]
    g_rho[0, :] += hy[0, :]
    g_rho[-1, :] += hy[-1, :]
    return g_m, g_rho
