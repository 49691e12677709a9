"""Trace files and the observed-data precompute of the FWI drivers.

``save_traces`` / ``load_traces`` read and write the reference's npz layout
(2DRingFDTD.py:291-327: keys ``traces``, ``time_s``, ``pulse``, ``dt``, ``tx``,
``theta``, ``x``, ``y``, ``radius_m``, ``sound_speed_m_s``, ``torch_device``,
``torch_dtype``, ``torch_compiled``, ``transmitter_indices``), with float16
trace storage as an option (``trace_dtype``). ``precompute_observed`` builds the
``(N transmitters, N receivers, nt)`` observed tensor of invert_ring.py:1136-1160
with the fused engine, in shot batches sized like the reference
(``observed_bytes_per_shot`` / ``auto_batch_size``).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from .fwi import observed_bytes_per_shot
from .torch_backend import TorchFDTD2DBatch, auto_batch_size, simulate_shots_batch

TRACE_DTYPES = {"float32": np.float32, "float16": np.float16, "float64": np.float64}


def save_traces(path, traces, time_s, array, tx, pulse, dt, c_map=None, device="cpu", dtype="float32",
                compiled=False, transmitter_indices=None, trace_dtype=None):
    """Write one npz with the reference's keys (2DRingFDTD.py:291-327).

    ``trace_dtype`` ("float16", "float32", "float64" or None = as given) sets the
    stored precision of ``traces``; the reference stores them as produced.
    """
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    if isinstance(traces, torch.Tensor):
        traces = traces.detach().cpu().numpy()
    traces = np.asarray(traces)
    if trace_dtype is not None:
        if trace_dtype not in TRACE_DTYPES:
            raise ValueError(f"trace_dtype must be one of {sorted(TRACE_DTYPES)}")
        traces = traces.astype(TRACE_DTYPES[trace_dtype])
    if isinstance(pulse, torch.Tensor):
        pulse = pulse.detach().cpu().numpy()
    np.savez(
        path,
        traces=traces,
        time_s=np.asarray(time_s),
        pulse=np.asarray(pulse),
        dt=dt,
        tx=tx,
        theta=array.theta,
        x=array.x,
        y=array.y,
        radius_m=array.radius_m,
        sound_speed_m_s=c_map,
        torch_device=np.asarray(str(device)),
        torch_dtype=np.asarray(str(dtype)),
        torch_compiled=np.asarray(bool(compiled)),
        transmitter_indices=(np.asarray(transmitter_indices, dtype=int)
                             if transmitter_indices is not None else np.asarray([tx], dtype=int)),
    )
    return path


def load_traces(path, dtype=np.float32):
    """Read a trace npz into a dict; ``traces`` comes back as ``dtype`` (None = stored)."""
    with np.load(Path(path), allow_pickle=True) as data:
        out = {k: data[k] for k in data.files}
    if dtype is not None:
        out["traces"] = out["traces"].astype(dtype)
    for key in ("dt", "radius_m", "tx"):
        if key in out and out[key].ndim == 0:
            out[key] = out[key].item()
    return out


def precompute_observed(solver, sampler, array, pulse, n_steps, parallel_shots="auto", source_values=None):
    """Observed gathers of every transmitter: ``(N_tx, N_rx, n_steps)`` float32 on the device.

    invert_ring.py:1136-1160: transmitter ``tx`` fires at ``array.inject_rows_cols(tx)``
    with the shared waveform; batches of ``parallel_shots`` shots ("auto" sizes
    them from free device memory like the reference).
    """
    model = solver.model
    n_tx = int(array.n_elements)
    if parallel_shots == "auto":
        parallel_shots = auto_batch_size(model.device, n_tx, observed_bytes_per_shot(
            n_steps, model.shape, sampler.n_elements))
    batch = max(1, min(int(parallel_shots), n_tx))
    observed = torch.empty((n_tx, sampler.n_elements, int(n_steps)), device=model.device, dtype=torch.float32)
    batched_solvers = {}
    for start in range(0, n_tx, batch):
        sources = np.arange(start, min(start + batch, n_tx))
        rows_cols = [array.inject_rows_cols(int(tx)) for tx in sources]
        rows = np.asarray([r for r, _ in rows_cols], dtype=np.int64)
        cols = np.asarray([c for _, c in rows_cols], dtype=np.int64)
        batched = batched_solvers.get(len(sources))
        if batched is None:
            batched = TorchFDTD2DBatch(solver, len(sources))
            batched_solvers[len(sources)] = batched
        traces, _ = simulate_shots_batch(solver, sampler, pulse, rows, cols, int(n_steps), batched=batched,
                                         source_values=source_values)
        observed[start:start + len(sources)].copy_(traces)
    return observed
