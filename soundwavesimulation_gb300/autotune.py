"""Launch-shape autotuner of the temporally blocked engine.

For one acquisition (grid, shots, receivers, sources), time a short forward of
each candidate launch shape — rows per lane, warps per CTA (region height) and
steps per launch (temporal-block depth, which sets the halo) — on the device
and keep the fastest. Results are cached per (grid, shots, receivers, device).
The planner's own default depth comes from a cost model (tiles x (T + 3) / T);
the autotuner measures instead of modelling.
"""

from __future__ import annotations

import ctypes
import sys
import time

import torch

from . import _lib
from .engine import ProblemTables, ptr, stream_handle

_CACHE: dict = {}

SHAPES = ((8, 16), (8, 12), (8, 10), (4, 32), (4, 16))   # (rows per lane, warps)
DEPTHS = (6, 8, 10, 12, 15, 19, 23)              # steps per launch


def candidates(shapes=SHAPES, depths=DEPTHS):
    for ky, warps in shapes:
        for t in depths:
            yield {"rows_per_lane": ky, "warps": warps, "steps_per_launch": t}


def autotune(medium, receivers, sources, waveforms, n_steps, launches=3, repeats=2, shapes=SHAPES,
             depths=DEPTHS, verbose=False, for_gradient=False):
    """Fastest tuning dict for this acquisition; probes ``launches`` temporal blocks per shape.

    The search runs in the engine library (``fdtd_autotune``) over the candidate
    shapes above, with one workspace from the caching allocator. With
    ``for_gradient`` each probe is a whole gradient pass (forward with
    checkpoints, recompute and adjoint launches), since the adjoint kernel
    prefers other shapes than the forward (its coefficient tile is read
    through L1, so its shared-memory footprint matters).
    """
    if tuple(shapes) != SHAPES or tuple(depths) != DEPTHS:
        raise ValueError("the library searches the standard shape and depth sets")
    dev = medium.device
    n_shots = len(sources[0])
    key = (medium.ny, medium.nx, n_shots, len(receivers[0]), str(dev), bool(for_gradient), int(n_steps))
    if key in _CACHE:
        return dict(_CACHE[key])
    lib = _lib.load()
    tables = ProblemTables(medium, receivers, sources, waveforms, n_steps)
    prob = tables.problem()
    t_start = time.perf_counter()
    nbytes = int(lib.fdtd_autotune_workspace_bytes(ctypes.byref(prob), int(bool(for_gradient)), launches))
    if nbytes == 0:
        raise RuntimeError("no candidate launch shape fits this problem")
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    cap = len(SHAPES) * len(DEPTHS)
    tried = (_lib.Tuning * cap)()
    rates = (ctypes.c_double * cap)()
    n_tried = ctypes.c_int32(cap)
    best = _lib.Tuning()
    best_rate = ctypes.c_double()
    _lib.check(lib.fdtd_autotune(ctypes.byref(prob), int(bool(for_gradient)), launches, repeats, ptr(ws), nbytes,
                                 ctypes.byref(best), ctypes.byref(best_rate), tried, rates, ctypes.byref(n_tried),
                                 stream_handle(dev)), "autotune")
    chosen = {k: best.as_dict()[k] for k in ("rows_per_lane", "warps", "steps_per_launch")}
    if verbose:
        report = sorted(((rates[i], tried[i].as_dict()) for i in range(n_tried.value)), key=lambda r: -r[0])
        for rate, t in report[:8]:
            print(f"  {rate:8.1f} Gcell/s  { {k: t[k] for k in chosen} }", file=sys.stderr)
        print(f"  autotune: {n_tried.value} shapes in {time.perf_counter() - t_start:.1f} s", file=sys.stderr)
    _CACHE[key] = dict(chosen)
    return chosen


def clear_cache():
    _CACHE.clear()
