"""Launch-shape autotuner of the temporally blocked engine.

For one acquisition (grid, shots, receivers, sources), time a short forward of
each candidate launch shape — rows per lane, warps per CTA (region height) and
steps per launch (temporal-block depth, which sets the halo) — on the device
and keep the fastest. Results are cached per (grid, shots, receivers, device).
The planner's own default depth comes from a cost model (tiles x (T + 3) / T);
the autotuner measures instead of modelling.
"""

from __future__ import annotations

import sys
import time

import torch

from .engine import FusedPlan

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

    With ``for_gradient`` each probe is a whole gradient pass (forward with
    checkpoints, recompute and adjoint launches), since the adjoint kernel
    prefers other shapes than the forward (its coefficient tile is read
    through L1, so its shared-memory footprint matters).
    """
    dev = medium.device
    n_shots = len(sources[0])
    key = (medium.ny, medium.nx, n_shots, len(receivers[0]), str(dev), shapes, depths, bool(for_gradient))
    if key in _CACHE:
        return dict(_CACHE[key])
    best, best_rate, report = None, 0.0, []
    t_start = time.perf_counter()
    for cand in candidates(shapes, depths):
        steps = min(int(n_steps), launches * cand["steps_per_launch"])
        try:
            plan = FusedPlan(medium, receivers, sources, waveforms, steps, tuning=cand,
                             for_gradient=for_gradient)
        except ValueError:
            continue  # shape not supported for this grid (tiling or shared memory)
        traces = plan.forward()
        grad = None
        if for_gradient:
            grad = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=dev)

        def one_pass():
            if for_gradient:
                plan.forward(traces, save_checkpoints=True)
                plan.adjoint(traces, grad)  # any residual: the cost does not depend on its values
            else:
                plan.forward(traces)

        one_pass()
        torch.cuda.synchronize(dev)
        stream = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            one_pass()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / repeats
        rate = float(medium.ny) * medium.nx * n_shots * steps / (ms * 1e-3) / 1e9
        report.append((rate, cand))
        if rate > best_rate:
            best, best_rate = dict(cand), rate
        del plan, traces, grad
    if best is None:
        raise RuntimeError("no candidate launch shape fits this problem")
    if verbose:
        for rate, cand in sorted(report, key=lambda r: -r[0])[:8]:
            print(f"  {rate:8.1f} Gcell/s  {cand}", file=sys.stderr)
        print(f"  autotune: {len(report)} shapes in {time.perf_counter() - t_start:.1f} s", file=sys.stderr)
    _CACHE[key] = dict(best)
    return best


def clear_cache():
    _CACHE.clear()
