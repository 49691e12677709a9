"""Benchmark: batched forward and FWI gradient Gcell-updates/s on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (512 x 512 grid, 128 shots, 4000 steps, the batched-forward
configuration): one bench step is one full batched forward pass over all shots
(the time loop inside the fused engine). The JSON line also carries the FWI
gradient at 512 x 512 x 128 shots (forward + checkpointed adjoint), the plain
per-shot one-step-per-launch form, the HBM roofline of the dominant kernel,
the end-to-end number through the public API with host buffers, and the
oracle port timed on the host cores. ``--impl reference`` times the CPU
restatement of the reference (NumPy) on a bounded sample of the same workload.
Under torchrun every rank runs its own 128 shots (weak scaling); the gradient
sums over ranks with one all-reduce.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
METRIC = "Gcell-updates/s fwd & FWI grad at 512²×128 shots; % HBM peak; vs plain"
UNIT = "Gcell-updates/s"
FWD_BYTES_PER_CELL = 12.0    # read u, read u_old, write u_next (float32)
GRAD_BYTES_PER_CELL = 28.0   # forward 12 + adjoint 12 + one read of the forward field 4
# DRAM bytes (read + write) of one forward launch at 512^2 x 128 shots, from one ncu
# capture of that launch, keyed by the digest of the kernel sources it was taken on
# and the launch shape (rows per lane, warps, steps per launch). A bench run on
# other sources or another shape reports the figure as null.
FWD_TRAFFIC = {("0510d886fb66", 8, 16, 15): 398.682880e6 + 219.159296e6}
KERNEL_SOURCES = ("soundwavesimulation_gb300/csrc/fdtd_tb.cu", "soundwavesimulation_gb300/csrc/fdtd_tb.cuh",
                  "soundwavesimulation_gb300/csrc/fdtd_device.cuh")


def kernel_digest():
    """First 12 hex digits of the SHA-256 of the temporally blocked kernel's sources."""
    import hashlib
    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        h.update((ROOT / rel).read_bytes())
    return h.hexdigest()[:12]


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        if shutil.which("nvidia-smi") is None:
            return self
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(
            ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
             "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _oracle_shots(job):
    """One worker's share of the CPU sample: the oracle port's batched forward on its shots."""
    sys.path.insert(0, str(ROOT))
    from oracle import fdtd_oracle as orc
    c, dx, dt, geo, fields, wave, n_steps = job
    orc.simulate_shots_batch(c, dx, dx, dt, geo, fields, wave, n_steps, dtype=np.float32)
    return fields.shape[0]


def cpu_workers():
    """Host cores available to this process."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def make_cpu_pool(workers):
    """Process pool for the CPU sample, started with spawn (safe beside a CUDA context)."""
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(workers)


def cpu_sample(acq, pool, workers, shots_per_worker=1, n_steps=480):
    """Time the oracle port (NumPy, float32) on a bounded sample of the workload, one
    process per host core, each advancing its own shots (shots are independent)."""
    sys.path.insert(0, str(ROOT))
    from oracle import fdtd_oracle as orc
    n_shots = min(acq.n_shots, workers * shots_per_worker)
    sub = acq.subset(n_shots=n_shots, n_steps=n_steps)
    rows, cols, w, _ = sub.source_tables()
    fields = orc.point_sources(sub.c.shape, rows, cols, w)
    geo = orc.ring_geometry(sub.n_elements, 0.45 * sub.n * sub.dx, sub.x, sub.x)
    chunks = [c for c in np.array_split(np.arange(n_shots), workers) if c.size]
    jobs = [(sub.c, sub.dx, sub.dt, geo, fields[c], sub.wavelet[:n_steps], n_steps) for c in chunks]
    pool.map(_oracle_shots, jobs[:1])  # workers up
    t0 = time.perf_counter()
    done = sum(pool.map(_oracle_shots, jobs))
    dt = time.perf_counter() - t0
    cells = float(sub.n) ** 2 * done * n_steps
    return (cells / dt / 1e9,
            f"{done} shots x {n_steps} of {acq.n_steps} steps at {acq.n}^2, {len(jobs)} processes (float32 NumPy)",
            len(jobs))


def parity_check(acq, traces, grad_tuning, device, shots=(0, 37, 74, 111)):
    """The host-core leg's checker: float64 C oracle (oracle/fdtd_oracle.c) against
    the engine on a few shots of the workload at its full grid and step count.

    Traces: the bench's own forward traces of those shots. Gradient: the FWI
    gradient of those shots from the blurred start, with float32 and with
    float16 checkpoints (and the timed plan's kept segments: grad_tuning), against
    the oracle's float64 adjoint gradient, rel-L2 on the inversion mask.
    """
    import torch
    sys.path.insert(0, str(ROOT))
    from oracle import c_oracle
    from soundwavesimulation_gb300 import interior_mask
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, residual_misfit
    from soundwavesimulation_gb300.phantoms import blurred_start
    t0 = time.perf_counter()
    c_oracle.build()
    sh = np.asarray(shots)
    rows, cols, w, wave = acq.source_tables()
    src = (rows[sh], cols[sh], w[sh])
    ref = c_oracle.forward_shots(acq.c, acq.dx, acq.dx, acq.dt, src, acq.ring.receiver_taps(), acq.wavelet,
                                 acq.n_steps)
    mine = traces[torch.as_tensor(sh, device=device)].cpu().numpy().astype(np.float64)
    trace_err = float(np.linalg.norm(mine - ref) / np.linalg.norm(ref))
    mask = interior_mask(acq.x, acq.x, 0.45 * acq.n * acq.dx, margin_m=3 * acq.dx)
    c0 = blurred_start(acq.c, 10.0, mask)
    m2 = (1.0 / c0 ** 2) ** 2
    observed = traces[torch.as_tensor(sh, device=device)].contiguous()
    _, g64 = c_oracle.gradient_shots(c0, acq.dx, acq.dx, acq.dt, src, acq.ring.receiver_taps(), acq.wavelet,
                                     acq.n_steps, observed.cpu().numpy().astype(np.float64), acq.tx[sh])
    g64 = np.where(mask, -g64 / m2, 0.0)
    start = DeviceMedium(c0, acq.dx, acq.dx, acq.dt, device)
    waves = torch.as_tensor(acq.wavelet[None], dtype=torch.float32, device=device)
    mute = torch.as_tensor(acq.tx[sh], dtype=torch.int32, device=device)
    errs = {}
    for name, store in (("f32", 0), ("f16", 1)):
        plan = FusedPlan(start, acq.ring.receiver_taps(), (rows[sh], cols[sh], w[sh], wave[sh]), waves,
                         acq.n_steps, tuning={**grad_tuning, "ckpt_store": store}, for_gradient=True)
        pred = plan.forward(save_checkpoints=True)
        res, _ = residual_misfit(pred, observed, mute)
        g = torch.zeros((acq.n, start.pitch), dtype=torch.float64, device=device)
        plan.adjoint(res, g)
        gm = np.where(mask, -g[:, :acq.n].cpu().numpy() / m2, 0.0)
        errs[name] = float(np.linalg.norm(gm - g64) / np.linalg.norm(g64))
        del plan, pred, res, g
    return {"traces_rel_l2_vs_fp64": trace_err, "grad_rel_l2_vs_fp64": errs, "shots": [int(v) for v in sh],
            "steps": acq.n_steps, "budgets": {"traces": 1e-5, "grad": 1e-3},
            "checker": "float64 C oracle on the host cores", "seconds": time.perf_counter() - t0}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT))
    from soundwavesimulation_gb300.phantoms import config
    acq = config(2)[0]
    workers = cpu_workers()
    pool = make_cpu_pool(workers)
    for _ in range(args.warmup):
        cpu_sample(acq, pool, workers, n_steps=20)
    vals = []
    t0 = time.perf_counter()
    sample, cores = "", workers
    for _ in range(args.steps):
        v, sample, cores = cpu_sample(acq, pool, workers)
        vals.append(v)
    wall = time.perf_counter() - t0
    pool.close()
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded abdomen-like phantom)",
        "config": {"workload": "batched forward 512x512, 128 shots, 4000 steps (bounded CPU sample)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def bench_gradient(args, acq, medium, rx, waves, observed, tuning, device, world, barrier,
                   solver, sampler, observed_nearest):
    """FWI gradient at the workload's grid and shots; returns the JSON object."""
    import torch
    from soundwavesimulation_gb300 import fwi, interior_mask
    from soundwavesimulation_gb300.engine import (DeviceMedium, FusedPlan, ProblemTables, gradient_plain,
                                                  residual_misfit)
    from soundwavesimulation_gb300.phantoms import blurred_start
    from soundwavesimulation_gb300.sharding import allreduce_misfit_and_gradient
    n, nt, S = acq.n, acq.n_steps, acq.n_shots
    mask = interior_mask(acq.x, acq.x, 0.45 * n * acq.dx, margin_m=3 * acq.dx)
    c_start = blurred_start(acq.c, 10.0, mask)
    start = DeviceMedium(c_start, acq.dx, acq.dx, acq.dt, device)
    plan = FusedPlan(start, rx, acq.source_tables(), waves, nt, tuning=tuning, for_gradient=True)
    mute = torch.as_tensor(acq.tx, dtype=torch.int32, device=device)
    g = torch.zeros((n, start.pitch), dtype=torch.float64, device=device)
    misfit = torch.zeros(1, dtype=torch.float64, device=device)
    work = torch.empty_like(observed)

    def step(p):
        g.zero_()
        misfit.zero_()
        tr = p.forward(work, save_checkpoints=True)
        residual_misfit(tr, observed, mute, residual=tr, misfit=misfit)
        p.adjoint(tr, g)

    def timed(p, steps):
        for _ in range(args.warmup):
            step(p)
        barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for k in range(steps):
            step(p)
            ev[k + 1].record(stream)
        barrier()
        return float(np.mean([ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]))

    stream = torch.cuda.current_stream()
    ms = timed(plan, args.steps)
    # the plan keeps the stencil stream of its last kept_segments checkpoint segments
    # (60 % of the free device memory); freed before the next plans take their share
    plan_tuning, plan_ws = dict(plan.tuning), plan.workspace_bytes
    del plan
    torch.cuda.empty_cache()
    # the mixed-precision form of the benchmark spec's target: float16 checkpoints
    # (power-of-two scale per field and shot), same launch shape
    plan16 = FusedPlan(start, rx, acq.source_tables(), waves, nt, tuning={**tuning, "ckpt_store": 1},
                       for_gradient=True)
    ms16 = timed(plan16, max(1, min(args.steps, 5)))
    del plan16
    torch.cuda.empty_cache()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        allreduce_misfit_and_gradient(misfit, g)
    value = acq.cell_updates * world / (ms * 1e-3) / 1e9
    launches = sum(1 for _ in range(0, nt, plan_tuning["steps_per_launch"]))
    # recompute launches: the segments before the kept ones
    C, T = plan_tuning["ckpt_every"], plan_tuning["steps_per_launch"]
    n_rec_seg = -(-nt // C) - max(plan_tuning["kept_segments"], 0)
    rec_launches = sum(-(-(min(a + C, nt) - a) // T) for a in range(0, n_rec_seg * C, C))

    # plain per-shot gradient (full history, one launch per kernel per step) on one shot
    one = acq.subset(n_shots=1)
    tables = ProblemTables(start, rx, one.source_tables(), waves, nt)
    gradient_plain(tables, observed[:1], mute[:1])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    Jp, gp = gradient_plain(tables, observed[:1], mute[:1])
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_value = float(n) ** 2 * nt / (plain_ms * 1e-3) / 1e9
    # the fused gradient of that one shot, for an agreement figure
    p1 = FusedPlan(start, rx, one.source_tables(), waves, nt, tuning=tuning, for_gradient=True)
    tr1 = p1.forward(save_checkpoints=True)
    J1 = torch.zeros(1, dtype=torch.float64, device=device)
    residual_misfit(tr1, observed[:1], mute[:1], residual=tr1, misfit=J1)
    g1 = torch.zeros_like(g)
    p1.adjoint(tr1, g1)
    agree = float(torch.linalg.vector_norm(g1 - gp) / torch.linalg.vector_norm(gp))
    del p1, tr1

    # end to end through the public API: host slowness in, host gradient out
    problem = fwi.TorchLeastSquaresFWI(solver, sampler, acq.ring, acq.wavelet, nt, acq.n_elements,
                                       _full_gather(observed_nearest, acq), mask, parallel_shots=S,
                                       tuning=tuning)
    m_host = 1.0 / c_start ** 2
    problem.gradient_c2(m_host, acq.tx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_steps = max(1, min(args.steps, 2))
    for _ in range(e_steps):
        problem.gradient_c2(m_host, acq.tx)
    e2e_s = (time.perf_counter() - t0) / e_steps
    hbm, peak_kind = peaks()
    achieved = GRAD_BYTES_PER_CELL * acq.cell_updates / (ms * 1e-3) / 1e9
    return {
        "value": value, "unit": UNIT, "ms_per_step": ms, "metric": "FWI gradient shot-cell-step updates/s",
        "workload": f"{n}x{n}, {S} shots, {nt} steps, blurred (sigma 10 cells) start, checkpoints every "
                    f"{plan_tuning['ckpt_every']} steps (float32), the forward keeping the stencil stream of "
                    f"the last {max(plan_tuning['kept_segments'], 0)} of {-(-nt // plan_tuning['ckpt_every'])} "
                    f"segments",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "note": f"28 B per shot-cell-step algorithmic; peak {peak_kind}"},
        "plain": {"value": plain_value, "unit": UNIT, "shots_sampled": 1, "speedup": value / world / plain_value,
                  "rel_l2_fused_vs_plain": agree},
        "f16_checkpoints": {"value": acq.cell_updates * world / (ms16 * 1e-3) / 1e9, "unit": UNIT,
                            "ms_per_step": ms16,
                            "speedup_vs_plain": acq.cell_updates / (ms16 * 1e-3) / 1e9 / plain_value,
                            "note": "rel-L2 against float64 in the parity block"},
        "e2e": {"value": acq.cell_updates * world / e2e_s / 1e9, "unit": UNIT,
                "h2d_bytes_per_step": int(m_host.size * 8), "d2h_bytes_per_step": int(n * n * 8)},
        "tuning": plan_tuning,
        "gpu_launches_per_step": 2 * launches + rec_launches + 2,
        "workspace_gib": plan_ws / 2 ** 30,
    }


def bench_pml(args, acq, waves, traces, device, barrier, cells=30):
    """The same forward with a PML of ``cells`` cells padded outside the grid (the
    layer the configuration names) instead of Mur edges: throughput in physical
    cell-updates/s and in computed (padded-grid) ones, and the trace change the
    layer makes against the Mur run (the Mur echoes it removes)."""
    import torch
    from soundwavesimulation_gb300.autotune import autotune
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan
    medium = DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, device, pml_cells=cells)
    rx = acq.ring.receiver_taps()
    tuning = autotune(medium, rx, acq.source_tables(), waves, acq.n_steps)
    plan = FusedPlan(medium, rx, acq.source_tables(), waves, acq.n_steps, tuning=tuning)
    out = torch.empty_like(traces)
    for _ in range(args.warmup):
        plan.forward(out)
    barrier()
    stream = torch.cuda.current_stream()
    steps = max(1, min(args.steps, 5))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for k in range(steps):
        plan.forward(out)
        ev[k + 1].record(stream)
    barrier()
    ms = float(np.mean([ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]))
    padded = float(medium.ny) * medium.nx * acq.n_shots * acq.n_steps
    change = float(torch.linalg.vector_norm(out - traces) / torch.linalg.vector_norm(traces))
    return {"cells": cells, "value": acq.cell_updates / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms,
            "computed_value": padded / (ms * 1e-3) / 1e9, "grid": [medium.ny, medium.nx], "tuning": plan.tuning,
            "trace_change_vs_mur": change,
            "note": "value counts physical cell-updates (512^2 per shot-step); computed_value the padded grid's"}


def _full_gather(traces, acq):
    """(n_elements, R, nt) observed gathers with the bench's shots at their transmitter rows."""
    import torch
    full = torch.zeros((acq.n_elements,) + tuple(traces.shape[1:]), dtype=torch.float32, device=traces.device)
    full[torch.as_tensor(acq.tx, device=traces.device)] = traces
    return full


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(device)
    sys.path.insert(0, str(ROOT))
    from soundwavesimulation_gb300 import torch_backend as tb
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, ProblemTables, forward_plain
    from soundwavesimulation_gb300.phantoms import config

    acq = config(2)[0]
    S, n, nt = acq.n_shots, acq.n, acq.n_steps
    medium = DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, device)
    rx = acq.ring.receiver_taps()
    waves = torch.as_tensor(acq.wavelet[None], dtype=torch.float32, device=device)
    if args.tuning:
        tuning = grad_tuning = json.loads(args.tuning)
    else:
        from soundwavesimulation_gb300.autotune import autotune
        t_tune = time.perf_counter()
        tuning = autotune(medium, rx, acq.source_tables(), waves, nt, verbose=rank == 0)
        grad_tuning = autotune(medium, rx, acq.source_tables(), waves, nt, verbose=rank == 0,
                               for_gradient=True)
        print(f"autotune {time.perf_counter() - t_tune:.1f} s -> forward {tuning}, gradient {grad_tuning}",
              file=sys.stderr)
    plan = FusedPlan(medium, rx, acq.source_tables(), waves, nt, tuning=tuning)
    traces = torch.empty((S, acq.n_elements, nt), dtype=torch.float32, device=device)
    launches_per_pass = math.ceil(nt / plan.tuning["steps_per_launch"])

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        plan.forward(traces)
    barrier()
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        barrier()
        t0 = time.perf_counter()
        ev[0].record(stream)
        for k in range(args.steps):
            plan.forward(traces)
            ev[k + 1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    ms = float(np.mean(per_step))
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = acq.cell_updates * world / (ms * 1e-3) / 1e9

    # plain per-shot form on a shot subset, scaled to the workload
    plain_shots = 2
    sub = acq.subset(n_shots=plain_shots)
    tables = ProblemTables(medium, rx, sub.source_tables(), waves, nt)
    ptraces = forward_plain(tables)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    forward_plain(tables, ptraces)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_value = float(n) ** 2 * plain_shots * nt / (plain_ms * 1e-3) / 1e9
    same = bool(torch.equal(ptraces, traces[:plain_shots]))

    # end to end through the public API with host buffers
    model = tb.TorchScalarWave2D(acq.c, acq.dx, device=device)
    solver = tb.TorchFDTD2D(model, acq.dt)
    sampler = tb.TorchRingSampler(acq.ring, device=device)
    batched = tb.TorchFDTD2DBatch(solver, S)
    host_traces = torch.empty((S, acq.n_elements, nt), dtype=torch.float32, pin_memory=True)
    rows, cols = acq.ring.rows[acq.tx], acq.ring.cols[acq.tx]

    def e2e_step():
        solver.set_c(acq.c)  # host medium in
        # traces out: written by the kernels straight into the pinned host buffer
        tb.simulate_shots_batch(solver, sampler, acq.wavelet, rows, cols, nt, batched=batched, out=host_traces)
        torch.cuda.synchronize()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    e_steps = max(1, args.steps)
    for _ in range(e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e_steps
    tr = host_traces.to(device)  # the public API's traces: the gradient leg's observed data
    e2e_value = acq.cell_updates * world / e2e_s / 1e9
    h2d = acq.c.size * 8 + nt * 4 + 2 * S * 8
    d2h = int(host_traces.numel()) * 4

    # ---- the same forward with the configuration's 30-cell PML instead of Mur edges
    pml = bench_pml(args, acq, waves, traces, device, barrier)

    # ---- FWI gradient, same grid and shots: forward with checkpoints + residual + adjoint
    grad = bench_gradient(args, acq, medium, rx, waves, traces, grad_tuning, device, world, barrier,
                          solver, sampler, tr)

    hbm, peak_kind = peaks()
    achieved = FWD_BYTES_PER_CELL * acq.cell_updates / (ms * 1e-3) / 1e9
    launch_us = ms * 1e3 / launches_per_pass
    digest = kernel_digest()
    shape = (digest, plan.tuning["rows_per_lane"], plan.tuning["warps"], plan.tuning["steps_per_launch"])
    traffic = FWD_TRAFFIC.get(shape) if (n, S) == (512, 128) else None
    # compulsory DRAM bytes of one launch: u_old and u read and written once per cell
    # (16 B per cell and shot) plus the launch's trace samples
    compulsory = 16.0 * n * n * S + 4.0 * acq.n_elements * S * plan.tuning["steps_per_launch"]
    out = None
    if rank == 0:
        workers = cpu_workers()
        pool = make_cpu_pool(workers)
        cpu_v, cpu_s, cpu_cores = cpu_sample(acq, pool, workers)
        pool.close()
        # the gradient's checks with the timed plan's kept segments (the others recomputed
        # from float32 / float16 checkpoints)
        parity = parity_check(acq, traces, {**grad_tuning, "kept_segments": grad["tuning"]["kept_segments"]},
                              device)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded abdomen-like phantom, Ricker)",
            "config": {"workload": "batched forward 512x512, 128 shots (every other element of 256), "
                                   "4000 steps, 0.8 MHz Ricker, bilinear sources",
                       "grid": [n, n], "shots": S, "steps": nt, "receivers": acq.n_elements,
                       "tuning": plan.tuning, "l2": "working set 256 MiB > L2 (no flush needed)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "launch_us": launch_us,
                         "dram_frac": (traffic / (launch_us * 1e-6) / 1e9 / hbm) if traffic else None,
                         "compulsory_bytes": compulsory, "kernel_digest": digest,
                         "note": f"12 B per cell-update algorithmic; peak {peak_kind}; temporal blocking "
                                 "makes the algorithmic fraction exceed the single-step roofline; traffic = "
                                 "ncu dram bytes read+written per launch, taken on the kernel sources of "
                                 "kernel_digest at this launch shape (null otherwise); dram_frac = traffic / "
                                 "launch_us / peak; compulsory_bytes = one read and one write of both state "
                                 "fields plus the launch's traces"},
            "plain": {"value": plain_value, "unit": UNIT, "shots_sampled": plain_shots,
                      "speedup": value / world / plain_value, "bitwise_equal_traces": same},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_cores, "kind": "port", "sample": cpu_s},
            "grad": grad,
            "pml": pml,
            "parity": parity,
            "gpu_launches": launches_per_pass * args.steps,
            "clocks": clocks.summary(),
            "wall_s": wall,
        }
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_profile(args):
    """A small bounded run of one engine pass for profiler captures (no JSON line).

    fwd: one batched forward; grad: forward with checkpoints + residual + adjoint
    (recompute and adjoint kernels). Shots and steps are cut to --shots / --nt.
    """
    import torch
    sys.path.insert(0, str(ROOT))
    from soundwavesimulation_gb300.engine import DeviceMedium, FusedPlan, residual_misfit
    from soundwavesimulation_gb300.phantoms import config
    device = torch.device("cuda", 0)
    acq = config(2)[0].subset(n_shots=args.shots, n_steps=args.nt)
    medium = DeviceMedium(acq.c, acq.dx, acq.dx, acq.dt, device)
    waves = torch.as_tensor(acq.wavelet[None], dtype=torch.float32, device=device)
    tuning = json.loads(args.tuning) if args.tuning else {}
    plan = FusedPlan(medium, acq.ring.receiver_taps(), acq.source_tables(), waves, acq.n_steps,
                     tuning=tuning, for_gradient=args.profile == "grad")
    grad = args.profile == "grad"
    times = []
    for _ in range(2):  # the second pass is timed
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        traces = plan.forward(save_checkpoints=grad)
        ev[1].record()
        if grad:
            res, _ = residual_misfit(traces, torch.zeros_like(traces), None)
            g = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=device)
            plan.adjoint(res, g)
        ev[2].record()
        torch.cuda.synchronize()
        times = [ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])]
    print(f"profile {args.profile}: {acq.n_shots} shots, {acq.n_steps} steps, tuning {plan.tuning}; "
          f"forward {times[0]:.2f} ms" + (f", residual+adjoint {times[1]:.2f} ms" if grad else ""))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", choices=["fwd", "grad"], default=None,
                    help="run one small engine pass for a profiler instead of the benchmark")
    ap.add_argument("--shots", type=int, default=64)
    ap.add_argument("--nt", type=int, default=36)
    ap.add_argument("--tuning", default="", help="JSON engine tuning for --profile")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
