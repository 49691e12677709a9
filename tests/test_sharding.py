"""Shot sharding and the gradient all-reduce on two gloo ranks (CPU, no GPU).

Each rank computes the oracle's float64 misfit and gradient for its shard of
shots; after the all-reduce both ranks must hold the full-acquisition sums.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from soundwavesimulation_gb300.sharding import (allreduce_misfit_and_gradient, shard_range,
                                                shard_sources)


@pytest.mark.parametrize("n,world", [(7, 2), (128, 2), (128, 8), (3, 4), (256, 3)])
def test_shard_ranges_partition(n, world):
    ranges = [shard_range(n, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
    sizes = [e - b for b, e in ranges]
    assert max(sizes) - min(sizes) <= 1
    assert np.array_equal(np.concatenate([shard_sources(np.arange(n), r, world) for r in range(world)]),
                          np.arange(n))


def _problem():
    from oracle import fdtd_oracle as orc
    n, dx, nt = 40, 1.0e-3, 120
    x = orc.axis_centers(n, dx)
    xx, yy = np.meshgrid(x, x, indexing="xy")
    c_true = np.where(xx ** 2 + yy ** 2 < 0.006 ** 2, 1650.0, 1500.0)
    c0 = np.full((n, n), 1500.0)
    dt = orc.stable_dt(2000.0, dx, dx, 0.4)
    geo = orc.ring_geometry(6, 0.015, x, x)
    wav = np.sin(2 * np.pi * 1.5e5 * np.arange(nt) * dt) * np.exp(-((np.arange(nt) * dt - 1e-5) / 4e-6) ** 2)
    src = orc.point_sources((n, n), geo["rows"], geo["cols"])
    obs, _, _, _ = orc.simulate_shots_batch(c_true, dx, dx, dt, geo, src, wav, nt)
    return orc, c0, dx, dt, geo, src, wav, nt, obs


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        orc, c0, dx, dt, geo, src, wav, nt, obs = _problem()
        mine = shard_sources(np.arange(6), rank, world)
        J, g = orc.misfit_and_gradient_c2(c0, dx, dx, dt, geo, src[mine], wav, nt, obs[mine], mine)
        J, gt = allreduce_misfit_and_gradient(J, torch.as_tensor(g))
        out[rank] = (J, gt.numpy())
    finally:
        dist.destroy_process_group()


def test_gradient_allreduce_two_gloo_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    orc, c0, dx, dt, geo, src, wav, nt, obs = _problem()
    J_full, g_full = orc.misfit_and_gradient_c2(c0, dx, dx, dt, geo, src, wav, nt, obs, np.arange(6))
    for r in range(2):
        J, g = out[r]
        assert J == pytest.approx(J_full, rel=1e-12)
        np.testing.assert_allclose(g, g_full, rtol=1e-10, atol=1e-12 * np.abs(g_full).max())
