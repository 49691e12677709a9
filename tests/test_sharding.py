"""Shot sharding and the gradient all-reduce on two gloo ranks (CPU, no GPU).

Each rank computes the oracle's float64 misfit and gradient for its shard of
shots; after the all-reduce both ranks must hold the full-acquisition sums.
``sharded_misfit_and_grad`` itself runs on the ranks over a stand-in problem
whose per-shard gradient is the oracle's (the GPU engine is not needed for the
sharding and reduction logic).
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from soundwavesimulation_gb300.sharding import (allreduce_misfit_and_gradient, shard_range,
                                                shard_sources, sharded_misfit_and_grad)


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


class _OracleProblem:
    """The part of TorchLeastSquaresFWI that sharded_misfit_and_grad uses, with
    the oracle's float64 gradient standing in for the device engine."""

    def __init__(self):
        from oracle import fdtd_oracle as orc
        self.orc = orc
        (_, self.c0, self.dx, self.dt, self.geo, self.src, self.wav, self.nt, self.obs) = _problem()
        n = self.c0.shape[0]
        x = orc.axis_centers(n, self.dx)
        self.mask = orc.interior_mask(x, x, 0.015, 2 * self.dx)
        self.model = type("Model", (), {"device": torch.device("cpu"), "shape": self.c0.shape})()
        self.alpha = 1.0e9

    def project(self, m):
        out = np.clip(np.asarray(m, float), 1.0 / 2000.0 ** 2, 1.0 / 1400.0 ** 2)
        out[~self.mask] = 1.0 / 1500.0 ** 2
        return out

    def _sample_sources(self):
        return np.arange(6)

    def gradient_c2(self, m, shots):
        shots = np.asarray(shots)
        return self.orc.misfit_and_gradient_c2(1.0 / np.sqrt(m), self.dx, self.dx, self.dt, self.geo,
                                               self.src[shots], self.wav, self.nt, self.obs[shots], shots)

    def regularization(self, m):
        return self.orc.tikhonov(m, self.mask, self.alpha)


def _m_start(problem):
    rng = np.random.default_rng(5)
    m = 1.0 / problem.c0 ** 2
    return m * (1.0 + 0.01 * rng.standard_normal(m.shape))


def _sharded_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        problem = _OracleProblem()
        out[rank] = sharded_misfit_and_grad(problem, _m_start(problem))
    finally:
        dist.destroy_process_group()


def test_sharded_misfit_and_grad_two_gloo_ranks():
    """The product's distributed objective on 2 ranks equals the one-rank result."""
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    problem = _OracleProblem()
    J_one, g_one = sharded_misfit_and_grad(problem, _m_start(problem))  # no process group: one rank
    assert np.any(g_one != 0.0) and np.all(g_one[~problem.mask] == 0.0)
    for r in range(2):
        J, g = out[r]
        assert J == pytest.approx(J_one, rel=1e-12)
        np.testing.assert_allclose(g, g_one, rtol=1e-10, atol=1e-12 * np.abs(g_one).max())
