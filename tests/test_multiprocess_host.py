"""Multi-process QJMC sharding on CPU (gloo, world size 2): trajectory blocks
per rank, one host-side reduction of the trajectory-summed observables and a
gather of the jump counts.  The per-rank trajectory runner is a host-only
stand-in with a closed-form result per trajectory, so no GPU is needed."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import tngpu as tn


def _fake_run(st, psi, H, jumpops, tmax, dt, obs, ntraj, draws=None, **kw):
    # per-trajectory "observable" rows = a function of that trajectory's draws
    rows = 3
    vals = np.stack([np.outer(np.arange(1, rows + 1), d[:4]) * (1 + 1j) for d in draws])
    nj = (draws[:, 0] * 10).astype(np.int32)
    return [0.0, 0.1, 0.2], vals.mean(axis=0), nj


def _fake_run_seeded(st, psi, H, jumpops, tmax, dt, obs, ntraj, seed=None, first_traj=0, **kw):
    draws = np.stack([tn.philox_uniforms(seed, first_traj + t, 9) for t in range(ntraj)])
    return _fake_run(st, psi, H, jumpops, tmax, dt, obs, ntraj, draws=draws)


def _worker_seeded(rank, world, port, ntraj, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times, avg, nj = tn.qjmc_ensemble_sharded(None, None, None, None, 0.2, 0.1, None, ntraj,
                                                  seed=4, run=_fake_run_seeded)
        if rank == 0:
            out.put((avg, nj))
    finally:
        dist.destroy_process_group()


def _worker(rank, world, port, draws, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times, avg, nj = tn.qjmc_ensemble_sharded(None, None, None, None, 0.2, 0.1, None,
                                                  draws.shape[0], draws, run=_fake_run)
        if rank == 0:
            out.put((avg, nj))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("ntraj", [7, 8])
def test_qjmc_sharded_matches_single_process(ntraj):
    draws = np.random.default_rng(ntraj).random((ntraj, 9))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, draws, q)) for r in range(2)]
    for p in procs:
        p.start()
    avg, nj = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, ref_avg, ref_nj = _fake_run(None, None, None, None, 0, 0, None, ntraj, draws=draws)
    assert np.allclose(avg, ref_avg, rtol=1e-14, atol=1e-14)
    assert nj.tolist() == ref_nj.tolist()


def test_shard_range_covers_all():
    for n in (1, 5, 16, 1024):
        for w in (1, 2, 3, 8):
            blocks = [tn.shard_range(n, r, w) for r in range(w)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(blocks[i][1] == blocks[i + 1][0] for i in range(w - 1))
            assert max(b - a for a, b in blocks) - min(b - a for a, b in blocks) <= 1


@pytest.mark.parametrize("ntraj", [5, 8])
def test_qjmc_sharded_seeded_streams_match_single_process(ntraj):
    """With a seed every rank draws trajectory t's own stream, so the
    sharded ensemble is the single-process one."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_seeded, args=(r, 2, port, ntraj, q)) for r in range(2)]
    for p in procs:
        p.start()
    avg, nj = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, ref_avg, ref_nj = _fake_run_seeded(None, None, None, None, 0, 0, None, ntraj, seed=4)
    assert np.allclose(avg, ref_avg, rtol=1e-14, atol=1e-14)
    assert nj.tolist() == ref_nj.tolist()
