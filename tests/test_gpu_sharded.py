"""Sharded QJMC with the real trajectory engine: two ranks (gloo, world size
2, processes on the one GPU of the test) each run their block of seeded
trajectories through tn_qjmc_ensemble and combine the trajectory-summed
observables and jump counts on the host; the result equals one process
running all trajectories.  The ranks meet only in host collectives, so their
kernels never wait on each other."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

N, DT, STEPS, NTRAJ, SEED = 8, 0.05, 20, 10, 77


def _model(tn):
    H, Lj, Z = tn.OpList(N), tn.OpList(N), tn.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
        Lj.add("s-", i, np.sqrt(0.5))
        Z.add("z", i)
    return H, Lj, Z


def _run(tn, sharded):
    H, Lj, Z = _model(tn)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    kw = dict(cutoff=1e-10, maxdim=16, engine="device")
    if sharded:
        return tn.qjmc_ensemble_sharded(st, psi, H, Lj, STEPS * DT, DT, Z, NTRAJ, seed=SEED, **kw)
    return tn.qjmc_ensemble(st, psi, H, Lj, STEPS * DT, DT, Z, NTRAJ, seed=SEED, **kw)


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import tngpu as tn
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, avg, nj = _run(tn, True)
        if rank == 0:
            out.put((avg, nj))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_engine_matches_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    avg, nj = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    import tngpu as tn
    _, ref_avg, ref_nj = _run(tn, False)
    assert nj.tolist() == ref_nj.tolist() and ref_nj.sum() > 0
    assert np.allclose(avg, ref_avg, rtol=0, atol=1e-12)
