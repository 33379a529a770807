"""Seeded QJMC ensembles (tn_qjmc_batch and tn_qjmc_ensemble with draws == NULL): trajectory t
draws from its own Philox4x32-10 stream, so the ensemble equals the one run
from the same streams passed explicitly (the parity mode), and a block of
trajectories started at first_traj equals the matching rows of the full
ensemble (what a sharded rank runs)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(tn, N):
    H, Lj, Z = tn.OpList(N), tn.OpList(N), tn.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
        Lj.add("s-", i, np.sqrt(0.1))
        Z.add("z", i)
    return H, Lj, Z


@pytest.mark.parametrize("engine", ["workers", "device"])
def test_seeded_ensemble_matches_explicit_streams(engine):
    import tngpu as tn
    N, dt, steps, ntraj = 8, 0.05, 30, 6
    H, Lj, Z = _model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    kw = dict(cutoff=1e-10, maxdim=16, workers=3, engine=engine)
    _, za, na = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, seed=11, **kw)
    draws = np.stack([tn.philox_uniforms(11, t, 3 * steps + 3) for t in range(ntraj)])
    _, zb, nb = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, draws=draws, **kw)
    assert na.tolist() == nb.tolist() and na.sum() > 0
    assert np.allclose(za, zb, atol=1e-12)
    # trajectories 2..5 as one rank of a sharded run would draw them
    _, zc, nc = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 4, seed=11, first_traj=2, **kw)
    assert nc.tolist() == na[2:].tolist()
    _, zd, _ = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 4, draws=draws[2:], **kw)
    assert np.allclose(zc, zd, atol=1e-12)
