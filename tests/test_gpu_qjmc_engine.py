"""The persistent trajectory engine (tn_qjmc_ensemble): every block of one
launch runs whole quantum-jump trajectories (qjmc.jl:28-220) on the device.

  * Against the oracle's qjmc_simulation run trajectory by trajectory on the
    same explicit uniform streams: identical jump channels and times in
    every trajectory, and the trajectory-averaged <Z_i>(t) to 1e-9 (chains
    with an even and an odd number of sites: the odd one puts one-site gates
    at the chain's end).
  * Against the host-worker engine (tn_qjmc_batch) on the same seeded
    streams: identical jump counts, averaged <Z_i>(t) to 1e-9.
  * The launch width (blocks per SM) does not change any trajectory.
  * A draw stream that runs out is reported as an error status.
  * Bonds wider than the block's thread count (Gram order 160) still match
    the oracle."""

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def _model(mod, N, g=0.5, h=0.8):
    H, Lj, Z = mod.OpList(N), mod.OpList(N), mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, h)
        Lj.add("s-", i, np.sqrt(g))
        Z.add("z", i)
    return H, Lj, Z


@pytest.mark.parametrize("N", [6, 7])
def test_engine_jump_records_match_oracle(tn, N):
    dt, steps, ntraj, every = 0.05, 30, 8, 5
    draws = np.random.default_rng(40 + N).random((ntraj, 3 * steps + 3))
    Ho, Lo, Zo = _model(O, N)
    avg, jumps, times = 0.0, [], []
    for t in range(ntraj):
        po = O.product_mps(O.spinhalf(), ["up"] * N)
        rec = {}
        j, jt = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                                  O.algorithms.UniformStream(draws[t]), [Zo], save=every * dt,
                                  cutoff=1e-10, maxdim=16, record=rec)
        avg = avg + np.real(np.array([r[0] for r in rec["ops"]]))
        jumps.append(list(j))
        times.append(list(jt))
    avg /= ntraj
    Hg, Lg, Zg = _model(tn, N)
    st = tn.spinhalf()
    pg = tn.productMPS(st, ["up"] * N)
    tg, out, nj, jg, jtg = tn.qjmc_ensemble(st, pg, Hg, Lg, steps * dt, dt, Zg, ntraj, draws=draws,
                                            save=every * dt, cutoff=1e-10, maxdim=16,
                                            engine="device", records=True)
    assert sum(len(j) for j in jumps) > ntraj  # the stream exercises the jump branch
    assert [list(map(int, j)) for j in jg] == jumps
    for a, b in zip(jtg, times):
        assert np.allclose(a, b, rtol=0, atol=1e-12)
    assert list(nj) == [len(j) for j in jumps]
    assert out.shape == avg.shape and np.allclose(np.real(out), avg, atol=1e-9)
    assert len(tg) == out.shape[0]


def test_engine_matches_worker_engine_seeded(tn):
    N, dt, steps, ntraj = 10, 0.02, 60, 16
    H, Lj, Z = _model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    kw = dict(cutoff=1e-10, maxdim=32, seed=5, save=10 * dt)
    _, za, na = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, engine="workers",
                                 workers=8, **kw)
    _, zb, nb = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, engine="device", **kw)
    assert na.tolist() == nb.tolist() and na.sum() > 0
    assert np.allclose(za, zb, atol=1e-9)


def test_engine_launch_width_invariance(tn):
    N, dt, steps, ntraj = 8, 0.05, 20, 12
    H, Lj, Z = _model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    res = [tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, seed=3, cutoff=1e-10,
                            maxdim=16, engine="device", blocks_per_sm=b, records=True)
           for b in (1, 4)]
    assert np.array_equal(res[0][1], res[1][1])
    assert res[0][3] == res[1][3] and res[0][4] == res[1][4]


def test_engine_reports_an_exhausted_stream(tn):
    N, dt, steps = 6, 0.05, 10
    H, Lj, Z = _model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    draws = np.full((2, 5), 0.5)  # two per step are needed: the third step runs out
    with pytest.raises(tn.TNError, match="exhausted"):
        tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 2, draws=draws, cutoff=1e-10,
                         maxdim=16, engine="device")
    with pytest.raises(ValueError, match="maxdim"):
        tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 2, draws=draws, cutoff=1e-10,
                         maxdim=0, engine="device")


def test_engine_wide_bonds_match_oracle(tn):
    """Gram orders above the block's thread count (bond dimension 80: n = 160
    rows of the tridiagonal reduction, several row passes per step) from a
    random N=14 MPS: jump records and <Z_i> against the oracle."""
    N, dt, steps, ntraj, D = 14, 0.05, 3, 3, 80
    draws = np.random.default_rng(90).random((ntraj, 3 * steps + 3))
    Ho, Lo, Zo = _model(O, N, g=2.0)
    po0 = O.random_mps(2, N, D, np.random.default_rng(91))
    avg, jumps = 0.0, []
    for t in range(ntraj):
        po = po0.copy()
        rec = {}
        j, _ = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                                 O.algorithms.UniformStream(draws[t]), [Zo], save=dt,
                                 cutoff=1e-12, maxdim=D, record=rec)
        avg = avg + np.real(np.array([r[0] for r in rec["ops"]]))
        jumps.append(list(j))
    avg /= ntraj
    Hg, Lg, Zg = _model(tn, N, g=2.0)
    st = tn.spinhalf()
    pg = tn.GMPS.from_tensors(po0.tensors, po0.center)
    assert max(pg.bonddims()) > 64
    _, out, nj, jg, _ = tn.qjmc_ensemble(st, pg, Hg, Lg, steps * dt, dt, Zg, ntraj, draws=draws,
                                         save=dt, cutoff=1e-12, maxdim=D, engine="device",
                                         records=True)
    assert [list(map(int, j)) for j in jg] == jumps
    assert np.allclose(np.real(out), avg, atol=1e-9)


def test_norm_based_unraveling_matches_oracle(tn):
    """classical=false (qjmc.jl:65-86): the jump decision compares the
    step's first draw with the squared norm of the unnormalised state.  The
    single-trajectory driver and the engine both give the oracle's jump
    records on the same streams."""
    N, dt, steps, ntraj = 6, 0.05, 30, 6
    draws = np.random.default_rng(77).random((ntraj, 3 * steps + 3))
    Ho, Lo, _ = _model(O, N)
    ref = []
    for t in range(ntraj):
        po = O.product_mps(O.spinhalf(), ["up"] * N)
        j, jt = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                                  O.algorithms.UniformStream(draws[t]), cutoff=1e-10, maxdim=16,
                                  classical=False)
        ref.append((list(j), list(jt)))
    assert sum(len(j) for j, _ in ref) > ntraj
    Hg, Lg, Zg = _model(tn, N)
    st = tn.spinhalf()
    for t in range(2):
        pg = tn.productMPS(st, ["up"] * N)
        j, jt = tn.qjmc_simulation(st, pg, Hg, Lg, steps * dt, dt, cutoff=1e-10, maxdim=16,
                                   classical=False, draws=draws[t])
        assert j == ref[t][0] and np.allclose(jt, ref[t][1], rtol=0, atol=1e-12)
    pg = tn.productMPS(st, ["up"] * N)
    _, _, _, jg, jtg = tn.qjmc_ensemble(st, pg, Hg, Lg, steps * dt, dt, Zg, ntraj, draws=draws,
                                        cutoff=1e-10, maxdim=16, engine="device", records=True,
                                        classical=False)
    assert [list(map(int, j)) for j in jg] == [j for j, _ in ref]


def test_engine_autotuned_width(tn, tmp_path):
    """blocks_per_sm="auto": on a cache miss the autotuner times the first
    steps of the ensemble at every width (the engine's CUDA-event launch
    time per trajectory-step) and keeps the fastest for the workload's
    bucket; the run gives the trajectories of any fixed width; a second call
    takes the width from the cache without probing."""
    N, dt, steps, ntraj = 8, 0.05, 20, 40
    H, Lj, Z = _model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N)
    kw = dict(seed=3, cutoff=1e-10, maxdim=16, engine="device", records=True)
    path = str(tmp_path / "widths.json")
    s = {}
    ra = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, blocks_per_sm="auto",
                          tune_cache=path, stats=s, **kw)
    timings = s["tune_seconds_per_traj_step"]
    print("probe seconds per trajectory-step:", timings, "->", s["blocks_per_sm"])
    assert s["tune_key"] == tn.autotune.bucket(16, 2, ntraj, N)
    assert sorted(timings) == [1, 2, 4, 8] and all(t > 0 for t in timings.values())
    assert s["blocks_per_sm"] == min(timings, key=lambda w: (timings[w], w))
    rb = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, blocks_per_sm=1, **kw)
    assert np.array_equal(ra[1], rb[1]) and ra[3] == rb[3] and ra[4] == rb[4]
    s2 = {}
    tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, blocks_per_sm="auto",
                     tune_cache=path, stats=s2, **kw)
    assert s2["tune_seconds_per_traj_step"] == {} and s2["blocks_per_sm"] == s["blocks_per_sm"]
    # the bench's form: the tuner on its own, with qjmc_ensemble's keywords
    w, t, key = tn.tune_qjmc_width(st, psi, H, Lj, dt, Z, ntraj, cache=path, seed=3,
                                   cutoff=1e-10, maxdim=16, save=10 * dt)
    assert (w, t, key) == (s["blocks_per_sm"], {}, s["tune_key"])
