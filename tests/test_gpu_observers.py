"""Parity of the device randomMPS procedure and of the TEBDEnergy and
QJMCEntropy observers against the oracle, through the C ABI.

randomGMPS (gmps.jl:276-291) canonicalises the random network, then replaces
site 1 by fresh draws.  The replacement contracts those draws with the bond-1
basis of sites 2..N, and an SVD fixes that basis only up to one sign (one
unitary inside a degenerate singular subspace) per vector, so two correct
implementations give different dense states from the same draws.  The test
therefore compares what the procedure determines: the canonicalised state
before the replacement (dense, exactly), the span of the bond-1 basis, the
bond-1 spectrum of the final state (the draws' singular values) and the bond
dimensions."""

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def _draws(N, D, seed):
    rng = np.random.default_rng(seed)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    out = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    out.append(O.fr(rng.standard_normal(2 * min(2, D)), (1, 2, min(2, D))))
    return out


def _right_block(tensors):
    """Dense matrix B[k, (s2 .. sN)] of sites 2..N with the bond-1 index k."""
    B = tensors[1]
    acc = B.reshape(B.shape[0], -1, order="F")  # [k, (s2, D2)]
    for A in tensors[2:]:
        Dl = A.shape[0]
        acc = acc.reshape(acc.shape[0], -1, Dl, order="F")  # [k, phys, Dl]
        acc = np.einsum("kpl,lsr->kpsr", acc, A).reshape(acc.shape[0], -1, A.shape[2], order="F")
        acc = acc.reshape(acc.shape[0], -1, order="F")
    return acc


@pytest.mark.parametrize("N,D,seed", [(6, 3, 1), (9, 4, 2), (8, 6, 7)])
def test_device_random_mps_matches_oracle_procedure(tn, N, D, seed):
    dr = _draws(N, D, seed)
    po = O.random_mps(2, N, D, dr)
    pg = tn.randomMPS(2, N, D, draws=dr)
    assert pg.bonddims() == po.bonddims() and pg.center == po.center == 1
    assert abs(pg.norm() - 1) < 1e-12
    # the canonicalised random network before site 1 is replaced: gauge free
    cg = tn.GMPS.from_tensors(dr[:N], 0)
    cg.movecenter(N)
    cg.movecenter(1)
    co = O.GMPS(1, 2, [np.asarray(t, dtype=np.complex128) for t in dr[:N]], 0)
    co.movecenter(N)
    co.movecenter(1)
    vg, vo = X.mps_to_dense(O.GMPS(1, 2, cg.tensors())), X.mps_to_dense(co)
    assert np.linalg.norm(vg - vo) <= 1e-12 * np.linalg.norm(vo)
    # sites 2..N of the final states span the same bond-1 space: B_g = U B_o
    tg, to = pg.tensors(), po.tensors
    Bg, Bo = _right_block(tg), _right_block(to)
    k = Bg.shape[0]
    assert np.allclose(Bg @ Bg.conj().T, np.eye(k), atol=1e-12)
    U = Bg @ Bo.conj().T
    assert np.allclose(U @ U.conj().T, np.eye(k), atol=1e-11)
    # bond-1 spectrum of the final state = singular values of the drawn site
    Sd = np.linalg.svd(dr[N].reshape(2, -1, order="F"), compute_uv=False)
    Sd = Sd / np.linalg.norm(Sd)
    assert np.allclose(pg.singular_values(1), Sd, atol=1e-12)
    assert np.allclose(po.singular_values(1), Sd, atol=1e-12)


def _xxz(mod, N, delta=0.5):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], 1.0)
        H.add(["y", "y"], [i, i + 1], 1.0)
        H.add(["z", "z"], [i, i + 1], delta)
    for i in range(1, N + 1):
        H.add("z", i, 0.3 * (-1) ** i)
    return H


def test_tebd_energy_observer_matches_oracle(tn):
    """TEBDEnergy (tebd.jl:168-193): the energy <psi|H|psi> recorded at every
    save of an imaginary-time run (gates exp(+dt H)) from a Neel state, and
    its convergence test on those records."""
    N, dt, steps = 12, 0.05, 24
    names = ["up" if i % 2 else "dn" for i in range(1, N + 1)]
    po = O.product_mps(O.spinhalf(), names)
    rec = {}
    O.tebd(O.spinhalf(), po, _xxz(O, N), dt, steps * dt, 2 * dt, [], cutoff=1e-10, maxdim=16,
           evol="imag", record=rec)
    pg = tn.productMPS(tn.spinhalf(), names)
    ob = tn.TEBDEnergy(tol=1e-12)
    _, E = tn.tebd(tn.spinhalf(), pg, _xxz(tn, N), dt, steps * dt, 2 * dt, [ob], cutoff=1e-10,
                   maxdim=16, evol="imag")
    assert len(ob.measurements) == len(rec["energy"]) == steps // 2 + 1
    assert np.allclose(ob.times, rec["times"], atol=1e-15)
    assert np.allclose(ob.measurements, rec["energy"], rtol=1e-10, atol=1e-10)
    assert abs(E - rec["energy"][-1]) <= 1e-10 * abs(E)
    # evol="imag" gates are exp(+dt H) (gatelist.jl:87, tensors.jl:319-334): <H> rises
    assert ob.measurements[-1] > ob.measurements[0]
    assert not ob.checkdone()  # far from converged at tol 1e-12
    loose = tn.TEBDEnergy(tol=1.0)
    for t, e in zip(ob.times, ob.measurements):
        loose.measure(t, None, 0.0, e)
    assert loose.checkdone()


def test_qjmc_entropy_observer_matches_oracle(tn):
    """QJMCEntropy (qjmc.jl:293-310): entropies at every bond at every save of
    one trajectory.  Each entropy moves the centre, so the trajectory after a
    measurement depends on it; the jump record must still be identical."""
    N, dt, steps = 8, 0.05, 30
    draws = np.random.default_rng(5).random(3 * steps + 3)

    def ising(mod):
        H, L = mod.OpList(N), mod.OpList(N)
        for i in range(1, N):
            H.add(["z", "z"], [i, i + 1], 1.0)
        for i in range(1, N + 1):
            H.add("x", i, 0.8)
            L.add("s-", i, np.sqrt(0.1))
        return H, L

    Ho, Lo = ising(O)
    po = O.product_mps(O.spinhalf(), ["up"] * N)
    rec = {}
    jo, to = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                               O.algorithms.UniformStream(draws), [], save=3 * dt, cutoff=1e-10,
                               maxdim=16, record=rec, entropies=True)
    Hg, Lg = ising(tn)
    ent = tn.QJMCEntropy()
    pg = tn.productMPS(tn.spinhalf(), ["up"] * N)
    jg, tg = tn.qjmc_simulation(tn.spinhalf(), pg, Hg, Lg, steps * dt, dt, [ent], save=3 * dt,
                                cutoff=1e-10, maxdim=16, draws=draws)
    assert jg == jo and len(jg) > 0
    assert np.allclose(tg, to, atol=0)
    assert len(ent.measurements) == len(rec["entropy"]) == steps // 3 + 1
    assert np.allclose(ent.times, rec["times"], atol=1e-15)
    for a, b in zip(ent.measurements, rec["entropy"]):
        assert len(a) == N - 1
        assert np.allclose(a, b, atol=1e-9)
    assert max(max(m) for m in ent.measurements) > 1e-3  # the trajectory entangles
    assert pg.bonddims() == po.bonddims()
