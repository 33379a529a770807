"""GPU parity: every call goes through libtngpu.so's C ABI and is compared
with the CPU oracle on the same seeded inputs.

Tolerances (FP64 path): unit contractions 1e-12 relative; energies 1e-10
relative; local observables and singular values 1e-9 absolute; kept bond
dimensions and jump records identical."""

import ctypes as C

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def crand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def f(a):
    return np.asfortranarray(a.astype(np.complex128))


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


# ---------------------------------------------------------------------------
# unit-level kernels
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("cl,cr,wl,wm,wr", [(1, 4, 1, 5, 5), (7, 13, 5, 5, 5), (33, 17, 3, 3, 3),
                                            (64, 64, 5, 5, 1), (130, 96, 4, 6, 5)])
def test_heff2_unit(tn, cl, cr, wl, wm, wr):
    ctx = tn.context()
    rng = np.random.default_rng(cl * 1000 + cr)
    d = 2
    L, W1, W2 = f(crand(rng, cl, wl, cl)), f(crand(rng, wl, d, d, wm)), f(crand(rng, wm, d, d, wr))
    R, th = f(crand(rng, cr, wr, cr)), f(crand(rng, cl, d, d, cr))
    out = np.zeros((cl, d, d, cr), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_heff2_apply(ctx.h, cl, cr, d, wl, wm, wr, dp(L), dp(W1), dp(W2), dp(R),
                                     dp(th), dp(out), 0))
    assert rel(out, O.core.heff2(L, W1, W2, R, th)) < 1e-12


@pytest.mark.parametrize("cl,cr,wl,wr", [(1, 2, 1, 5), (9, 17, 5, 5), (64, 32, 3, 3), (100, 128, 5, 1)])
def test_env_updates_unit(tn, cl, cr, wl, wr):
    ctx = tn.context()
    rng = np.random.default_rng(7 + cl)
    d = 2
    A, W = f(crand(rng, cl, d, cr)), f(crand(rng, wl, d, d, wr))
    L, R = f(crand(rng, cl, wl, cl)), f(crand(rng, cr, wr, cr))
    outl = np.zeros((cr, wr, cr), dtype=np.complex128, order="F")
    outr = np.zeros((cl, wl, cl), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_env_left(ctx.h, cl, cr, d, wl, wr, dp(L), dp(A), dp(W), dp(outl), 0))
    ctx.check(ctx.lib.tn_env_right(ctx.h, cl, cr, d, wl, wr, dp(R), dp(A), dp(W), dp(outr), 0))
    assert rel(outl, O.core.env_left(L, A, W, A)) < 1e-12
    assert rel(outr, O.core.env_right(R, A, W, A)) < 1e-12


@pytest.mark.parametrize("cl,cm,cr", [(1, 2, 4), (16, 31, 8), (128, 128, 128)])
def test_gate2_unit(tn, cl, cm, cr):
    ctx = tn.context()
    rng = np.random.default_rng(cm)
    d = 2
    A1, A2, G = f(crand(rng, cl, d, cm)), f(crand(rng, cm, d, cr)), f(crand(rng, d, d, d, d))
    out = np.zeros((cl, d, d, cr), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_gate2_apply(ctx.h, cl, cm, cr, d, dp(A1), dp(A2), dp(G), dp(out)))
    th = np.tensordot(A1, A2, axes=([2], [0]))
    ref = np.einsum("aijb,piqj->apqb", th, G)
    assert rel(out, ref) < 1e-12


def _matrix_with_spectrum(rng, m, n, S):
    U, _ = np.linalg.qr(crand(rng, m, m))
    V, _ = np.linalg.qr(crand(rng, n, n))
    k = len(S)
    return f(U[:, :k] @ np.diag(S) @ V[:, :k].conj().T)


@pytest.mark.parametrize("direction", [0, 1])
@pytest.mark.parametrize("case", [
    dict(S=[1, 0.5, 1e-3, 1e-6, 0.0], cutoff=1e-8, maxdim=0, mindim=1),
    dict(S=[1, 0.5, 1e-3, 1e-6, 0.0], cutoff=0.0, maxdim=0, mindim=1),
    dict(S=[1, 0.5, 1e-3, 1e-6, 0.0], cutoff=1e-13, maxdim=2, mindim=1),
    dict(S=[1, 0.5, 1e-3, 1e-6, 0.0], cutoff=0.9, maxdim=0, mindim=3),
    dict(S=list(np.geomspace(1, 1e-7, 40)), cutoff=1e-10, maxdim=0, mindim=1),
    # fewer kept vectors than the Gram order: top-eigenpair solver, weight
    # below the computed eigenvalues from the Gram trace
    dict(S=list(np.geomspace(1, 1e-9, 200)), cutoff=1e-14, maxdim=120, mindim=1),
    dict(S=list(np.geomspace(1, 1e-9, 200)), cutoff=1e-10, maxdim=150, mindim=1),
    dict(S=list(np.geomspace(1, 1e-9, 200)), cutoff=0.0, maxdim=50, mindim=80),
])
def test_truncate_keep_rule_and_factors(tn, case, direction):
    ctx = tn.context()
    rng = np.random.default_rng(len(case["S"]) + direction)
    m, n = 12, 50
    S = np.asarray(case["S"], dtype=float)
    if S.size > min(m, n):
        m = n = S.size + 3
    M = _matrix_with_spectrum(rng, m, n, S)
    U, So, Vt = O.trunc_svd(M, case["cutoff"], case["maxdim"], case["mindim"])
    k = C.c_int64(min(m, n))
    Xo = np.zeros((m, min(m, n)), dtype=np.complex128, order="F")
    Yo = np.zeros((min(m, n), n), dtype=np.complex128, order="F")
    Sg = np.zeros(min(m, n))
    t = tn._lib.trunc(case["cutoff"], case["maxdim"], case["mindim"])
    ctx.check(ctx.lib.tn_truncate(ctx.h, m, n, dp(M), C.byref(t), direction, dp(Xo), dp(Yo), dp(Sg),
                                  C.byref(k)))
    kk = k.value
    assert kk == So.size
    Xg = np.asfortranarray(Xo.ravel(order="F")[: m * kk].reshape((m, kk), order="F"))
    Yg = np.asfortranarray(Yo.ravel(order="F")[: kk * n].reshape((kk, n), order="F"))
    assert np.allclose(Sg[:kk], So, atol=1e-9)
    assert np.allclose(Xg @ Yg, (U * So) @ Vt, atol=1e-9)
    if direction == 0:
        assert np.allclose(Xg.conj().T @ Xg, np.eye(kk), atol=1e-12)
    else:
        assert np.allclose(Yg @ Yg.conj().T, np.eye(kk), atol=1e-12)


@pytest.mark.parametrize("direction", [0, 1])
@pytest.mark.parametrize("m,n", [(150, 300), (300, 150), (256, 640), (640, 256)])
def test_truncate_rectangular_top_k(tn, m, n, direction):
    """Rectangular splits on the top-eigenpair path: the Gram order is the
    isometric side (m or n) and exceeds the kept count.  The 256 x 640 shapes
    put a Gram product with inner dimension 640 on a grid of 4 x 4 tiles,
    which splits K (partials summed in chunk order)."""
    ctx = tn.context()
    rng = np.random.default_rng(m + 2 * n + direction)
    S = np.geomspace(1, 1e-9, min(m, n))
    M = _matrix_with_spectrum(rng, m, n, S)
    cutoff, maxdim = 1e-12, 60
    U, So, Vt = O.trunc_svd(M, cutoff, maxdim, 1)
    k = C.c_int64(min(m, n))
    Xo = np.zeros((m, min(m, n)), dtype=np.complex128, order="F")
    Yo = np.zeros((min(m, n), n), dtype=np.complex128, order="F")
    Sg = np.zeros(min(m, n))
    t = tn._lib.trunc(cutoff, maxdim, 1)
    ctx.check(ctx.lib.tn_truncate(ctx.h, m, n, dp(M), C.byref(t), direction, dp(Xo), dp(Yo), dp(Sg),
                                  C.byref(k)))
    kk = k.value
    assert kk == So.size == maxdim
    Xg = np.asfortranarray(Xo.ravel(order="F")[: m * kk].reshape((m, kk), order="F"))
    Yg = np.asfortranarray(Yo.ravel(order="F")[: kk * n].reshape((kk, n), order="F"))
    assert np.allclose(Sg[:kk], So, atol=1e-9)
    assert np.allclose(Xg @ Yg, (U * So) @ Vt, atol=1e-9)
    iso = Xg.conj().T @ Xg if direction == 0 else Yg @ Yg.conj().T
    assert np.allclose(iso, np.eye(kk), atol=1e-12)


# ---------------------------------------------------------------------------
# MPS operations
# ---------------------------------------------------------------------------
def _draws(N, D, seed):
    rng = np.random.default_rng(seed)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    out = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    out.append(O.fr(rng.standard_normal(2 * min(2, D)), (1, 2, min(2, D))))
    return out


def test_random_mps_norm_entropy_singular_values(tn):
    N, D = 10, 6
    dr = _draws(N, D, 11)
    po = O.random_mps(2, N, D, dr)
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    assert pg.bonddims() == po.bonddims() and pg.center == po.center == 1
    assert abs(pg.norm() - 1) < 1e-12
    for site in (3, 5, 9):
        assert abs(pg.entropy(site) - po.entropy(site)) < 1e-9
        assert np.allclose(pg.singular_values(site), po.singular_values(site), atol=1e-9)
    # the dense states agree up to a global phase
    vg = X.mps_to_dense(O.GMPS(1, 2, pg.tensors()))
    vo = X.mps_to_dense(po)
    assert abs(abs(np.vdot(vg, vo)) - 1) < 1e-10


def test_device_random_mps_is_canonical(tn):
    N, D = 12, 8
    pg = tn.randomMPS(2, N, D, rng=np.random.default_rng(5))
    assert pg.center == 1 and abs(pg.norm() - 1) < 1e-12
    assert pg.bonddims() == [1, 2, 4, 8, 8, 8, 8, 8, 8, 4, 2, 1, 1][: N + 1] or pg.bonddims()[1] == 2
    ts = pg.tensors()
    for A in ts[1:]:  # right-orthonormal sites 2..N
        M = A.reshape(A.shape[0], -1, order="F")
        assert np.allclose(M @ M.conj().T, np.eye(A.shape[0]), atol=1e-12)


def test_truncating_movecenter_matches(tn):
    N, D = 12, 16
    dr = _draws(N, D, 12)
    po = O.random_mps(2, N, D, dr)
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    po.movecenter(N, cutoff=1e-3, maxdim=5)
    pg.movecenter(N, cutoff=1e-3, maxdim=5)
    assert pg.bonddims() == po.bonddims()
    vg = X.mps_to_dense(O.GMPS(1, 2, pg.tensors()))
    vo = X.mps_to_dense(po)
    assert abs(abs(np.vdot(vg, vo)) / (np.linalg.norm(vg) * np.linalg.norm(vo)) - 1) < 1e-10


def test_inner_terms(tn):
    N = 8
    dr = _draws(N, 4, 13)
    po = O.random_mps(2, N, 4, dr)
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    ops_o, ops_g = O.OpList(N), tn.OpList(N)
    for H in (ops_o, ops_g):
        H.add("z", 3)
        H.add(["x", "y"], [4, 5], 0.5)
        H.add(["z", "z"], [2, 6], -1.5)
        H.add("s+", 8, 2.0)
    got = tn.inner(tn.spinhalf(), pg, ops_g, pg)
    ref = O.inner(O.spinhalf(), po, ops_o, po)
    assert np.allclose(got, ref, atol=1e-12)


# ---------------------------------------------------------------------------
# DMRG: the TFIM workload (N=20, D=4 start, chi<=64, 5 sweeps, Lanczos 8x2)
# ---------------------------------------------------------------------------
def tfim(mod, N, J=1.0, h=0.5):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -J)
    for i in range(1, N + 1):
        H.add("x", i, -h)
    return H


def xxz(mod, N, J=1.0, delta=1.0, field=None):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], J)
        H.add(["y", "y"], [i, i + 1], J)
        H.add(["z", "z"], [i, i + 1], J * delta)
    if field:
        for i in range(1, N + 1):
            H.add("z", i, field(i))
    return H


def test_dmrg_config1_tfim_parity(tn):
    N, D = 20, 4
    dr = _draws(N, D, 1)
    kw = dict(maxdim=64, cutoff=1e-10, minsweeps=5, maxsweeps=5, numconverges=np.inf,
              krylovdim=8, kryloviter=2)
    po = O.random_mps(2, N, D, dr)
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    _, Eo = O.dmrg(po, O.mpo_from_oplist(O.spinhalf(), tfim(O, N)), **kw)
    _, Eg = tn.dmrg(pg, tn.MPO(tn.spinhalf(), tfim(tn, N)), verbose=False, **kw)
    assert abs(Eg - np.real(Eo)) <= 1e-10 * abs(Eo)
    assert pg.bonddims() == po.bonddims()
    Sg, So = pg.singular_values(10), po.singular_values(10)
    assert Sg.shape == So.shape and np.allclose(Sg, So, atol=1e-9)
    # known answer: free-fermion ground energy (ordered phase, 5 sweeps)
    assert abs(Eg - X.tfim_free_fermion_energy(N, 1.0, 0.5)) < 1e-4


def test_dmrg_xxz_parity_small(tn):
    N, D = 16, 8
    dr = _draws(N, D, 2)
    kw = dict(maxdim=32, cutoff=1e-12, minsweeps=4, maxsweeps=4, numconverges=np.inf)
    po = O.random_mps(2, N, D, dr)
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    _, Eo = O.dmrg(po, O.mpo_from_oplist(O.spinhalf(), xxz(O, N)), **kw)
    _, Eg = tn.dmrg(pg, tn.MPO(tn.spinhalf(), xxz(tn, N)), verbose=False, **kw)
    assert abs(Eg - np.real(Eo)) <= 1e-10 * abs(Eo)
    assert pg.bonddims() == po.bonddims()
    z_o, z_g = O.OpList(N), tn.OpList(N)
    for i in range(1, N + 1):
        z_o.add("z", i)
        z_g.add("z", i)
    assert np.allclose(tn.inner(tn.spinhalf(), pg, z_g, pg), O.inner(O.spinhalf(), po, z_o, po), atol=1e-9)


# ---------------------------------------------------------------------------
# TEBD: config 3 shape at reduced N / steps
# ---------------------------------------------------------------------------
def test_tebd_quench_parity(tn):
    N, steps, dt = 16, 12, 0.05
    field = lambda i: 0.2 * (-1) ** i  # noqa: E731
    names = ["up" if i % 2 else "dn" for i in range(1, N + 1)]
    zo, zg = O.OpList(N), tn.OpList(N)
    for i in range(1, N + 1):
        zo.add("z", i)
        zg.add("z", i)
    po = O.product_mps(O.spinhalf(), names)
    rec = {}
    O.tebd(O.spinhalf(), po, xxz(O, N, 1.0, 0.5, field), dt, steps * dt, dt, [zo], cutoff=1e-10,
           maxdim=12, evol="real", record=rec)
    pg = tn.productMPS(tn.spinhalf(), names)
    ob = tn.TEBDOperators(tn.spinhalf(), zg)
    nm = tn.TEBDNorm()
    tn.tebd(tn.spinhalf(), pg, xxz(tn, N, 1.0, 0.5, field), dt, steps * dt, dt, [ob, nm],
            cutoff=1e-10, maxdim=12, evol="real")
    assert len(ob.measurements) == len(rec["ops"]) == steps + 1
    for a, b in zip(ob.measurements, rec["ops"]):
        assert np.allclose(np.real(a), np.real(b[0]), atol=1e-9)
    assert np.allclose(nm.measurements, rec["lognorm"], atol=1e-9)
    assert pg.bonddims() == po.bonddims()
    assert abs(pg.entropy(N // 2) - po.entropy(N // 2)) < 1e-9


def test_tebd_xx_chain_n64_matches_free_fermion_dynamics(tn):
    """The TEBD quench at the N=64 size, against an exact answer: the XX
    chain (delta=0) is free fermions with hopping 2, so <Z_i>(t) from a Neel
    state follows from the single-particle propagator.  Agreement up to the
    second-order Trotter error (4e-5 at N=24 for the same dt and t)."""
    import scipy.linalg as sla
    N, dt, steps = 64, 0.01, 50
    names = ["up" if i % 2 else "dn" for i in range(1, N + 1)]
    zg = tn.OpList(N)
    for i in range(1, N + 1):
        zg.add("z", i)
    pg = tn.productMPS(tn.spinhalf(), names)
    ob = tn.TEBDOperators(tn.spinhalf(), zg)
    tn.tebd(tn.spinhalf(), pg, xxz(tn, N, 1.0, 0.0), dt, steps * dt, steps * dt, [ob],
            cutoff=1e-12, maxdim=64, evol="real")
    z_gpu = np.real(np.asarray(ob.measurements[-1]))
    h = 2.0 * (np.eye(N, k=1) + np.eye(N, k=-1))
    U = sla.expm(-1j * h * steps * dt)
    n0 = np.array([1.0 if i % 2 else 0.0 for i in range(1, N + 1)])
    z_exact = 2.0 * np.real(np.diag(U @ np.diag(n0) @ U.conj().T)) - 1.0
    assert np.max(np.abs(z_gpu - z_exact)) < 2e-4, np.max(np.abs(z_gpu - z_exact))


def test_tebd_imaginary_time_ground_state(tn):
    # evol="imag" applies exp(+dt H) (gatelist.jl:87,100): pass -H to target
    # the ground state, as the reference's users do
    N = 10
    H = (-1.0) * xxz(tn, N)
    pg = tn.productMPS(tn.spinhalf(), ["up" if i % 2 else "dn" for i in range(1, N + 1)])
    _, E = tn.tebd(tn.spinhalf(), pg, H, 0.05, 4.0, 4.0, [], cutoff=1e-12, maxdim=32)
    E_ed = np.linalg.eigvalsh(X.oplist_to_dense(O.spinhalf(), xxz(O, N)))[0]
    assert abs(-E - E_ed) < 5e-3  # Trotter error at dt=0.05


# ---------------------------------------------------------------------------
# QJMC: config 4 shape at reduced N / steps, identical jump records
# ---------------------------------------------------------------------------
def ising_qjmc(mod, N):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
    Lj = mod.OpList(N)
    for i in range(1, N + 1):
        Lj.add("s-", i, np.sqrt(0.1))
    return H, Lj


@pytest.mark.parametrize("fast", [True, False])
def test_qjmc_trajectory_parity(tn, fast):
    N, dt, steps = 8, 0.05, 40
    draws = np.random.default_rng(5).random(3 * steps + 3)  # a stream with two jumps
    Ho, Lo = ising_qjmc(O, N)
    zo = O.OpList(N)
    for i in range(1, N + 1):
        zo.add("z", i)
    po = O.product_mps(O.spinhalf(), ["up"] * N)
    rec = {}
    jo, to = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                               O.algorithms.UniformStream(draws), [zo], cutoff=1e-10, maxdim=16,
                               record=rec)
    Hg, Lg = ising_qjmc(tn, N)
    zg = tn.OpList(N)
    for i in range(1, N + 1):
        zg.add("z", i)
    obs = tn.QJMCOperators(zg, tn.spinhalf())
    observers = [obs] if fast else [obs, tn.QJMCActivity()]
    pg = tn.productMPS(tn.spinhalf(), ["up"] * N)
    jg, tg = tn.qjmc_simulation(tn.spinhalf(), pg, Hg, Lg, steps * dt, dt, observers, cutoff=1e-10,
                                maxdim=16, draws=draws)
    assert jg == jo and len(jg) > 0
    assert np.allclose(tg, to, atol=0)
    assert len(obs.measurements) == len(rec["ops"])
    for a, b in zip(obs.measurements, rec["ops"]):
        assert np.allclose(np.real(a), np.real(b[0]), atol=1e-9)
    assert pg.bonddims() == po.bonddims()


def test_error_status_on_bad_input(tn):
    ctx = tn.context()
    pg = tn.productMPS(tn.spinhalf(), ["up"] * 4)
    with pytest.raises(tn.TNError, match="out of range"):
        pg.movecenter(9)
    # the context stays usable after an error
    pg.movecenter(2)
    assert pg.center == 2


@pytest.mark.parametrize("workers,ntraj", [(3, 6), (8, 12)])
def test_qjmc_ensemble_matches_per_trajectory_oracle(tn, workers, ntraj):
    """Concurrent trajectories (one host worker, stream and solver each)
    against the oracle run trajectory by trajectory on the same draw rows:
    averaged <Z_i>(t) and jump counts."""
    N, dt, steps = 6, 0.05, 30
    draws = np.random.default_rng(9).random((ntraj, 3 * steps + 3))
    Ho, Lo = ising_qjmc(O, N)
    zo = O.OpList(N)
    for i in range(1, N + 1):
        zo.add("z", i)
    avg, counts = 0.0, []
    for t in range(ntraj):
        po = O.product_mps(O.spinhalf(), ["up"] * N)
        rec = {}
        j, _ = O.qjmc_simulation(O.spinhalf(), po, Ho, Lo, steps * dt, dt,
                                 O.algorithms.UniformStream(draws[t]), [zo], save=5 * dt,
                                 cutoff=1e-10, maxdim=16, record=rec)
        avg = avg + np.real(np.array([r[0] for r in rec["ops"]]))
        counts.append(len(j))
    avg /= ntraj
    Hg, Lg = ising_qjmc(tn, N)
    zg = tn.OpList(N)
    for i in range(1, N + 1):
        zg.add("z", i)
    pg = tn.productMPS(tn.spinhalf(), ["up"] * N)
    times, out, nj = tn.qjmc_ensemble(tn.spinhalf(), pg, Hg, Lg, steps * dt, dt, zg, ntraj,
                                      draws=draws, save=5 * dt, cutoff=1e-10, maxdim=16,
                                      workers=workers, engine="workers")
    assert list(nj) == counts and sum(counts) > 0
    assert out.shape == avg.shape and np.allclose(np.real(out), avg, atol=1e-9)
    assert len(times) == out.shape[0]
