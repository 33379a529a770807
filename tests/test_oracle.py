"""Pins the CPU oracle against known-answer physics (the reference ships no
golden vectors: test/runtests.jl is an empty testset)."""

import json
import os

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def known_answers():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def tfim(N, J=1.0, h=0.5):
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -J)
    for i in range(1, N + 1):
        H.add("x", i, -h)
    return H


def xxz(N, J=1.0, delta=1.0, field=None):
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], J)
        H.add(["y", "y"], [i, i + 1], J)
        H.add(["z", "z"], [i, i + 1], J * delta)
    if field is not None:
        for i in range(1, N + 1):
            H.add("z", i, field(i))
    return H


def test_free_fermion_formula_matches_ed():
    st = O.spinhalf()
    N = 8
    E_ed = np.linalg.eigvalsh(X.oplist_to_dense(st, tfim(N)))[0]
    assert abs(X.tfim_free_fermion_energy(N, 1.0, 0.5) - E_ed) < 1e-11


@pytest.mark.parametrize("which", ["tfim", "xxz", "xxz_field"])
def test_mpo_builder_matches_dense(which):
    st = O.spinhalf()
    N = 6
    H = {"tfim": tfim(N), "xxz": xxz(N), "xxz_field": xxz(N, 1.0, 0.5, lambda i: 0.2 * (-1) ** i)}[which]
    W = O.mpo_from_oplist(st, H)
    dense = X.oplist_to_dense(st, H)
    assert np.allclose(X.mpo_to_dense(W), dense, atol=1e-12)
    w = max(W[i].shape[3] for i in range(1, N))
    assert w == {"tfim": 3, "xxz": 5, "xxz_field": 5}[which]


def test_svd_keep_rule():
    S = np.array([1.0, 0.5, 1e-3, 1e-6, 0.0])
    assert O.svd_keep(S) == 5                     # no cutoff: zeros kept
    assert O.svd_keep(S, maxdim=2) == 2
    assert O.svd_keep(S, cutoff=1e-8) == 3         # tail from 4 holds 1e-12/1.25
    assert O.svd_keep(S, cutoff=1e-13) == 4
    assert O.svd_keep(S, cutoff=0.9) == 1
    assert O.svd_keep(S, cutoff=0.9, mindim=3) == 3
    assert O.svd_keep(np.zeros(3), cutoff=1e-10) == 1
    # a tail weight exactly at the cutoff is discarded: the comparison is
    # strict (tensors.jl:211); equal singular values make the weights exact
    S = np.ones(4)  # tail weights 1, 3/4, 1/2, 1/4
    assert O.svd_keep(S, cutoff=0.5) == 2
    assert O.svd_keep(S, cutoff=0.5 - 2.0 ** -40) == 3
    assert O.svd_keep(S, cutoff=0.25) == 3 and O.svd_keep(S, cutoff=0.2) == 4


def test_lanczos_converges_to_lowest():
    rng = np.random.default_rng(0)
    n = 40
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A + A.conj().T
    x0 = rng.standard_normal(n) + 0j
    e, v = O.lanczos_lowest(lambda x: A @ x, x0, 20, 30)
    assert abs(e - np.linalg.eigvalsh(A)[0]) < 1e-10
    assert np.linalg.norm(A @ v - e * v) < 1e-7


def test_lanczos_invariant_subspace_small_problem():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((4, 4))
    A = A + A.T
    e, v = O.lanczos_lowest(lambda x: A @ x, np.ones(4) + 0j, 8, 2)
    assert abs(e - np.linalg.eigvalsh(A)[0]) < 1e-12


def test_lanczos_matvec_count_matches_krylovkit_schedule():
    rng = np.random.default_rng(2)
    n = 200
    A = np.diag(np.linspace(-1, 1, n)) + 0j
    st = {}
    O.lanczos_lowest(lambda x: A @ x, rng.standard_normal(n) + 0j, 3, 2, stats=st)
    assert st["numops"] == 5        # 3 + (3 - keep=1)
    st = {}
    O.lanczos_lowest(lambda x: A @ x, rng.standard_normal(n) + 0j, 8, 2, stats=st)
    assert st["numops"] == 12       # 8 + (8 - keep=4)


def test_dmrg_tfim_free_fermion():
    st = O.spinhalf()
    N = 12
    W = O.mpo_from_oplist(st, tfim(N))
    psi = O.random_mps(2, N, 4, np.random.default_rng(1))
    psi, E = O.dmrg(psi, W, maxdim=64, cutoff=1e-12, maxsweeps=12, minsweeps=12,
                    numconverges=np.inf, krylovdim=8, kryloviter=2)
    assert abs(np.real(E) - X.tfim_free_fermion_energy(N, 1.0, 0.5)) < 1e-9


def test_dmrg_xxz_ed():
    st = O.spinhalf()
    N = 10
    H = xxz(N)
    W = O.mpo_from_oplist(st, H)
    psi = O.random_mps(2, N, 8, np.random.default_rng(2))
    psi, E = O.dmrg(psi, W, maxdim=64, cutoff=1e-12, maxsweeps=8, minsweeps=8,
                    numconverges=np.inf)
    E_ed = np.linalg.eigvalsh(X.oplist_to_dense(st, H))[0]
    assert abs(np.real(E) - E_ed) < 1e-8
    # energy of the returned state agrees with the Lanczos value
    v = X.mps_to_dense(psi)
    assert abs(X.dense_expect(v, X.oplist_to_dense(st, H)) - E_ed) < 1e-8


def test_random_mps_is_normalised_and_canonical():
    psi = O.random_mps(2, 8, 4, np.random.default_rng(3))
    assert psi.center == 1
    assert abs(np.linalg.norm(X.mps_to_dense(psi)) - 1) < 1e-12
    assert psi.bonddims() == [1, 2, 4, 4, 4, 4, 4, 2, 1]


def test_tebd_untruncated_matches_dense_gates():
    st = O.spinhalf()
    N = 8
    H = xxz(N, 1.0, 0.5, lambda i: 0.2 * (-1) ** i)
    psi = O.product_mps(st, ["up" if i % 2 else "dn" for i in range(1, N + 1)])
    v0 = X.mps_to_dense(psi)
    rows = O.trotterize(st, H, 0.05, order=2, evol="real")
    # the last gate of the even row is a one-site field gate
    assert rows[1][1][-1].ndim == 2 and rows[1][0][-1] == N
    zops = O.OpList(N)
    for i in range(1, N + 1):
        zops.add("z", i)
    rec = {}
    O.tebd(st, psi, H, 0.05, 0.25, 0.05, [zops], cutoff=0.0, maxdim=0, evol="real", record=rec)
    v = v0
    for _ in range(5):
        v = X.apply_rows_dense(v, rows, N, 2)
    v = v / np.linalg.norm(v)
    z_dense = [X.dense_expect(v, X.oplist_to_dense(st, _single(N, "z", i))) for i in range(1, N + 1)]
    assert np.allclose(np.real(rec["ops"][-1][0]), np.real(z_dense), atol=1e-10)
    assert abs(abs(np.vdot(X.mps_to_dense(psi), v)) - 1) < 1e-10


def _single(N, name, i):
    o = O.OpList(N)
    o.add(name, i)
    return o


def test_inner_matches_dense():
    st = O.spinhalf()
    N = 6
    psi = O.random_mps(2, N, 3, np.random.default_rng(4))
    ops = O.OpList(N)
    ops.add("z", 2)
    ops.add(["x", "y"], [3, 4], 0.7)
    ops.add(["z", "x"], [1, 3], 1.3)
    got = O.inner(st, psi, ops, psi)
    v = X.mps_to_dense(psi)
    for k in range(3):
        one = O.OpList(N)
        one.add(ops.ops[k], ops.sites[k], ops.coeffs[k])
        assert abs(got[k] - np.vdot(v, X.oplist_to_dense(st, one) @ v)) < 1e-12


def test_qjmc_single_site_decay_closed_form():
    """H = 0, L = sqrt(g) s-: from |up>, no-jump evolution keeps |up> and the
    jump probability per step is 1 - exp(-g dt) exactly."""
    st = O.spinhalf()
    N, g, dt = 1, 0.3, 0.01
    H = O.OpList(N)
    H.add("z", 1, 0.0)
    L = O.OpList(N)
    L.add("s-", 1, np.sqrt(g))
    psi = O.product_mps(st, ["up"])
    # draws: step1 (unused, decision=0.5 -> no jump), step2 (unused, 0.9999 -> jump, pick 0.1)
    draws = [0.3, 0.5, 0.3, 0.9999, 0.1, 0.2, 0.5]
    stream = O.algorithms.UniformStream(draws)
    jumps, times = O.qjmc_simulation(st, psi, H, L, 3 * dt, dt, stream, cutoff=1e-12)
    assert jumps == [1] and abs(times[0] - 2 * dt) < 1e-15
    assert np.allclose(np.abs(psi[1].ravel()), [0, 1])


def test_qjmc_single_site_decay_closed_form_norm_based():
    """classical=false (qjmc.jl:65-86), H = 0, L = sqrt(g) s-: from |up> the
    unnormalised state after a step has squared norm exp(-g dt), so a jump
    happens at the first step whose one draw exceeds it (a second draw then
    picks the channel); after it |down> keeps norm 1 and never jumps again."""
    st = O.spinhalf()
    N, g, dt = 1, 0.3, 0.01
    H = O.OpList(N)
    H.add("z", 1, 0.0)
    L = O.OpList(N)
    L.add("s-", 1, np.sqrt(g))
    p = np.exp(-g * dt)
    # step 1 just below the threshold, step 2 just above it (then the pick),
    # steps 3-4 at the top of [0, 1)
    draws = [p - 1e-9, p + 1e-9, 0.7, 0.999999, 0.999999]
    psi = O.product_mps(st, ["up"])
    jumps, times = O.qjmc_simulation(st, psi, H, L, 4 * dt, dt, O.algorithms.UniformStream(draws),
                                     cutoff=1e-12, classical=False)
    assert jumps == [1] and abs(times[0] - 2 * dt) < 1e-15
    assert np.allclose(np.abs(psi[1].ravel()), [0, 1])


@pytest.mark.parametrize("classical", [True, False])
def test_qjmc_matches_lindblad(classical):
    """Both unravelings of qjmc_simulation (classical=true: escape rates;
    classical=false: the norm of the unnormalised state, qjmc.jl:65-86)
    reproduce the Lindblad master equation statistically."""
    st = O.spinhalf()
    N, dt, T = 2, 0.02, 0.6
    H = O.OpList(N)
    H.add(["z", "z"], [1, 2], 1.0)
    H.add("x", 1, 0.8)
    H.add("x", 2, 0.8)
    L = O.OpList(N)
    for i in (1, 2):
        L.add("s-", i, np.sqrt(0.5))
    zops = O.OpList(N)
    zops.add("z", 1)
    zops.add("z", 2)
    rng = np.random.default_rng(7)
    ntraj = 150
    zs = []
    for _ in range(ntraj):
        psi = O.product_mps(st, ["up", "up"])
        rec = {}
        O.qjmc_simulation(st, psi, H, L, T, dt, lambda: float(rng.random()), [zops],
                          save=T, cutoff=1e-12, record=rec, classical=classical)
        zs.append(np.real(rec["ops"][-1][0]))
    zs = np.array(zs)
    Hd = X.oplist_to_dense(st, H)
    Ls = [X.oplist_to_dense(st, _single(N, "s-", i)) * np.sqrt(0.5) for i in (1, 2)]
    v0 = np.zeros(4, dtype=complex)
    v0[0] = 1
    rho = X.lindblad_evolve(Hd, Ls, np.outer(v0, v0.conj()), [T])[0]
    for i in (1, 2):
        ex = np.real(np.trace(rho @ X.oplist_to_dense(st, _single(N, "z", i))))
        err = zs[:, i - 1].std() / np.sqrt(ntraj)
        assert abs(zs[:, i - 1].mean() - ex) < 4 * err + 0.03


def test_tebd_xx_chain_matches_free_fermion_dynamics():
    """Beyond exact-diagonalisation sizes: the XX chain H = sum (X X + Y Y)
    maps (Jordan-Wigner) to free fermions with hopping 2, so <Z_i>(t) from
    a Neel state follows from the single-particle propagator exp(-i h t).
    The oracle's real-time TEBD (N=24, chi<=64, dt=0.01) must agree up to
    its second-order Trotter error."""
    st = O.spinhalf()
    N, dt, steps = 24, 0.01, 50
    H = xxz(N, 1.0, 0.0)
    names = ["up" if i % 2 else "dn" for i in range(1, N + 1)]
    psi = O.product_mps(st, names)
    zops = O.OpList(N)
    for i in range(1, N + 1):
        zops.add("z", i)
    rec = {}
    O.tebd(st, psi, H, dt, steps * dt, steps * dt, [zops], cutoff=1e-12, maxdim=64, evol="real",
           record=rec)
    z_tebd = np.real(np.asarray(rec["ops"][-1][0]))
    # free fermions: n_i = (1 + Z_i) / 2 with "up" occupied; C(t) = U C(0) U^H
    z_exact = np.asarray(known_answers()["xx_open_N24_neel_t0.5_z"])
    n0 = np.array([1.0 if i % 2 else 0.0 for i in range(1, N + 1)])
    assert np.max(np.abs(z_tebd - z_exact)) < 2e-4, np.max(np.abs(z_tebd - z_exact))  # 4e-5 measured
    # and the dynamics is far from trivial at this time
    assert np.max(np.abs(z_exact - (2.0 * n0 - 1.0))) > 0.5


def test_dmrg_xx_chain_free_fermion_energy():
    """Oracle DMRG beyond exact-diagonalisation sizes: the XX chain at N=32
    (free fermions with hopping 2, single-particle energies 4 cos(k pi/(N+1)))
    has ground energy = sum of the negative single-particle energies."""
    N = 32
    rng = np.random.default_rng(8)
    shapes = [((1 if i == 0 else 8), 2, (1 if i == N - 1 else 8)) for i in range(N)]
    draws = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    draws.append(O.fr(rng.standard_normal(4), (1, 2, 2)))
    psi = O.random_mps(2, N, 8, draws)
    H = O.mpo_from_oplist(O.spinhalf(), xxz(N, 1.0, 0.0))
    _, E = O.dmrg(psi, H, maxdim=48, cutoff=1e-12, minsweeps=6, maxsweeps=6, numconverges=np.inf)
    E_exact = known_answers()["xx_open_N32_energy"]
    assert abs(np.real(E) - E_exact) <= 1e-6 * abs(E_exact), (np.real(E), E_exact)


def test_known_answer_fixtures_are_current():
    """tests/golden/known_answers.json equals what its generating script
    computes, and its TFIM value equals the oracle's free-fermion helper."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    fresh, stored = m.answers(), known_answers()
    assert set(fresh) == set(stored)
    for k in fresh:
        assert np.allclose(fresh[k], stored[k], rtol=1e-13, atol=1e-13), k
    assert abs(stored["tfim_open_N20_J1_h0.5_energy"] - X.tfim_free_fermion_energy(20, 1.0, 0.5)) < 1e-12


def test_dmrg_sum_of_mpos_and_projector_matches_ed():
    """dmrg(psi, Hs...; coeffs) (dmrg.jl:128-154): a sum of two MPOs gives the
    ground energy of their weighted sum, and an MPS term coeff |phi0><phi0|
    (ProjMPS(phi0, psi; squared=true)) lifts the ground state so that DMRG
    finds the first excited state."""
    st = O.spinhalf()
    N = 8
    Hxy, Hzz = O.OpList(N), O.OpList(N)
    for i in range(1, N):
        Hxy.add(["x", "x"], [i, i + 1], 1.0)
        Hxy.add(["y", "y"], [i, i + 1], 1.0)
        Hzz.add(["z", "z"], [i, i + 1], 1.0)
    W1, W2 = O.mpo_from_oplist(st, Hxy), O.mpo_from_oplist(st, Hzz)
    kw = dict(maxdim=32, cutoff=1e-12, maxsweeps=8, minsweeps=8, numconverges=np.inf)
    psi = O.random_mps(2, N, 4, np.random.default_rng(3))
    psi, E = O.dmrg(psi, [W1, W2], coeffs=[1.0, 0.7], **kw)
    dense = X.oplist_to_dense(st, Hxy) + 0.7 * X.oplist_to_dense(st, Hzz)
    assert abs(np.real(E) - np.linalg.eigvalsh(dense)[0]) < 1e-8
    # excited state of a gapped transverse-field Ising chain
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -1.0)
    for i in range(1, N + 1):
        H.add("x", i, -1.5)
    W = O.mpo_from_oplist(st, H)
    ev = np.linalg.eigvalsh(X.oplist_to_dense(st, H))
    g = O.random_mps(2, N, 4, np.random.default_rng(4))
    g, E0 = O.dmrg(g, W, **kw)
    assert abs(np.real(E0) - ev[0]) < 1e-9
    ex = O.random_mps(2, N, 4, np.random.default_rng(5))
    ex, E1 = O.dmrg(ex, [W, g], coeffs=[1.0, 20.0], **kw)
    assert abs(np.real(E1) - ev[1]) < 1e-8
    assert abs(np.vdot(X.mps_to_dense(g), X.mps_to_dense(ex))) < 1e-5


def test_philox4x32_10_known_answers():
    """The oracle's Philox4x32-10 against the generator's published
    known-answer vectors (Salmon et al., SC 2011)."""
    from oracle.philox import philox4x32_10
    kats = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
            ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
            ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
             (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for c, k, e in kats:
        assert philox4x32_10(c, k) == e


def test_mpo_mps_product_and_vmps_match_dense():
    """applyMPO (MPOMPSProduct, mpo.jl:125-146) equals the dense operator on
    the dense state, and vmps (vmps.jl:1-105) fits the dense weighted sum of
    two MPSs when nothing is truncated."""
    st = O.spinhalf()
    N = 6
    H = xxz(N, 1.0, 0.5)
    W = O.mpo_from_oplist(st, H)
    rng = np.random.default_rng(8)
    psi = O.random_mps(2, N, 3, rng)
    phi = O.mpo_mps_product(W, psi)
    ref = X.oplist_to_dense(st, H) @ X.mps_to_dense(psi)
    assert np.linalg.norm(X.mps_to_dense(phi) - ref) < 1e-10 * np.linalg.norm(ref)
    assert phi.center == 1
    p1, p2 = O.random_mps(2, N, 3, rng), O.random_mps(2, N, 2, rng)
    stats = {}
    fit = O.vmps(p1, p2, coeffs=[1.0, -0.5j], cutoff=0.0, maxdim=64, stats=stats)
    target = X.mps_to_dense(p1) - 0.5j * X.mps_to_dense(p2)
    assert np.linalg.norm(X.mps_to_dense(fit) - target) < 1e-10 * np.linalg.norm(target)
    assert abs(stats["cost"] + np.vdot(target, target).real) < 1e-9
    # the projector |p2><p2| / <p2|p2> applied to p1
    P = O.MPSProjector(p2)
    v2 = X.mps_to_dense(p2)
    ref = v2 * np.vdot(v2, X.mps_to_dense(p1)) / np.vdot(v2, v2)
    assert np.allclose(X.mps_to_dense(P.apply(p1)), ref, atol=1e-12)


def test_tebd_with_projector_finds_excited_state():
    """tebd(...; projectors) (tebd.jl:23-41,67-73): imaginary time with the
    ground state projected out every step converges to the first excited
    state of a gapped transverse-field Ising chain.  The all-up start overlaps
    both parity sectors (a Neel start has no weight on the first excited
    state); the tolerance covers the O(dt) Trotter bias at dt = 0.05."""
    st = O.spinhalf()
    N = 6
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -1.0)
    for i in range(1, N + 1):
        H.add("x", i, -1.5)
    ev = np.linalg.eigvalsh(X.oplist_to_dense(st, H))
    W = O.mpo_from_oplist(st, H)
    g = O.random_mps(2, N, 4, np.random.default_rng(1))
    g, _ = O.dmrg(g, W, maxdim=32, cutoff=1e-14, minsweeps=8, maxsweeps=8, numconverges=np.inf)
    mH = O.OpList(N)  # the gates are exp(+dt H'): H' = -H for cooling
    for ops, sites, c in zip(H.ops, H.sites, H.coeffs):
        mH.add(ops, sites, -c)
    psi = O.product_mps(st, ["up"] * N)
    psi, _ = O.tebd(st, psi, mH, 0.05, 8.0, 8.0, cutoff=1e-12, maxdim=32, projectors=[g],
                    projection_every=1)
    v = X.mps_to_dense(psi)
    v /= np.linalg.norm(v)
    assert abs(X.dense_expect(v, X.oplist_to_dense(st, H)) - ev[1]) < 2e-5
    assert abs(np.vdot(X.mps_to_dense(g), v)) < 1e-6


def test_heff2_reference_order_matches_optimal_order():
    """The reference's contraction order (the CPU baseline's) and the
    oracle's optimal order give the same two-site product."""
    rng = np.random.default_rng(12)

    def c(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    L, W1, W2, R, th = c(6, 3, 6), c(3, 2, 2, 4), c(4, 2, 2, 5), c(7, 5, 7), c(6, 2, 2, 7)
    a = O.core.heff2(L, W1, W2, R, th)
    b = O.core.heff2_reference_order(L, W1, W2, R, th)
    assert np.allclose(a, b, rtol=1e-13, atol=1e-12)


def test_mpo_algebra_and_thermal_state_match_dense():
    """MPOMPOProduct, adjoint and trace (mpo.jl:32-39, 147-167, 229-252)
    against dense matrices, and the thermal-state workflow of
    examples/thermal.jl (the identity evolved by exp(-dt H) gates to beta/2,
    energy Tr(H U^dag U) / Tr(U^dag U)) against exact diagonalisation, within
    the second-order Trotter error at dt = 0.05."""
    import scipy.linalg as sl
    st = O.spinhalf()
    N = 5
    H = tfim(N, 1.0, 1.0)
    W = O.mpo_from_oplist(st, H)
    Hd = X.oplist_to_dense(st, H)
    assert np.allclose(X.mpo_to_dense(O.mpo_mpo_product(W, W)), Hd @ Hd, atol=1e-10)
    assert np.allclose(X.mpo_to_dense(O.adjoint_mpo(W)), Hd.conj().T, atol=1e-12)
    assert abs(O.trace_mpos(W, W) - np.trace(Hd @ Hd)) < 1e-9
    beta, dt = 1.0, 0.05
    mH = O.OpList(N)
    for ops, sites, c in zip(H.ops, H.sites, H.coeffs):
        mH.add(ops, sites, -c)
    rows = O.trotterize(st, mH, dt)
    U = O.product_mpo(st, ["id"] * N)
    for _ in range(int(round(beta / 2 / dt))):
        O.applygates(U, rows, cutoff=1e-12, maxdim=64)
    Ud = X.mpo_to_dense(U)
    assert np.linalg.norm(Ud - sl.expm(-beta / 2 * Hd)) <= 2e-3 * np.linalg.norm(Ud)
    Ua = O.adjoint_mpo(U)
    E = O.trace_mpos(W, Ua, U) / O.trace_mpos(Ua, U)
    ev = np.linalg.eigvalsh(Hd)
    w = np.exp(-beta * ev)
    assert abs(E - np.sum(w * ev) / np.sum(w)) < 1e-4


def _complex_mps(rng, N, D, d=2):
    dims = [1] + [min(D, d ** min(i, N - i)) for i in range(1, N)] + [1]
    ts = [O.fr(rng.standard_normal((dims[i], d, dims[i + 1]))
               + 1j * rng.standard_normal((dims[i], d, dims[i + 1])), (dims[i], d, dims[i + 1]))
          for i in range(N)]
    return O.GMPS(1, d, ts, 0)


def _schmidt(vec, N, bond, d=2):
    """Schmidt coefficients of a normalised dense state across (bond, bond+1);
    the dense vector is column-major, site 1 fastest."""
    M = O.fr(vec / np.linalg.norm(vec), (d ** bond, d ** (N - bond)))
    return np.linalg.svd(M, compute_uv=False)


def test_gauge_moves_match_dense_state():
    """movecenter! (gmps.jl:60-112) without truncation keeps the dense state
    and leaves the sites left of the centre left-orthonormal and those right
    of it right-orthonormal."""
    rng = np.random.default_rng(11)
    N = 7
    psi = _complex_mps(rng, N, 5)
    v0 = X.mps_to_dense(psi)
    for c in (4, 1, N, 3):
        psi.movecenter(c)
        assert psi.center == c
        assert np.allclose(X.mps_to_dense(psi), v0, atol=1e-12 * np.linalg.norm(v0))
        for i in range(1, N + 1):
            A = psi[i]
            if i < c:
                M = O.fr(A, (-1, A.shape[2]))
                assert np.allclose(M.conj().T @ M, np.eye(A.shape[2]), atol=1e-12)
            elif i > c:
                M = O.fr(A, (A.shape[0], -1))
                assert np.allclose(M @ M.conj().T, np.eye(A.shape[0]), atol=1e-12)


def test_entropy_and_spectra_match_dense_schmidt_values():
    """entropy(psi, i) (gmps.jl:184-189) is -sum s^2 ln s^2 of the dense
    state's Schmidt values across bond i; a product state gives 0 and a
    GHZ state ln 2 at every bond."""
    rng = np.random.default_rng(12)
    N = 8
    psi = _complex_mps(rng, N, 6)
    psi.normalize()
    v = X.mps_to_dense(psi)
    for bond in range(1, N):
        s = _schmidt(v, N, bond)
        s = s[s > 1e-14]
        assert abs(psi.entropy(bond) - float(-np.sum(s ** 2 * np.log(s ** 2)))) < 1e-10
        sv = psi.singular_values(bond)
        assert np.allclose(np.sort(sv)[::-1][:len(s)], s, atol=1e-12)
    prod = O.product_mps(O.spinhalf(), ["up", "dn"] * 3)
    assert all(abs(prod.entropy(b)) < 1e-14 for b in range(1, 6))
    ghz = []
    for i in range(N):
        t = np.zeros((1 if i == 0 else 2, 2, 1 if i == N - 1 else 2), dtype=np.complex128)
        for k in range(2):
            t[0 if i == 0 else k, k, 0 if i == N - 1 else k] = 1.0
        ghz.append(t)
    g = O.GMPS(1, 2, ghz, 0)
    g.normalize()
    assert all(abs(g.entropy(b) - np.log(2)) < 1e-12 for b in range(1, N))


@pytest.mark.parametrize("direction", [False, True])
def test_replacesites_matches_dense_split(direction):
    """replacesites! (gmps.jl:199-267): an untruncated split keeps the dense
    state with theta in place; truncated to k it keeps theta's k largest
    singular values, and the centre lands where the reference puts it."""
    rng = np.random.default_rng(13)
    N, site = 5, 2
    psi = _complex_mps(rng, N, 4)
    psi.movecenter(site)
    Dl, Dr = psi[site].shape[0], psi[site + 1].shape[2]
    theta = rng.standard_normal((Dl, 2, 2, Dr)) + 1j * rng.standard_normal((Dl, 2, 2, Dr))
    ref = O.GMPS(1, 2, [psi[i] for i in range(1, N + 1)], psi.center)
    # the dense state with theta in place of sites (site, site+1)
    left = ref[1]
    for i in range(2, site):
        left = np.tensordot(left, ref[i], axes=([left.ndim - 1], [0]))
    full = np.tensordot(left, theta, axes=([left.ndim - 1], [0]))
    for i in range(site + 2, N + 1):
        full = np.tensordot(full, ref[i], axes=([full.ndim - 1], [0]))
    dense = O.fr(full[0, ..., 0], (-1,))
    a = O.GMPS(1, 2, [ref[i] for i in range(1, N + 1)], ref.center)
    a.replacesites(theta, site, direction)
    assert a.center == (site if direction else site + 1)
    assert np.allclose(X.mps_to_dense(a), dense, atol=1e-12 * np.linalg.norm(dense))
    s = np.linalg.svd(O.fr(theta, (Dl * 2, 2 * Dr)), compute_uv=False)
    k = 2
    b = O.GMPS(1, 2, [ref[i] for i in range(1, N + 1)], ref.center)
    b.replacesites(theta, site, direction, maxdim=k)
    c = b[b.center]
    # the centre holds U S: [Dl, s1, k] at the left site (direction true),
    # [k, s2, Dr] at the right one
    kept = np.linalg.svd(O.fr(c, (-1, c.shape[2])) if direction else O.fr(c, (c.shape[0], -1)),
                         compute_uv=False)
    assert np.allclose(np.sort(kept)[::-1][:k], s[:k], rtol=1e-12)
    assert b[site].shape[2] == k


def test_emission_rates_match_dense_expectations():
    """qjmc_emission_rates (qjmc.jl:170-220): |c^2 <psi|L^dag L|psi>| for a
    normalised state equals the dense expectation of each channel."""
    rng = np.random.default_rng(14)
    N = 6
    psi = _complex_mps(rng, N, 4)
    psi.normalize()
    v = X.mps_to_dense(psi)
    st = O.spinhalf()
    Lj = O.OpList(N)
    for i in range(1, N + 1):
        Lj.add("s-", i, np.sqrt(0.1 * i))
    Lj.add("z", 3, 0.5)
    rates = O.qjmc_emission_rates(st, psi, Lj)
    for k in range(len(Lj.ops)):
        single = O.OpList(N)
        single.add(Lj.ops[k][0], Lj.sites[k][0], 1.0)
        Ld = X.oplist_to_dense(st, single)
        ex = abs(Lj.coeffs[k]) ** 2 * np.real(np.vdot(Ld @ v, Ld @ v))
        assert abs(rates[k] - ex) < 1e-12


def test_trotter_rows_converge_at_second_order():
    """trotterize(...; order=2) (gatelist.jl:75-121): [odd(dt/2), even(dt),
    odd(dt/2)] rows applied to a dense state approach exp(-iHT) with an
    error falling as dt^2 (order=1: as dt)."""
    import scipy.linalg as sla
    st = O.spinhalf()
    N, T = 6, 0.4
    H = xxz(N, 1.0, 0.5, lambda i: 0.3 * i)
    v0 = X.mps_to_dense(O.product_mps(st, ["up" if i % 2 else "dn" for i in range(1, N + 1)]))
    exact = sla.expm(-1j * T * X.oplist_to_dense(st, H)) @ v0
    for order, rate in ((2, 4.0), (1, 2.0)):
        errs = []
        for n in (8, 16):
            rows = O.trotterize(st, H, T / n, order=order, evol="real")
            v = v0
            for _ in range(n):
                v = X.apply_rows_dense(v, rows, N, 2)
            errs.append(np.linalg.norm(v - exact))
        assert abs(errs[0] / errs[1] - rate) < 0.1 * rate, (order, errs)  # 4.007 and 2.012


def test_qjmc_gates_give_the_no_jump_evolution():
    """qjmc_gates (qjmc.jl:9-26): the Trotter rows of H_eff = -iH - 1/2 sum
    c^2 L^dag L (imaginary-time gates exp(dt H_eff)) applied to a dense
    state match exp(T H_eff), the unnormalised no-jump evolution, to the
    second-order Trotter error."""
    import scipy.linalg as sla
    st = O.spinhalf()
    N, T, n = 4, 0.3, 30
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
    Lj = O.OpList(N)
    for i in range(1, N + 1):
        Lj.add("s-", i, np.sqrt(0.5))
    heff, rows = O.qjmc_gates(st, H, Lj, T / n)
    Hd = X.oplist_to_dense(st, H)
    Ld = [np.sqrt(0.5) * X.oplist_to_dense(st, _single(N, "s-", i)) for i in range(1, N + 1)]
    Heff = -1j * Hd - 0.5 * sum(L.conj().T @ L for L in Ld)
    assert np.allclose(X.oplist_to_dense(st, heff), Heff, atol=1e-14)
    v0 = X.mps_to_dense(O.product_mps(st, ["up"] * N))
    v = v0
    for _ in range(n):
        v = X.apply_rows_dense(v, rows, N, 2)
    exact = sla.expm(T * Heff) @ v0
    assert np.linalg.norm(v - exact) < 1e-3 * np.linalg.norm(exact)
    assert abs(np.linalg.norm(v) ** 2 - np.linalg.norm(exact) ** 2) < 1e-3


def _fixture_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_oracle_fixtures", os.path.join(GOLDEN, "make_oracle_fixtures.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_oracle_reproduces_its_committed_outputs():
    """tests/golden/oracle_outputs.json holds the parity cases' explicit
    inputs (randomGMPS draws, uniform streams) and the oracle's outputs;
    recomputing from the stored inputs gives the stored outputs (energies
    1e-10 relative, spectra, entropies and <Z_i> 1e-9, bond dimensions and
    jump records identical)."""
    m = _fixture_module()
    with open(os.path.join(GOLDEN, "oracle_outputs.json")) as f:
        fx = json.load(f)
    for name in ("dmrg_tfim_N20_config1", "dmrg_xxz_N16"):
        c = fx[name]
        E, dims, S, ent, z = m.run_dmrg_case(c)
        assert abs(E - c["energy_last_lanczos"]) <= 1e-10 * abs(E), name
        assert dims == c["bonddims"], name
        assert np.allclose(S, c["singular_values"], atol=1e-9), name
        assert abs(ent - c["entropy_bond"]) < 1e-9 and np.allclose(z, c["z"], atol=1e-9), name
    c = fx["tebd_xxz_N16_quench"]
    z, ln, dims, ent = m.run_tebd_case(c)
    assert np.allclose(z, c["z_per_step"], atol=1e-9) and np.allclose(ln, c["lognorm"], atol=1e-9)
    assert dims == c["bonddims"] and abs(ent - c["entropy_mid"]) < 1e-9
    for name in ("qjmc_ising_N8_classical", "qjmc_ising_N8_norm_based"):
        c = fx[name]
        j, t, z = m.run_qjmc_case(c)
        assert j == c["jumps"] and len(j) > 0, name
        assert np.allclose(t, c["jump_times"], rtol=0, atol=1e-12), name
        assert np.allclose(z, c["z_per_step"], atol=1e-9), name
    # the stored randomGMPS draws are the seeded ones the parity tests use
    dr = m.seeded_draws(20, 4, 1)
    assert all(np.array_equal(a, m.dec(e)) for a, e in
               zip(dr, fx["dmrg_tfim_N20_config1"]["randomMPS_draws"]))
