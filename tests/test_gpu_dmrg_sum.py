"""dmrg(psi, Hs...; coeffs) over a sum of terms (dmrg.jl:128-154,
projmpssum.jl:51-108) on the device, through tn_dmrg_sum, against the
oracle's ProjMPSSum DMRG on the same initial tensors: two MPO terms with
coefficients, and an MPS penalty term coeff |phi><phi| (ProjMPS(phi, psi;
squared=true), projmps.jl:103-145) that turns the ground-state search into
an excited-state search."""

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def _xy_zz(mod, N):
    Hxy, Hzz = mod.OpList(N), mod.OpList(N)
    for i in range(1, N):
        Hxy.add(["x", "x"], [i, i + 1], 1.0)
        Hxy.add(["y", "y"], [i, i + 1], 1.0)
        Hzz.add(["z", "z"], [i, i + 1], 1.0)
    return Hxy, Hzz


def _tfim(mod, N, h=1.5):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -1.0)
    for i in range(1, N + 1):
        H.add("x", i, -h)
    return H


KW = dict(maxdim=24, cutoff=1e-12, maxsweeps=4, minsweeps=4, numconverges=np.inf)


def test_dmrg_two_mpo_terms_match_oracle(tn):
    N = 10
    st_o, st_g = O.spinhalf(), tn.spinhalf()
    Ho, Hg = _xy_zz(O, N), _xy_zz(tn, N)
    po = O.random_mps(2, N, 4, np.random.default_rng(21))
    pg = tn.GMPS.from_tensors(po.tensors, po.center)
    Wo = [O.mpo_from_oplist(st_o, h) for h in Ho]
    Wg = [tn.MPO(st_g, h) for h in Hg]
    st = {}
    _, Eg = tn.dmrg(pg, *Wg, coeffs=[1.0, 0.7], verbose=False, stats=st, **KW)
    _, Eo = O.dmrg(po, Wo, coeffs=[1.0, 0.7], **KW)
    assert abs(Eg - np.real(Eo)) <= 1e-10 * abs(Eo)
    assert pg.bonddims() == po.bonddims()
    dense = X.oplist_to_dense(st_o, Ho[0]) + 0.7 * X.oplist_to_dense(st_o, Ho[1])
    v = X.mps_to_dense(po)
    assert abs(st["energy_fp64"] - X.dense_expect(v, dense)) < 1e-9
    assert abs(Eg - np.linalg.eigvalsh(dense)[0]) < 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-env64"])
def test_dmrg_projector_term_finds_excited_state(tn, precision):
    N = 8
    st_o, st_g = O.spinhalf(), tn.spinhalf()
    Wo, Wg = O.mpo_from_oplist(st_o, _tfim(O, N)), tn.MPO(st_g, _tfim(tn, N))
    ev = np.linalg.eigvalsh(X.oplist_to_dense(st_o, _tfim(O, N)))
    go = O.random_mps(2, N, 4, np.random.default_rng(4))
    go, _ = O.dmrg(go, Wo, **KW)
    gg = tn.GMPS.from_tensors(go.tensors, go.center)  # the same ground state on both sides
    eo = O.random_mps(2, N, 4, np.random.default_rng(5))
    eg = tn.GMPS.from_tensors(eo.tensors, eo.center)
    st = {}
    _, Eg = tn.dmrg(eg, Wg, gg, coeffs=[1.0, 20.0], verbose=False, stats=st,
                    precision=precision, **KW)
    _, Eo = O.dmrg(eo, [Wo, go], coeffs=[1.0, 20.0], **KW)
    if precision == "fp64":
        assert abs(Eg - np.real(Eo)) <= 1e-10 * abs(Eo)
        assert eg.bonddims() == eo.bonddims()
    # the final state: first excited energy, orthogonal to the ground state
    vg = X.mps_to_dense(O.GMPS(1, 2, eg.tensors()))
    E1 = X.dense_expect(vg, X.oplist_to_dense(st_o, _tfim(O, N)))
    assert abs(E1 - ev[1]) < 1e-7
    ov = np.vdot(X.mps_to_dense(go), vg)
    assert abs(ov) < 1e-4
    # energy_fp64 = <H> + 20 |<phi|psi>|^2 of the final state
    assert abs(st["energy_fp64"] - (E1 + 20.0 * abs(ov) ** 2)) < 1e-9
    assert gg.bonddims() == go.bonddims()  # the projector state is not modified
