"""MPO algebra on the device against the oracle: MPOs held in fused form
(an MPS of physical dimension d^2), the MPO-MPO product (MPOMPOProduct,
mpo.jl:147-167), adjoint and trace (mpo.jl:32-39, 229-252), and the
thermal-state workflow of examples/thermal.jl: applygates! on an MPO from
the identity (gates on the output index, gatelist.jl:137-171 with rank 2)
and the energy Tr(H U^dag U) / Tr(U^dag U)."""

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def _tfim(mod, N, J=1.0, h=1.0):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], J)
    for i in range(1, N + 1):
        H.add("x", i, h)
    return H


def _dense_mpo(ts):
    return X.mpo_to_dense(O.GMPS(2, ts[0].shape[1], ts, 0))


@pytest.mark.parametrize("maxdim", [0, 5])
def test_mpo_mpo_product_matches_oracle(tn, maxdim):
    N = 6
    Wo = O.mpo_from_oplist(O.spinhalf(), _tfim(O, N))
    Wg = tn.MPO(tn.spinhalf(), _tfim(tn, N))
    cut = 0.0 if maxdim == 0 else 1e-14
    Po = O.mpo_mpo_product(Wo, Wo, cutoff=cut, maxdim=maxdim)
    Pg = tn.applyMPO(tn.as_gmpo(Wg), tn.as_gmpo(Wg), cutoff=cut, maxdim=maxdim)
    assert Pg.center == 1 and Pg.bonddims() == Po.bonddims()
    dg, do = _dense_mpo(Pg.tensors()), X.mpo_to_dense(Po)
    assert np.linalg.norm(dg - do) <= 1e-11 * np.linalg.norm(do)
    if maxdim == 0:
        Hd = X.oplist_to_dense(O.spinhalf(), _tfim(O, N))
        assert np.linalg.norm(dg - Hd @ Hd) <= 1e-11 * np.linalg.norm(Hd @ Hd)


def test_adjoint_and_trace_match_dense(tn):
    N = 5
    Wg = tn.as_gmpo(tn.MPO(tn.spinhalf(), _tfim(tn, N, 0.7, -0.4)))
    Hd = X.oplist_to_dense(O.spinhalf(), _tfim(O, N, 0.7, -0.4))
    assert np.allclose(_dense_mpo(tn.adjoint(Wg).tensors()), Hd.conj().T, atol=1e-12)
    assert abs(tn.trace(Wg) - np.trace(Hd)) < 1e-10
    assert abs(tn.trace(Wg, Wg) - np.trace(Hd @ Hd)) < 1e-9
    assert abs(tn.trace(Wg, Wg, Wg) - np.trace(Hd @ Hd @ Hd)) < 1e-8


def test_thermal_state_matches_oracle_and_ed(tn):
    N, beta, dt = 6, 1.0, 0.05
    st_o, st_g = O.spinhalf(), tn.spinhalf()
    Ho, Hg = _tfim(O, N), _tfim(tn, N)
    mo, mg = O.OpList(N), tn.OpList(N)  # trotterize(sh, -1*H, dt)
    for ops, sites, c in zip(Ho.ops, Ho.sites, Ho.coeffs):
        mo.add(ops, sites, -c)
        mg.add(ops, sites, -c)
    rows = O.trotterize(st_o, mo, dt)
    gates = tn.trotterize(st_g, mg, dt)
    Uo = O.product_mpo(st_o, ["id"] * N)
    Ug = tn.productMPO(st_g, ["id"] * N)
    for _ in range(int(round(beta / 2 / dt))):
        O.applygates(Uo, rows, cutoff=1e-12, maxdim=32)
        tn.applygates(Ug, gates, cutoff=1e-12, maxdim=32)
    assert Ug.bonddims() == Uo.bonddims()
    dg, do = _dense_mpo(Ug.tensors()), X.mpo_to_dense(Uo)
    # 30 rows of truncated splits at cutoff 1e-12: the two implementations'
    # roundings meet the truncation's sensitivity at ~1e-10 (1.1e-10 measured)
    assert np.linalg.norm(dg - do) <= 1e-8 * np.linalg.norm(do)
    Wg = tn.MPO(st_g, Hg)
    Ua = tn.adjoint(Ug)
    E = tn.trace(Wg, Ua, Ug) / tn.trace(Ua, Ug)
    Wo = O.mpo_from_oplist(st_o, Ho)
    Eo = O.trace_mpos(Wo, O.adjoint_mpo(Uo), Uo) / O.trace_mpos(O.adjoint_mpo(Uo), Uo)
    assert abs(E - Eo) <= 1e-9 * abs(Eo)
    ev = np.linalg.eigvalsh(X.oplist_to_dense(st_o, Ho))
    w = np.exp(-beta * ev)
    assert abs(E - np.sum(w * ev) / np.sum(w)) < 1e-4


@pytest.mark.parametrize("ext", [".npz", ".h5"])
def test_mps_checkpoint_round_trip_on_device(tn, tmp_path, ext):
    """write_mps / read_mps (the GMPS group layout of gmps.jl:359-383, as an
    HDF5 file or an .npz archive) on a device MPS after a DMRG run: the
    read-back state has the same tensors, centre and energy."""
    N = 8
    st = tn.spinhalf()
    W = tn.MPO(st, _tfim(tn, N))
    po = O.random_mps(2, N, 4, np.random.default_rng(3))
    psi = tn.GMPS.from_tensors(po.tensors, po.center)
    _, E = tn.dmrg(psi, W, maxdim=16, cutoff=1e-12, minsweeps=2, maxsweeps=2, verbose=False)
    path = str(tmp_path / ("state" + ext))
    tn.write_mps(path, psi, name="ground")
    back = tn.read_mps(path, name="ground")
    assert back.center == psi.center and back.bonddims() == psi.bonddims()
    for a, b in zip(psi.tensors(), back.tensors()):
        assert np.array_equal(a, b)
    H = _tfim(tn, N)
    e_back = float(np.real(np.sum(tn.inner(st, back, H, back))))
    assert abs(e_back - E) < 1e-9 * abs(E)
