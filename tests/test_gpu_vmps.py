"""MPS algebra on the device against the oracle and dense vectors: the
MPO-MPS product (MPOMPSProduct, mpo.jl:105-146), overlaps (inner(phi, psi),
mpo.jl:181-250), scaling (abstractmps.jl:100-107), MPSProjector
(projector.jl:1-47), variational fitting (vmps.jl:1-105) and TEBD with
projectors (tebd.jl:23-41,67-73), all through the C ABI."""

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def _tfim(mod, N, h=1.5):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -1.0)
    for i in range(1, N + 1):
        H.add("x", i, -h)
    return H


def _pair(tn, N, D, seed):
    po = O.random_mps(2, N, D, np.random.default_rng(seed))
    return po, tn.GMPS.from_tensors(po.tensors, po.center)


def _dense(g):
    return X.mps_to_dense(O.GMPS(1, g.dim, g.tensors(), g.center))


def test_overlap_and_scale_match_dense(tn):
    N = 8
    ao, ag = _pair(tn, N, 5, 1)
    bo, bg = _pair(tn, N, 3, 2)
    ref = np.vdot(X.mps_to_dense(ao), X.mps_to_dense(bo))
    assert abs(tn.overlap(ag, bg) - ref) < 1e-12
    assert abs(O.overlap(ao, bo) - ref) < 1e-12
    c = 0.3 - 1.7j
    sg = bg * c
    assert np.allclose(_dense(sg), c * X.mps_to_dense(bo), atol=1e-12)
    assert np.allclose(_dense(bg), X.mps_to_dense(bo), atol=1e-12)  # the original untouched


@pytest.mark.parametrize("maxdim", [0, 6])
def test_mpo_mps_product_matches_oracle(tn, maxdim):
    N = 8
    po, pg = _pair(tn, N, 4, 3)
    Wo, Wg = O.mpo_from_oplist(O.spinhalf(), _tfim(O, N)), tn.MPO(tn.spinhalf(), _tfim(tn, N))
    cut = 0.0 if maxdim == 0 else 1e-14
    go = O.mpo_mps_product(Wo, po, cutoff=cut, maxdim=maxdim)
    gg = tn.applyMPO(Wg, pg, cutoff=cut, maxdim=maxdim)
    assert gg.center == 1
    assert gg.bonddims() == go.bonddims()
    vg, vo = _dense(gg), X.mps_to_dense(go)
    assert np.linalg.norm(vg - vo) <= 1e-11 * np.linalg.norm(vo)
    if maxdim == 0:
        Hd = X.oplist_to_dense(O.spinhalf(), _tfim(O, N))
        exact = Hd @ X.mps_to_dense(po)
        assert np.linalg.norm(vg - exact) <= 1e-11 * np.linalg.norm(exact)


def test_vmps_fits_weighted_sum(tn):
    N = 8
    ao, ag = _pair(tn, N, 4, 4)
    bo, bg = _pair(tn, N, 4, 5)
    cs = [1.0, 0.5 - 0.25j]
    kw = dict(maxdim=8, cutoff=1e-14, minsweeps=2, maxsweeps=6)
    sg, so = {}, {}
    fg = tn.vmps(ag, bg, coeffs=cs, stats=sg, **kw)
    fo = O.vmps(ao, bo, coeffs=cs, stats=so, **kw)
    assert sg["sweeps"] == so["sweeps"]
    assert abs(sg["cost"] - so["cost"]) <= 1e-10 * abs(so["cost"])
    assert fg.bonddims() == fo.bonddims()
    target = cs[0] * X.mps_to_dense(ao) + cs[1] * X.mps_to_dense(bo)
    vg = _dense(fg)
    # D = 8 holds the sum of two D = 4 states exactly
    assert np.linalg.norm(vg - target) <= 1e-9 * np.linalg.norm(target)
    assert abs(sg["cost"] + np.linalg.norm(target) ** 2) <= 1e-9 * np.linalg.norm(target) ** 2


def test_mps_projector_apply(tn):
    N = 6
    lo, lg = _pair(tn, N, 3, 6)
    ro, rg = _pair(tn, N, 2, 7)
    po, pg = _pair(tn, N, 4, 8)
    Pg, Po = tn.MPSProjector(lg, rg), O.MPSProjector(lo, ro)
    assert abs(Pg.constant - Po.constant) < 1e-12
    vg = _dense(tn.applyMPO(Pg, pg))
    vo = X.mps_to_dense(Po.apply(po))
    assert np.linalg.norm(vg - vo) <= 1e-12 * np.linalg.norm(vo)
    vl, vr, vp = (X.mps_to_dense(x) for x in (lo, ro, po))
    exact = vr * np.vdot(vl, vp) / np.vdot(vl, vr)
    assert np.linalg.norm(vg - exact) <= 1e-12 * np.linalg.norm(exact)


def test_tebd_with_projector_matches_oracle(tn):
    """Imaginary time with the ground state projected out converges to the
    first excited state; device and oracle follow the same trajectory."""
    N = 6
    st_o, st_g = O.spinhalf(), tn.spinhalf()
    H = _tfim(O, N)
    ev = np.linalg.eigvalsh(X.oplist_to_dense(st_o, H))
    go = O.random_mps(2, N, 4, np.random.default_rng(1))
    go, _ = O.dmrg(go, O.mpo_from_oplist(st_o, H), maxdim=32, cutoff=1e-14, minsweeps=8,
                   maxsweeps=8, numconverges=np.inf)
    gg = tn.GMPS.from_tensors(go.tensors, go.center)
    mo, mg = O.OpList(N), tn.OpList(N)  # the gates are exp(+dt H'): H' = -H cools
    for ops, sites, c in zip(H.ops, H.sites, H.coeffs):
        mo.add(ops, sites, -c)
        mg.add(ops, sites, -c)
    kw = dict(cutoff=1e-12, maxdim=32, projection_every=1)
    po, _ = O.tebd(st_o, O.product_mps(st_o, ["up"] * N), mo, 0.05, 2.0, 2.0, projectors=[go], **kw)
    pg, _ = tn.tebd(st_g, tn.productMPS(st_g, ["up"] * N), mg, 0.05, 2.0, 2.0, projectors=[gg],
                    **kw)
    vo, vg = X.mps_to_dense(po), _dense(pg)
    vo, vg = vo / np.linalg.norm(vo), vg / np.linalg.norm(vg)
    assert abs(abs(np.vdot(vo, vg)) - 1) < 1e-9
    assert abs(np.vdot(X.mps_to_dense(go), vg)) < 1e-7
    # longer evolution on the device alone reaches E1 within the O(dt) Trotter bias
    pg, _ = tn.tebd(st_g, pg, mg, 0.05, 6.0, 6.0, projectors=[gg], **kw)
    vg = _dense(pg)
    vg /= np.linalg.norm(vg)
    assert abs(X.dense_expect(vg, X.oplist_to_dense(st_o, H)) - ev[1]) < 2e-5
