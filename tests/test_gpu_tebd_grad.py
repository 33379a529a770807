"""TEBD adjoint: gradient of <Z_site>(T) with respect to per-segment field
values h_k of H_k = sum Z Z + h_k sum X, against central finite differences
(step 1e-6) of the GPU forward and of the oracle's forward.  Tolerance: the
gradient agrees with the differences to 1e-5 relative to its largest
component; the objective agrees with the oracle to 1e-10."""

import numpy as np
import pytest

import oracle as O
from oracle import algorithms as OA

pytestmark = pytest.mark.gpu

EPS = 1e-6


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def ising(lib, N):
    def H_of(h):
        H = lib.OpList(N)
        for i in range(1, N):
            H.add(["z", "z"], [i, i + 1], 1.0)
        for i in range(1, N + 1):
            H.add("x", i, float(h))
        return H
    return H_of


def case(N, K, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 1.0, K)


def gpu_fd(prob, psi0, h, idx):
    out = []
    for k in idx:
        hp, hm = h.copy(), h.copy()
        hp[k] += EPS
        hm[k] -= EPS
        out.append((prob.value(psi0, hp) - prob.value(psi0, hm)) / (2 * EPS))
    return np.asarray(out)


def oracle_f(N, h, nsub, dt, site, **kw):
    st = O.spinhalf()
    psi = O.product_mps(st, ["up"] * N)
    Hs = [ising(O, N)(x) for x in h]
    return OA.tebd_segments_objective(st, psi, Hs, dt, nsub, "z", site, **kw)


@pytest.mark.parametrize("maxdim,cutoff", [(3, 1e-12), (0, 1e-14)])
def test_tebd_grad_matches_finite_differences(tn, maxdim, cutoff):
    N, K, nsub, dt, site = 6, 4, 3, 0.05, 3
    h = case(N, K, 5)
    st = tn.spinhalf()
    psi0 = tn.productMPS(st, ["up"] * N)
    prob = tn.TEBDGradProblem(st, ising(tn, N), dt, nsub, "z", site, cutoff=cutoff,
                              maxdim=maxdim, checkpoint=2)
    f, back = prob.rrule(psi0, h)
    g = back()
    # objective against the oracle's forward
    fo = oracle_f(N, h, nsub, dt, site, cutoff=cutoff, maxdim=maxdim)
    assert abs(f - fo) <= 1e-10 * max(1.0, abs(fo)), (f, fo)
    # every coordinate against GPU central differences
    fd = gpu_fd(prob, psi0, h, range(K))
    scale = np.max(np.abs(fd))
    assert np.max(np.abs(g - fd)) <= 1e-5 * scale, (g, fd)
    # two coordinates against central differences of the oracle's forward
    for k in (0, K - 1):
        hp, hm = h.copy(), h.copy()
        hp[k] += EPS
        hm[k] -= EPS
        fdo = (oracle_f(N, hp, nsub, dt, site, cutoff=cutoff, maxdim=maxdim)
               - oracle_f(N, hm, nsub, dt, site, cutoff=cutoff, maxdim=maxdim)) / (2 * EPS)
        assert abs(g[k] - fdo) <= 1e-5 * scale, (k, g[k], fdo)
    # the input state is left unchanged
    assert psi0.bonddims() == [1] * (N + 1)


def test_tebd_grad_checkpoint_interval_invariant(tn):
    N, K, nsub, dt, site = 8, 3, 4, 0.05, 4
    h = case(N, K, 7)
    st = tn.spinhalf()
    psi0 = tn.productMPS(st, ["up"] * N)
    grads = []
    for every in (1, 5, 100):
        prob = tn.TEBDGradProblem(st, ising(tn, N), dt, nsub, "z", site, cutoff=1e-12,
                                  maxdim=4, checkpoint=every)
        f, back = prob.rrule(psi0, h)
        grads.append((f, back()))
    for f, g in grads[1:]:
        assert f == grads[0][0]
        assert np.allclose(g, grads[0][1], rtol=1e-12, atol=1e-14)
