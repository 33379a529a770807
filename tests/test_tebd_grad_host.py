"""Host side of the TEBD adjoint (no GPU): the derivative gates built from
the Frechet derivative of the matrix exponential, and the oracle's
segment-wise TEBD objective against its own tebd loop."""

import numpy as np

import oracle as O
from oracle import algorithms as OA


def _ising(lib, N):
    def H_of(h):
        H = lib.OpList(N)
        for i in range(1, N):
            H.add(["z", "z"], [i, i + 1], 1.0)
        for i in range(1, N + 1):
            H.add("x", i, float(h))
        return H
    return H_of


def test_trotter_rows_dparam_matches_differences():
    import tngpu.models as M
    N, dt, p, e = 5, 0.07, 0.37, 1e-6
    st = M.spinhalf()
    H_of = _ising(M, N)
    drows = M.trotter_rows_dparam(st, H_of(p), H_of(p + 1.0), dt, 2, "real")
    rp = M.trotter_rows(st, H_of(p + e), dt, 2, "real")
    rm = M.trotter_rows(st, H_of(p - e), dt, 2, "real")
    n = 0
    for (sd, dgs), (sp, gp), (_, gm) in zip(drows, rp, rm):
        assert sd == sp
        for dg, a, b in zip(dgs, gp, gm):
            fd = (a - b) / (2 * e)
            assert np.max(np.abs(dg - fd)) <= 1e-8 * max(1.0, np.max(np.abs(fd)))
            n += 1
    assert n == 2 * (N // 2 + N % 2) + (N // 2)  # odd row twice (2nd order) plus the even row


def test_segment_objective_matches_tebd_loop():
    N, dt, nsub, h = 6, 0.05, 4, 0.6
    st = O.spinhalf()
    H = _ising(O, N)(h)
    f = OA.tebd_segments_objective(st, O.product_mps(st, ["up"] * N), [H], dt, nsub, "z", 3,
                                   cutoff=1e-12, maxdim=4)
    psi = O.product_mps(st, ["up"] * N)
    OA.tebd(st, psi, H, dt, nsub * dt, nsub * dt, cutoff=1e-12, maxdim=4, evol="real")
    ob = O.OpList(N)
    ob.add(["z"], [3], 1.0)
    ref = float(np.real(np.sum(O.inner(st, psi, ob, psi))))
    assert abs(f - ref) < 1e-12


def test_rrule_chains_gate_cotangents_to_parameters(monkeypatch):
    """TEBDGradProblem.rrule turns per-gate cotangents df/dconj(G) into
    df/dh_k = Re sum conj(gbar) dG/dh_k, with dG/dh_k from the Frechet
    derivative; checked with the library call replaced by a linear stand-in
    f = Re sum_k sum_g <C_g, G_g(h_k)> whose gradient is known."""
    import tngpu.algorithms as A
    import tngpu.models as M
    N, dt, nsub = 4, 0.05, 2
    st = M.spinhalf()
    H_of = _ising(M, N)
    prob = A.TEBDGradProblem(st, H_of, dt, nsub, "z", 2)
    hs = np.array([0.3, 0.7])
    rng = np.random.default_rng(1)
    rows = [M.trotter_rows(st, H_of(h), dt, 2, "real") for h in hs]
    cots = [rng.standard_normal(g.shape) + 1j * rng.standard_normal(g.shape)
            for r in rows for _, gs in r for g in gs]

    def f_of(h):
        rr = [M.trotter_rows(st, H_of(x), dt, 2, "real") for x in h]
        gates = [g for r in rr for _, gs in r for g in gs]
        return float(sum(np.real(np.vdot(c, g)) for c, g in zip(cots, gates)))

    def fake_call(psi0, params, want):
        grads = np.concatenate([c.ravel(order="F") for c in cots]).view(np.float64)
        return f_of(params), rows, grads

    monkeypatch.setattr(prob, "_call", fake_call)
    f, back = prob.rrule(None, hs)
    g = back()
    e = 1e-6
    for k in range(len(hs)):
        hp, hm = hs.copy(), hs.copy()
        hp[k] += e
        hm[k] -= e
        fd = (f_of(hp) - f_of(hm)) / (2 * e)
        assert abs(g[k] - fd) <= 1e-7 * max(1.0, abs(fd)), (k, g[k], fd)
    assert f == f_of(hs)
    assert np.allclose(back(2.0), 2.0 * g)
