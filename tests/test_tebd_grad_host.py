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
