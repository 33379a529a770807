"""Mixed-precision path: the 3xTF32 tcgen05 GEMM and the H_eff product built
on it, compared with FP64 references.  Tolerance: 3xTF32 products with FP32
accumulation reach ~1e-6 relative; the tests allow 2e-5 relative in the
Frobenius norm."""

import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.fixture(scope="module")
def tn():
    import tngpu
    return tngpu


def crand(rng, *shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("m,n,k,conj", [(128, 128, 32, 0), (1, 1, 1, 0), (200, 77, 45, 0),
                                        (300, 260, 1030, 1), (64, 513, 257, 1), (1024, 640, 2048, 0)])
def test_tc_gemm(tn, m, n, k, conj):
    ctx = tn.context()
    rng = np.random.default_rng(m + n + k)
    A = crand(rng, k, m) if conj else crand(rng, m, k)
    B = crand(rng, k, n)
    Cg = np.zeros((m, n), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_gemm(ctx.h, m, n, k, dp(A), conj, dp(B), dp(Cg), 1))
    ref = (A.conj().T if conj else A) @ B
    assert rel(Cg, ref) < TOL
    # the FP64 path of the same entry point is exact to rounding
    C64 = np.zeros_like(Cg)
    ctx.check(ctx.lib.tn_gemm(ctx.h, m, n, k, dp(A), conj, dp(B), dp(C64), 0))
    assert rel(C64, ref) < 1e-13


@pytest.mark.parametrize("cl,cr,w", [(1, 4, 5), (37, 19, 5), (128, 128, 5), (300, 200, 3), (512, 512, 5)])
def test_heff2_mixed(tn, cl, cr, w):
    ctx = tn.context()
    rng = np.random.default_rng(cl * 7 + cr)
    d = 2
    wl = 1 if cl == 1 else w
    L, W1, W2 = crand(rng, cl, wl, cl), crand(rng, wl, d, d, w), crand(rng, w, d, d, w)
    R, th = crand(rng, cr, w, cr), crand(rng, cl, d, d, cr)
    out = np.zeros((cl, d, d, cr), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_heff2_apply(ctx.h, cl, cr, d, wl, w, w, dp(L), dp(W1), dp(W2), dp(R),
                                     dp(th), dp(out), 1))
    ref = O.core.heff2(L, W1, W2, R, th)
    assert rel(out, ref) < TOL


def _xxz(tn, N):
    H = tn.OpList(N)
    for i in range(1, N):
        for o in "xyz":
            H.add([o, o], [i, i + 1], 1.0)
    return H


@pytest.mark.parametrize("precision", ["mixed", "mixed-env64"])
def test_dmrg_mixed_matches_fp64(tn, precision):
    """Mixed-precision DMRG (3xTF32 matvecs and projections; environments in
    3xTF32 or FP64; FP64 Lanczos and truncation) against the plain FP64 run
    from the same state: |dE/E| <= 1e-9 on the FP64-recomputed energy.  Kept
    bond dimensions set by the 1e-12 cutoff may differ by a few where sigma^2
    sits at the cutoff: the 3xTF32 H_eff products perturb the state at ~1e-7
    in both modes."""
    N, D = 24, 8
    rng = np.random.default_rng(3)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    draws = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    draws.append(O.fr(rng.standard_normal(4), (1, 2, 2)))
    po = O.random_mps(2, N, D, draws)
    W = tn.MPO(tn.spinhalf(), _xxz(tn, N))
    kw = dict(maxdim=128, cutoff=1e-12, minsweeps=8, maxsweeps=8, numconverges=np.inf, verbose=False)
    p64 = tn.GMPS.from_tensors(po.tensors, po.center)
    st64 = {}
    tn.dmrg(p64, W, stats=st64, **kw)
    E64 = st64["energy_fp64"]  # FP64 <psi|H|psi> of the FP64 run's final state
    pmx = tn.GMPS.from_tensors(po.tensors, po.center)
    st = {}
    _, Emx = tn.dmrg(pmx, W, precision=precision, stats=st, **kw)
    assert abs(st["energy_fp64"] - E64) <= 1e-9 * abs(E64), (st["energy_fp64"], E64, Emx)
    assert Emx == st["energy_fp64"]  # mixed modes return the FP64 Rayleigh quotient
    assert abs(max(pmx.bonddims()) - max(p64.bonddims())) <= 4


@pytest.mark.parametrize("cl,cr,wl,wr", [(1, 2, 1, 5), (9, 17, 5, 5), (64, 96, 5, 5), (300, 256, 5, 3)])
def test_env_updates_mixed(tn, cl, cr, wl, wr):
    ctx = tn.context()
    rng = np.random.default_rng(11 + cl)
    d = 2
    A, W = crand(rng, cl, d, cr), crand(rng, wl, d, d, wr)
    L, R = crand(rng, cl, wl, cl), crand(rng, cr, wr, cr)
    outl = np.zeros((cr, wr, cr), dtype=np.complex128, order="F")
    outr = np.zeros((cl, wl, cl), dtype=np.complex128, order="F")
    ctx.check(ctx.lib.tn_env_left(ctx.h, cl, cr, d, wl, wr, dp(L), dp(A), dp(W), dp(outl), 1))
    ctx.check(ctx.lib.tn_env_right(ctx.h, cl, cr, d, wl, wr, dp(R), dp(A), dp(W), dp(outr), 1))
    assert rel(outl, O.core.env_left(L, A, W, A)) < TOL
    assert rel(outr, O.core.env_right(R, A, W, A)) < TOL


def test_tebd_mixed_matches_fp64(tn):
    """Mixed TEBD (3xTF32 two-site contractions and truncation projections)
    against FP64 from the same state: local <Z_i> and the centre entropy to
    1e-5 (3e-6 measured after five steps at chi 128), identical bond
    dimensions."""
    N, D = 14, 128
    rng = np.random.default_rng(21)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    draws = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    draws.append(O.fr(rng.standard_normal(4), (1, 2, 2)))
    po = O.random_mps(2, N, D, draws)
    H = tn.OpList(N)
    for i in range(1, N):
        for o, c in (("x", 1.0), ("y", 1.0), ("z", 0.5)):
            H.add([o, o], [i, i + 1], c)
    Z = tn.OpList(N)
    for i in range(1, N + 1):
        Z.add("z", i)
    st = tn.spinhalf()
    out = {}
    for prec in ("fp64", "mixed"):
        p = tn.GMPS.from_tensors(po.tensors, po.center)
        tn.tebd(st, p, H, 0.05, 0.25, 0.25, cutoff=1e-14, maxdim=D, evol="real", precision=prec)
        out[prec] = (np.real(tn.inner(st, p, Z, p)), p.entropy(N // 2), p.bonddims())
    z64, s64, d64 = out["fp64"]
    zmx, smx, dmx = out["mixed"]
    assert max(d64) == D
    assert dmx == d64
    assert np.max(np.abs(zmx - z64)) <= 1e-5, np.max(np.abs(zmx - z64))
    assert abs(smx - s64) <= 1e-5, (smx, s64)


def test_dmrg_fp64_residual_refinement(tn):
    """refine (mixed modes): each bond's Ritz vector gets refinement steps
    against its FP64 residual, one Lanczos cycle each whose first product is
    FP64 and fixes the projected matrix's first row.  From a state converged
    by FP64 DMRG, one mixed-env64 sweep pair without and with two refinement
    steps; the FP64 residual norms of the split vectors come back per bond.
    Without refinement the residual reported after equals the one before
    (the same vector); with it the median residual falls at least 3x and the
    largest does not grow; both energies stay within 1e-9 of FP64.  FP64
    mode rejects refine (its Lanczos is the reference's)."""
    N, D = 16, 8
    rng = np.random.default_rng(5)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    draws = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    draws.append(O.fr(rng.standard_normal(4), (1, 2, 2)))
    po = O.random_mps(2, N, D, draws)
    W = tn.MPO(tn.spinhalf(), _xxz(tn, N))
    kw = dict(maxdim=64, cutoff=1e-12, numconverges=np.inf, verbose=False)
    p = tn.GMPS.from_tensors(po.tensors, po.center)
    st = {}
    tn.dmrg(p, W, minsweeps=6, maxsweeps=6, stats=st, **kw)
    E64 = st["energy_fp64"]
    tensors, center = p.tensors(), p.center
    res = {}
    for r in (0, 2):
        q = tn.GMPS.from_tensors(tensors, center)
        s = {}
        tn.dmrg(q, W, minsweeps=2, maxsweeps=2, precision="mixed-env64", refine=r, residuals=True,
                stats=s, **kw)
        res[r] = (np.array(s["bond_resid_in"]), np.array(s["bond_resid_out"]), s["energy_fp64"])
        assert len(res[r][0]) == 2 * (N - 1) and np.all(res[r][0] > 0)
        assert abs(s["energy_fp64"] - E64) <= 1e-9 * abs(E64), (r, s["energy_fp64"], E64)
    rin0, rout0, _ = res[0]
    rin, rout, _ = res[2]
    print("refine=0 resid:", np.median(rin0), rin0.max())
    print("refine=2 resid in/out:", np.median(rin), rin.max(), np.median(rout), rout.max())
    assert np.array_equal(rin0, rout0)
    assert np.median(rout) <= np.median(rin) / 3
    assert rout.max() <= rin.max()
    q = tn.GMPS.from_tensors(tensors, center)
    with pytest.raises(tn.TNError, match="refine"):
        tn.dmrg(q, W, minsweeps=1, maxsweeps=1, refine=1, **kw)
