"""The library's FP64 Hermitian eigensolver (tn_eigh_top) against
numpy.linalg.eigh.

It sets the cut of every truncated split in place of LAPACK's SVD
(tensors.jl:191-195 via the Gram matrix), so it must give eigenvalues to
FP64 accuracy (absolute, a few ulps of |G|), orthonormal eigenvectors with
small residuals, and the exact top-k invariant subspace wherever the spectrum
has a gap there.  The cases cover full and partial spectra, graded
rank-deficient Gram matrices (the DMRG shape: most eigenvalues at the FP64
noise floor) and exactly degenerate multiplets."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import tngpu
    return tngpu.context()


def _eigh_top(ctx, G, want):
    n = G.shape[0]
    Gf = np.asfortranarray(G.astype(np.complex128))
    lam = np.zeros(want)
    V = np.zeros((n, want), dtype=np.complex128, order="F")
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ctx.check(ctx.lib.tn_eigh_top(ctx.h, n, dp(Gf), want, dp(lam), dp(V)))
    return lam, V


def _check(G, lam, V, tol=1e-12):
    n, want = V.shape
    ref = np.linalg.eigvalsh(G)[::-1][:want]
    nrm = max(np.abs(np.linalg.eigvalsh(G)).max(), 1e-300)
    assert np.all(np.diff(lam) <= 1e-12 * nrm)  # descending
    assert np.abs(lam - ref).max() <= 64 * n * 2.2e-16 * nrm
    assert np.abs(V.conj().T @ V - np.eye(want)).max() <= tol * max(1, n / 64)
    res = np.linalg.norm(G @ V - V * lam) / nrm
    assert res <= 1e-12 * np.sqrt(n * want)
    return ref


def _random_hermitian(rng, n):
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return 0.5 * (A + A.conj().T)


@pytest.mark.parametrize("n,want", [(1, 1), (2, 2), (3, 1), (17, 17), (64, 20), (200, 200),
                                    (513, 100)])
def test_eigh_random_hermitian(ctx, n, want):
    rng = np.random.default_rng(n)
    G = _random_hermitian(rng, n)
    lam, V = _eigh_top(ctx, G, want)
    _check(G, lam, V)


@pytest.mark.parametrize("n,rank,want", [(96, 12, 40), (300, 40, 100), (700, 90, 350)])
def test_eigh_graded_rank_deficient_gram(ctx, n, rank, want):
    """G = M M^H with a geometrically graded spectrum over 1e-14 and a null
    space: the kept subspace beyond the rank is the null space, whose basis
    is arbitrary; the top `rank` subspace must match exactly."""
    rng = np.random.default_rng(rank)
    M = rng.standard_normal((n, rank)) + 1j * rng.standard_normal((n, rank))
    M, _ = np.linalg.qr(M)
    s = np.logspace(0, -7, rank)  # sigma^2 over 1e-14
    G = (M * s**2) @ M.conj().T
    lam, V = _eigh_top(ctx, G, want)
    _check(G, lam, V)
    # FP64 fixes an eigenvector to eps |G| / gap, so the top-r projector is
    # exact where the gap is large (eigenvalues above 1e-4: error ~1e-12) ...
    r = int(np.sum(s**2 > 1e-4))
    P = V[:, :r] @ V[:, :r].conj().T
    Pr = (M[:, :r]) @ M[:, :r].conj().T
    assert np.abs(P - Pr).max() < 1e-9
    # ... and the null-space vectors are orthogonal to the range directions
    # above 1e-8 (the 1e-14 ones are only 1e-14 from the null space)
    big = s**2 > 1e-8
    assert np.abs(M[:, big].conj().T @ V[:, rank:]).max() < 1e-6


def test_eigh_exact_multiplets(ctx):
    """Degenerate multiplets (as SU(2) symmetry gives the entanglement
    spectrum of the Heisenberg chain): each multiplet's eigenspace must be
    returned as an orthonormal basis of that eigenspace."""
    rng = np.random.default_rng(7)
    n = 160
    mult = [1, 3, 5, 3, 1, 7, 3, 5, 1, 9]
    vals = []
    for k, m in enumerate(mult):
        vals += [10.0 ** (-k)] * m
    vals += [0.0] * (n - len(vals))
    U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    G = (U * np.asarray(vals)) @ U.conj().T
    want = len(vals) - vals.count(0.0) + 10
    lam, V = _eigh_top(ctx, G, want)
    _check(G, lam, V)
    start = 0
    for k, m in enumerate(mult):
        Ue = U[:, start:start + m]
        Ve = V[:, start:start + m]
        # same eigenspace: the overlap matrix is unitary, to eps / gap with a
        # gap of 0.9 x 10^-k to the next multiplet
        O = Ue.conj().T @ Ve
        assert np.abs(O @ O.conj().T - np.eye(m)).max() < 1e-12 * 10.0**k, (k, m)
        start += m


def test_eigh_diagonal_and_zero(ctx):
    G = np.diag([3.0, 1.0, 2.0, 0.0, 0.0]).astype(np.complex128)
    lam, V = _eigh_top(ctx, G, 5)
    assert np.allclose(lam, [3, 2, 1, 0, 0], atol=1e-15)
    assert np.abs(V.conj().T @ V - np.eye(5)).max() < 1e-14
    lam, V = _eigh_top(ctx, np.zeros((4, 4), dtype=np.complex128), 2)
    assert np.allclose(lam, 0.0, atol=1e-300)
    assert np.abs(V.conj().T @ V - np.eye(2)).max() < 1e-14
