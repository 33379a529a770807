"""Known-answer physics used to pin the oracle.  Test infrastructure only.

Dense states use the column-major site order of the reference's dense
quantum states (structures/qs/gqs.jl): psi[s1, s2, ..., sN] with s1 fastest.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .core import fr

__all__ = ["mps_to_dense", "mpo_to_dense", "oplist_to_dense", "tfim_free_fermion_energy",
           "apply_rows_dense", "lindblad_evolve", "dense_expect"]


def mps_to_dense(psi):
    """Contract an MPS into psi[s1..sN] (returned flattened column-major)."""
    t = psi[1]
    for i in range(2, len(psi) + 1):
        t = np.tensordot(t, psi[i], axes=([t.ndim - 1], [0]))
    t = t[0, ..., 0]
    return fr(t, (-1,))


def oplist_to_dense(st, H):
    """Dense operator of an OpList, built term by term as QO(st, H) does
    (structures/qs/qo.jl:224-242).  Matrix rows/cols use column-major site
    order (site 1 fastest), so the Kronecker order is reversed."""
    N, d = H.length, st.dim
    out = np.zeros((d ** N, d ** N), dtype=np.complex128)
    for ops, sites, c in zip(H.ops, H.sites, H.coeffs):
        m = np.ones((1, 1), dtype=np.complex128)
        for j in range(N, 0, -1):
            o = st.op(ops[sites.index(j)]) if j in sites else np.eye(d)
            m = np.kron(m, o)
        out += c * m
    return out


def mpo_to_dense(O):
    """Dense matrix of an MPO W[wl, s_out, s_in, wr]."""
    N = len(O)
    t = O[1][0]  # [so, si, wr]
    d = t.shape[0]
    M = t  # [(out...), (in...), w]
    outdim = d
    for i in range(2, N + 1):
        W = O[i]
        M = np.einsum("abw,wcdx->acbdx", M, W)  # out_old, out_new, in_old, in_new
        outdim *= d
        M = fr(M, (outdim, outdim, W.shape[3]))
    return M[:, :, 0]


def tfim_free_fermion_energy(N, J, h):
    """Ground energy of H = -J sum X_i X_{i+1} - h sum Z_i (open chain, which is
    unitarily equivalent to -J sum Z Z - h sum X) from the Jordan-Wigner
    quadratic form: E0 = -h N + tr(A)/2 - sum_k Lambda_k / 2, Lambda the
    singular values of A - B (Lieb, Schultz & Mattis 1961; Pfeuty 1970)."""
    A = np.zeros((N, N))
    B = np.zeros((N, N))
    for i in range(N):
        A[i, i] = 2 * h
    for i in range(N - 1):
        A[i, i + 1] = A[i + 1, i] = -J
        B[i, i + 1] = -J
        B[i + 1, i] = J
    lam = np.linalg.svd(A - B, compute_uv=False)
    return -h * N + 0.5 * np.trace(A) - 0.5 * np.sum(lam)


def apply_rows_dense(vec, rows, N, d):
    """Apply Trotter rows to a dense state without truncation, in list order
    (the dense-state path of gatelist.jl:230-255)."""
    t = fr(vec, (d,) * N)
    for sites, gates in rows:
        for s, g in zip(sites, gates):
            n = g.ndim // 2
            axes_in = [s - 1 + k for k in range(n)]
            t = np.tensordot(g, t, axes=([2 * k + 1 for k in range(n)], axes_in))
            # result axes: outputs (n) followed by the remaining state axes
            rest = [a for a in range(N) if a not in axes_in]
            order = [0] * N
            for k, a in enumerate(axes_in):
                order[a] = k
            for k, a in enumerate(rest):
                order[a] = n + k
            t = np.transpose(t, order)
    return fr(t, (-1,))


def dense_expect(vec, op_dense):
    return np.vdot(vec, op_dense @ vec) / np.vdot(vec, vec)


def lindblad_evolve(H, Ls, rho0, times):
    """Exact Lindblad evolution d rho/dt = -i[H,rho] + sum L rho L^dag -
    1/2 {L^dag L, rho} by exponentiating the vectorised generator."""
    n = H.shape[0]
    I = np.eye(n)
    # column-stacking vec: vec(A X B) = (B^T kron A) vec(X)
    Lg = -1j * (np.kron(I, H) - np.kron(H.T, I))
    for L in Ls:
        LdL = L.conj().T @ L
        Lg += np.kron(L.conj(), L) - 0.5 * np.kron(I, LdL) - 0.5 * np.kron(LdL.T, I)
    v0 = rho0.reshape(-1, order="F")
    out = []
    for t in times:
        out.append((sla.expm(Lg * t) @ v0).reshape(n, n, order="F"))
    return out
