"""Oracle core: site types, operator lists, the truncated SVD rule, GMPS gauge
moves, the MPO builder and the environment cache.  Test infrastructure only.

Every array is complex128 and every reshape is column-major (order='F') so the
index bookkeeping reads like the Julia source it restates.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla

__all__ = [
    "Sitetypes", "spinhalf", "OpList", "svd_keep", "trunc_svd", "GMPS",
    "random_mps", "product_mps", "mpo_from_oplist", "ProjMPS", "inner",
    "applyop", "totensor", "sitetensor", "siterange", "siteindexs", "fr",
    "ProjMPSSum", "overlap", "scaled", "mpo_mps_product", "product_mpo", "adjoint_mpo", "mpo_mpo_product", "trace_mpos", "MPSProjector",
]


def fr(x, shape):
    """Column-major reshape (Julia ``reshape``)."""
    return np.reshape(x, shape, order="F")


# ---------------------------------------------------------------------------
# Site types (src/sitetypes.jl:1-166, src/lattices/spinhalf.jl:1-23)
# ---------------------------------------------------------------------------
class Sitetypes:
    """Named local states and operators (sitetypes.jl:1-18)."""

    def __init__(self, dim):
        self.dim = dim
        self.statenames, self.states = [], []
        self.opnames, self.ops, self.opdags = [], [], []
        self.temp = 0

    def add_state(self, name, vec):
        vec = np.asarray(vec, dtype=np.complex128)
        if vec.shape != (self.dim,):
            raise ValueError(f"The vector must be dimension {self.dim}.")
        if name in self.statenames:
            raise ValueError(f"The state name {name} already exists.")
        self.statenames.append(name)
        self.states.append(vec)

    def add_op(self, name, mat, dag="None"):
        mat = np.asarray(mat, dtype=np.complex128)
        if mat.shape != (self.dim, self.dim):
            raise ValueError(f"The matrix must be dimensions ({self.dim}, {self.dim}).")
        if name in self.opnames:
            raise ValueError(f"The operator name {name} already exists.")
        self.opnames.append(name)
        self.ops.append(mat)
        self.opdags.append(dag)

    def state(self, name):
        """sitetypes.jl:27-37"""
        if name not in self.statenames:
            raise KeyError(f"The state {name} is undefined.")
        return self.states[self.statenames.index(name)].copy()

    def op(self, name):
        """sitetypes.jl:45-55"""
        if name not in self.opnames:
            raise KeyError(f"The operator {name} is undefined.")
        return self.ops[self.opnames.index(name)].copy()

    def dag(self, name):
        """sitetypes.jl:62-72"""
        if name not in self.opnames:
            raise KeyError(f"The operator {name} is undefined.")
        return self.opdags[self.opnames.index(name)]

    def opprod(self, names):
        """Name of the product of operators; first stored match within 1e-12
        in summed absolute difference, else a new temp pair (sitetypes.jl:144-166)."""
        prod = None
        for i, n in enumerate(names):
            prod = self.op(n) if i == 0 else prod @ self.op(n)
        for i, o in enumerate(self.ops):
            if np.sum(np.abs(prod - o)) < 1e-12:
                return self.opnames[i]
        dagm = np.conj(prod.T)
        name, dagname = f"temp{self.temp}", f"temp{self.temp + 1}"
        self.add_op(name, prod, dagname)
        self.add_op(dagname, dagm, name)
        self.temp += 2
        return name


def spinhalf():
    """Spin-1/2 site type (lattices/spinhalf.jl:1-23)."""
    st = Sitetypes(2)
    st.add_state("up", [1, 0])
    st.add_state("dn", [0, 1])
    st.add_state("s", [0.5 ** 0.5, 0.5 ** 0.5])
    st.add_state("as", [0.5 ** 0.5, -0.5 ** 0.5])
    st.add_op("x", [[0, 1], [1, 0]], "x")
    st.add_op("y", [[0, -1j], [1j, 0]], "y")
    st.add_op("z", [[1, 0], [0, -1]], "z")
    st.add_op("id", [[1, 0], [0, 1]], "id")
    st.add_op("pu", [[1, 0], [0, 0]], "pu")
    st.add_op("pd", [[0, 0], [0, 1]], "pd")
    st.add_op("n", [[1, 0], [0, 0]], "n")
    st.add_op("s+", [[0, 1], [0, 0]], "s-")
    st.add_op("s-", [[0, 0], [1, 0]], "s+")
    return st


# ---------------------------------------------------------------------------
# Operator lists (structures/mps/oplist.jl:1-183)
# ---------------------------------------------------------------------------
class OpList:
    """Sum of products of local operators (oplist.jl:1-13); sites are 1-based."""

    def __init__(self, length):
        self.length = length
        self.ops, self.sites, self.coeffs = [], [], []

    def add(self, ops, sites, coeff=1.0):
        """oplist.jl:33-55 (terms sorted by site, validated)."""
        if isinstance(ops, str):
            ops, sites = [ops], [sites]
        if len(ops) != len(sites):
            raise ValueError("The lists must be the same length.")
        perm = np.argsort(sites, kind="stable")
        sites = [int(sites[p]) for p in perm]
        ops = [ops[p] for p in perm]
        last = 0
        for s in sites:
            if s < 0 or s > self.length:
                raise ValueError(f"The sites must be between 1 and {self.length}.")
            if sites.count(s) > 1:
                raise ValueError("There are two or more operators on the same site.")
            if s <= last:
                raise ValueError("The site list must be ordered.")
            last = s
        self.ops.append(list(ops))
        self.sites.append(sites)
        self.coeffs.append(complex(coeff))
        return self

    def scaled(self, c):
        """x * oplist (oplist.jl:80-94)."""
        o = OpList(self.length)
        o.ops = [list(x) for x in self.ops]
        o.sites = [list(x) for x in self.sites]
        o.coeffs = [complex(c) * x for x in self.coeffs]
        return o

    def __add__(self, other):
        """add(oplist1, oplist2) (oplist.jl:67-77)."""
        o = OpList(max(self.length, other.length))
        o.ops = [list(x) for x in self.ops + other.ops]
        o.sites = [list(x) for x in self.sites + other.sites]
        o.coeffs = list(self.coeffs) + list(other.coeffs)
        return o


def siterange(oplist):
    """oplist.jl:102-109"""
    rng = 1
    for s in oplist.sites:
        rng = max(rng, s[-1] - s[0] + 1)
    return rng


def siteindexs(oplist, site):
    """oplist.jl:117-125 (0-based term indices of terms starting at ``site``)."""
    return [i for i, s in enumerate(oplist.sites) if s[0] == site]


def totensor(oplist, st, idx):
    """Tensor [o1,i1,o2,i2,...] of one term padded with identities up to the
    list's range, clipped at the chain end (oplist.jl:134-156)."""
    ops, sites = oplist.ops[idx], oplist.sites[idx]
    rng = min(siterange(oplist), oplist.length - sites[0] + 1)
    prod = np.ones((1, 1), dtype=np.complex128)
    k = 0
    for s in range(1, rng + 1):
        if sites[0] + s - 1 in sites:
            name = ops[k]
            k += 1
        else:
            name = "id"
        o = fr(st.op(name), (1, st.dim, st.dim, 1))
        prod = np.tensordot(prod, o, axes=([prod.ndim - 1], [0]))
    prod = np.trace(prod, axis1=0, axis2=prod.ndim - 1)
    return oplist.coeffs[idx] * prod


def sitetensor(oplist, st, site):
    """Sum of all terms starting at ``site`` (oplist.jl:164-183); None if none."""
    idxs = siteindexs(oplist, site)
    if not idxs:
        return None
    ten = None
    for i in idxs:
        t = totensor(oplist, st, i)
        ten = t if ten is None else ten + t
    return ten


# ---------------------------------------------------------------------------
# Truncated SVD (src/tensors.jl:168-227)
# ---------------------------------------------------------------------------
def svd_keep(S, cutoff=0.0, maxdim=0, mindim=1):
    """Number of singular values kept (tensors.jl:200-215).

    ``findfirst(S == 0)`` at tensors.jl:205 compares a vector with a scalar and
    is a no-op, so zero singular values are not dropped by it."""
    sz = len(S)
    mindim = min(mindim, sz)
    maxdim = sz if (maxdim == 0 or maxdim > sz) else maxdim
    if maxdim == 0:
        maxdim = 1
    if cutoff != 0:
        S2 = S.astype(np.float64) ** 2
        with np.errstate(invalid="ignore", divide="ignore"):
            cum = np.cumsum(S2[::-1])[::-1] / np.sum(S2)
        hit = np.nonzero(cum > cutoff)[0]
        last = int(hit[-1]) + 1 if hit.size else 1
        maxdim = min(maxdim, last)
    return max(maxdim, mindim)


def _lapack_svd(M):
    """Divide and conquer, falling back to QR iteration (tensors.jl:189-195)."""
    try:
        return sla.svd(M, full_matrices=False, lapack_driver="gesdd")
    except np.linalg.LinAlgError:
        return sla.svd(M, full_matrices=False, lapack_driver="gesvd")


def trunc_svd(M, cutoff=0.0, maxdim=0, mindim=1):
    """SVD of a matrix with the reference keep rule; returns U, S, Vt truncated."""
    U, S, Vt = _lapack_svd(M)
    k = svd_keep(S, cutoff, maxdim, mindim)
    return U[:, :k], S[:k], Vt[:k, :]


# ---------------------------------------------------------------------------
# GMPS (structures/mps/gmps.jl, mps.jl)
# ---------------------------------------------------------------------------
class GMPS:
    """Rank-1 (MPS) or rank-2 (MPO) tensor train; ``center`` is 1-based, 0 =
    unset (gmps.jl:8-13)."""

    def __init__(self, rank, dim, tensors, center=0):
        self.rank, self.dim = rank, dim
        self.tensors = [np.asarray(t, dtype=np.complex128) for t in tensors]
        self.center = center

    def __len__(self):
        return len(self.tensors)

    def __getitem__(self, i):  # 1-based
        return self.tensors[i - 1]

    def __setitem__(self, i, x):
        self.tensors[i - 1] = x

    def copy(self):
        return GMPS(self.rank, self.dim, [t.copy() for t in self.tensors], self.center)

    def bonddims(self):
        """[1, chi_1, ..., chi_{N-1}, 1]"""
        return [self.tensors[0].shape[0]] + [t.shape[-1] for t in self.tensors]

    def maxbonddim(self):
        """abstractmps.jl:75-81"""
        return max([1] + [self[i + 1].shape[0] for i in range(1, len(self))])

    # -- gauge moves (gmps.jl:60-112) -------------------------------------
    def moveleft(self, idx, cutoff=0.0, maxdim=0, mindim=1):
        """SVD with the left bond as columns: M[(s,Dr),Dl] = A[Dl,s,Dr]
        (gmps.jl:60-67; tensors.jl:181-187 ordering)."""
        if 1 < idx <= len(self):
            A = self[idx]
            Dl = A.shape[0]
            M = fr(A, (Dl, -1)).T
            U, S, Vt = trunc_svd(M, cutoff, maxdim, mindim)
            k = S.size
            self[idx] = fr(U.T, (k,) + A.shape[1:])
            V = S[:, None] * Vt  # [k, Dl]
            B = self[idx - 1]
            self[idx - 1] = np.tensordot(B, V, axes=([B.ndim - 1], [1]))

    def moveright(self, idx, cutoff=0.0, maxdim=0, mindim=1):
        """SVD with the right bond as columns: M[(Dl,s),Dr] (gmps.jl:75-82)."""
        if 0 < idx < len(self):
            A = self[idx]
            Dr = A.shape[-1]
            M = fr(A, (-1, Dr))
            U, S, Vt = trunc_svd(M, cutoff, maxdim, mindim)
            k = S.size
            self[idx] = fr(U, A.shape[:-1] + (k,))
            V = S[:, None] * Vt  # [k, Dr]
            self[idx + 1] = np.tensordot(V, self[idx + 1], axes=([1], [0]))

    def movecenter(self, idx, **kw):
        """gmps.jl:90-112"""
        N = len(self)
        if idx < 1 or idx > N:
            raise IndexError("The index is out of range.")
        if self.center == 0:
            for i in range(1, idx):
                self.moveright(i, **kw)
            for i in range(1, N - idx + 1):
                self.moveleft(N + 1 - i, **kw)
        elif idx > self.center:
            for i in range(self.center, idx):
                self.moveright(i, **kw)
        elif idx < self.center:
            c = self.center
            for i in range(1, c - idx + 1):
                self.moveleft(c + 1 - i, **kw)
        self.center = idx

    def norm(self):
        """gmps.jl:29-37 (moves the centre to 1 when unset)."""
        if self.center == 0:
            self.movecenter(1)
        A = self[self.center]
        return np.sqrt(np.vdot(A, A))

    def normalize(self):
        """gmps.jl:46-51"""
        if self.center == 0:
            self.movecenter(1)
        self[self.center] = self[self.center] / self.norm()

    def entropy(self, site):
        """-sum s^2 ln s^2 of the untruncated SVD at the centre (gmps.jl:184-189)."""
        self.movecenter(site)
        A = self[site]
        S = _lapack_svd(fr(A, (-1, A.shape[-1])))[1]
        S2 = S ** 2
        # an exact zero gives 0 * -Inf = NaN, as in the reference
        with np.errstate(divide="ignore", invalid="ignore"):
            return float(-np.sum(S2 * np.log(S2)))

    def singular_values(self, site):
        """Spectrum across bond (site, site+1) after moving the centre there."""
        self.movecenter(site)
        A = self[site]
        return _lapack_svd(fr(A, (-1, A.shape[-1])))[1]

    def replacesites(self, theta, site, direction=False, normalize=False,
                     cutoff=0.0, maxdim=0, mindim=1):
        """Two-site split of theta[Dl,s1,s2,Dr] (gmps.jl:199-267).

        direction False (sweeping right): SVD of M[(s2,Dr),(Dl,s1)]; left site
        gets Vt rows as [Dl,s1,k], right site gets U*S as [k,s2,Dr]; centre =
        site+1.  direction True: SVD of M[(Dl,s1),(s2,Dr)]; left gets U*S,
        right gets Vt; centre = site.  One-site tensors take the nsites == 1
        branch (gmps.jl:204-213)."""
        if self.rank == 2 and theta.ndim == 6:
            # rank-2 two-site tensor [Dl, o1, i1, o2, i2, Dr]: the SVD groups
            # (Dl, o1, i1) against (o2, i2, Dr), the fused physical index
            # o + d i of each site (gmps.jl:199-267 with rank 2)
            Dl, d, _, _, _, Dr = theta.shape
            fused = GMPS(1, d * d, [fr(t, (t.shape[0], d * d, t.shape[-1])) for t in self.tensors],
                         self.center)
            fused.replacesites(fr(theta, (Dl, d * d, d * d, Dr)), site, direction, False,
                               cutoff=cutoff, maxdim=maxdim, mindim=mindim)
            self.tensors = [fr(t, (t.shape[0], d, d, t.shape[-1])) for t in fused.tensors]
            self.center = fused.center
            if normalize:
                self.normalize()
            return
        if theta.ndim == 3 or (self.rank == 2 and theta.ndim == 4):
            self[site] = theta
            nxt = site + 1 - 2 * int(direction)
            if 0 < nxt <= len(self):
                self.movecenter(nxt)
            if normalize:
                self.normalize()
            return
        Dl, d1, d2, Dr = theta.shape
        if not direction:
            M = fr(theta, (Dl * d1, d2 * Dr)).T
            U, S, Vt = trunc_svd(M, cutoff, maxdim, mindim)
            k = S.size
            self[site + 1] = fr((U * S[None, :]).T, (k, d2, Dr))
            self[site] = fr(Vt.T, (Dl, d1, k))
            self.center = site + 1
        else:
            M = fr(theta, (Dl * d1, d2 * Dr))
            U, S, Vt = trunc_svd(M, cutoff, maxdim, mindim)
            k = S.size
            self[site] = fr(U * S[None, :], (Dl, d1, k))
            self[site + 1] = fr(Vt, (k, d2, Dr))
            self.center = site
        if normalize:
            self.normalize()


def random_mps(dim, N, bonddim, rng_or_tensors):
    """randomGMPS (gmps.jl:276-291): i.i.d. real normal site tensors with bond
    dim ``bonddim`` (edges 1); movecenter!(N); movecenter!(1); site 1 replaced
    by a fresh normal [1, d, min(d, bonddim)] tensor; normalize!.

    ``rng_or_tensors`` is either a numpy Generator (draws filled in
    column-major order) or an explicit list of N+1 real arrays (the N site
    tensors followed by the replacement first site)."""
    shapes = [((1 if i == 0 else bonddim), dim, (1 if i == N - 1 else bonddim)) for i in range(N)]
    first = (1, dim, min(dim, bonddim))
    if isinstance(rng_or_tensors, np.random.Generator):
        g = rng_or_tensors
        draws = [fr(g.standard_normal(int(np.prod(s))), s) for s in shapes]
        draws.append(fr(g.standard_normal(int(np.prod(first))), first))
    else:
        draws = [np.asarray(t, dtype=np.float64) for t in rng_or_tensors]
    psi = GMPS(1, dim, draws[:N], 0)
    psi.movecenter(N)
    psi.movecenter(1)
    psi[1] = draws[N].astype(np.complex128)
    psi.normalize()
    return psi


def product_mps(st, names):
    """productMPS(st, names) (mps.jl:68-76); centre unset."""
    return GMPS(1, st.dim, [fr(st.state(n), (1, st.dim, 1)) for n in names], 0)


# ---------------------------------------------------------------------------
# MPO from an operator list (structures/mps/mpo.jl:323-470)
# ---------------------------------------------------------------------------
def _expand(O, D1, D2):
    """mpo.jl:462-470"""
    a, d, _, b = O.shape
    new = np.zeros((a + D1, d, d, b + D2), dtype=np.complex128)
    d1 = 1 if a == 1 else a - 1
    new[:d1, :, :, :b - 1] = O[:d1, :, :, :b - 1]
    new[:d1, :, :, -1] = O[:d1, :, :, -1]
    new[a + D1 - 1, :, :, b + D2 - 1] = O[a - 1, :, :, b - 1]
    return new


def mpo_from_oplist(st, H, cutoff=1e-15, maxdim=0, mindim=1):
    """Finite-state-machine MPO assembly followed by a left-to-right then
    right-to-left truncated-SVD compression (mpo.jl:323-459)."""
    N, d = H.length, st.dim
    ten = np.zeros((2, d, d, 2), dtype=np.complex128)
    ten[0, :, :, 0] = st.op("id")
    ten[1, :, :, 1] = st.op("id")
    O = [None] * N
    O[0] = ten[0:1, :, :, 0:2].copy()
    for i in range(1, N - 1):
        O[i] = ten.copy()
    O[N - 1] = ten[0:2, :, :, 1:2].copy()

    maxrng = siterange(H)
    rngs = [[] for _ in range(maxrng)]
    for i in range(len(H.ops)):
        rngs[H.sites[i][-1] - H.sites[i][0]].append(i)

    for i in range(1, maxrng + 1):
        nextterms = [[] for _ in range(i)]
        coeffs = [[] for _ in range(i)]
        ingoings = [[] for _ in range(i)]
        outgoings = [[] for _ in range(i)]
        for site in range(1, N + 1):
            idxs = [j for j in rngs[i - 1] if H.sites[j][0] == site]
            if i == 1:
                for idx in idxs:
                    O[site - 1][0, :, :, -1] += H.coeffs[idx] * st.op(H.ops[idx][0])
                continue
            for j in idxs:
                ops, sites = H.ops[j], H.sites[j]
                outgoing = 0
                for k in range(1, i + 1):
                    ingoing = outgoing
                    for l in range(1, len(outgoings[k - 1]) + 2):
                        outgoing = l
                        if outgoing not in outgoings[k - 1]:
                            break
                    outgoing = 0 if k == i else outgoing
                    s = site + k - 1
                    opn = ops[sites.index(s)] if s in sites else "id"
                    nextterms[k - 1].append(opn)
                    coeffs[k - 1].append(H.coeffs[j] if k == 1 else 1.0)
                    ingoings[k - 1].append(ingoing)
                    outgoings[k - 1].append(outgoing)
            terms, ins, outs, cos = nextterms[0], ingoings[0], outgoings[0], coeffs[0]
            for j in range(i - 1):
                nextterms[j], ingoings[j] = nextterms[j + 1], ingoings[j + 1]
                outgoings[j], coeffs[j] = outgoings[j + 1], coeffs[j + 1]
            nextterms[i - 1], ingoings[i - 1], outgoings[i - 1], coeffs[i - 1] = [], [], [], []
            if terms:
                inlen = sum(1 for x in ins if x != 0)
                outlen = sum(1 for x in outs if x != 0)
                instart = O[site - 1].shape[0] - 1
                outstart = O[site - 1].shape[3] - 1
                O[site - 1] = _expand(O[site - 1], inlen, outlen)
                for j in range(len(terms)):
                    x = 1 if ins[j] == 0 else instart + ins[j]
                    y = outstart + 1 + outlen if outs[j] == 0 else outstart + outs[j]
                    O[site - 1][x - 1, :, :, y - 1] = cos[j] * st.op(terms[j])

    for site in range(N - 1):
        M = O[site]
        a, _, _, b = M.shape
        U, S, Vt = trunc_svd(fr(M, (-1, b)), cutoff, maxdim, mindim)
        k = S.size
        O[site] = fr(U * S[None, :], (a, d, d, k))
        O[site + 1] = np.tensordot(Vt, O[site + 1], axes=([1], [0]))
    for site in range(N - 1, 0, -1):
        M = O[site]
        a = M.shape[0]
        U, S, Vt = trunc_svd(fr(M, (a, -1)).T, cutoff, maxdim, mindim)
        k = S.size
        O[site] = fr((U * S[None, :]).T, (k,) + M.shape[1:])
        O[site - 1] = np.tensordot(O[site - 1], Vt, axes=([3], [1]))
    return GMPS(2, d, O, 0)


# ---------------------------------------------------------------------------
# Environment cache (structures/mps/projmps.jl, abstractprojmps.jl)
# ---------------------------------------------------------------------------
def _edge(n):
    return np.ones((1,) * n, dtype=np.complex128)


def env_left(L, A, W, B):
    """L'[a',w',b'] = sum L[a,w,b] conj(A[a,s',a']) W[w,s',s,w'] B[b,s,b']
    (projmps.jl:50-66).  W None gives the rank-1 overlap block L'[a',b']."""
    if W is None:
        t = np.tensordot(L, np.conj(A), axes=([0], [0]))            # b, s, a'
        return np.tensordot(t, B, axes=([0, 1], [0, 1]))            # a', b'
    t = np.tensordot(L, np.conj(A), axes=([0], [0]))                # w, b, s', a'
    t = np.tensordot(t, W, axes=([0, 2], [0, 1]))                   # b, a', s, w'
    t = np.tensordot(t, B, axes=([0, 2], [0, 1]))                   # a', w', b'
    return t


def env_right(R, A, W, B):
    """R[a,w,b] = sum B[b,s,b'] R[a',w',b'] W[w,s',s,w'] conj(A[a,s',a'])
    (projmps.jl:74-95)."""
    if W is None:
        t = np.tensordot(B, R, axes=([2], [1]))                     # b, s, a'
        return np.tensordot(np.conj(A), t, axes=([1, 2], [1, 2]))   # a, b
    t = np.tensordot(B, R, axes=([2], [2]))                         # b, s, a', w'
    t = np.tensordot(W, t, axes=([2, 3], [1, 3]))                   # w, s', b, a'
    t = np.tensordot(np.conj(A), t, axes=([1, 2], [1, 3]))          # a, w, b
    return t


def heff2(L, W1, W2, R, theta):
    """Two-site effective Hamiltonian product (projmps.jl:103-145, rank-2 branch):
    out[a,s1',s2',c'] = sum L[a,w,b] W1[w,s1',s1,w'] W2[w',s2',s2,w'']
    theta[b,s1,s2,c] R[c',w'',c]."""
    t = np.tensordot(L, theta, axes=([2], [0]))              # a w s1 s2 c
    t = np.einsum("awijc,wpiv,vqjx->apqxc", t, W1, W2, optimize=True)
    return np.tensordot(t, R, axes=([3, 4], [1, 2]))          # a p q c'


def heff2_reference_order(L, W1, W2, R, theta):
    """The same product in the reference's contraction order
    (projmps.jl:103-145, rank-2 branch): the left block is contracted with
    the MPO tensors first (prod[a, b, s1', s1, s2', s2, w''], chi^2 d^4 w
    entries; projmps.jl:116-130), then with the two-site tensor over (b, s1,
    s2) (projmps.jl:133) and with the right block over (w'', c)
    (projmps.jl:134-135): about 2.5x the flops of heff2's order at chi=1024,
    w=5.  The CPU baseline times this order."""
    prod = np.transpose(L, (0, 2, 1))                                   # a b w
    prod = np.tensordot(prod, W1, axes=([2], [0]))                      # a b s1' s1 w'
    prod = np.tensordot(prod, W2, axes=([4], [0]))                      # a b s1' s1 s2' s2 w''
    prod = np.tensordot(prod, theta, axes=([1, 3, 5], [0, 1, 2]))       # a s1' s2' w'' c
    return np.tensordot(prod, R, axes=([3, 4], [1, 2]))                 # a s1' s2' c'


def product_mpo(st, names):
    """productMPO(st, names) (mpo.jl:85-93): sites [1, d, d, 1] of the named
    operators, centre unset."""
    return GMPS(2, st.dim, [fr(st.op(n), (1, st.dim, st.dim, 1)) for n in names], 0)


def adjoint_mpo(O):
    """adjoint(O) (mpo.jl:32-39): every site conjugated with its two physical
    indices swapped."""
    out = O.copy()
    out.tensors = [np.conj(np.transpose(t, (0, 2, 1, 3))) for t in O.tensors]
    return out


def mpo_mpo_product(O1, O2, cutoff=0.0, maxdim=0, mindim=1):
    """MPOMPOProduct(O1, O2; kwargs) (mpo.jl:147-167): sites
    M[(a, b), o, i, (a', b')] = sum_k O1[a, o, k, a'] O2[b, k, i, b'] (a
    fastest in each pair), left-canonicalised while they are built, then the
    centre moved to site 1 with the truncation."""
    N = len(O1)
    ts = []
    for i in range(1, N + 1):
        M = np.einsum("aokx,bkiy->aboixy", O1[i], O2[i])
        da, db, d, _, dx, dy = M.shape
        ts.append(fr(M, (da * db, d, d, dx * dy)))
    O = GMPS(2, O1.dim, ts, 0)
    for i in range(1, N):
        O.moveright(i)
    O.center = 0
    O.movecenter(1, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
    return O


def trace_mpos(*ops):
    """trace(O1, ..., Ok) = Tr(O1 O2 ... Ok) (mpo.jl:229-252) by a transfer
    tensor over the k bond indices, site by site."""
    k = len(ops)
    letters = "abcdefghij"
    bonds, nbonds, phys = letters[:k], letters[k:2 * k], "pqrstuvwxy"[:k]
    E = np.ones((1,) * k, dtype=np.complex128)
    for site in range(1, len(ops[0]) + 1):
        # operator j maps physical index phys[j+1] (its input) from phys[j]
        terms = [f"{bonds[j]}{phys[j]}{phys[(j + 1) % k]}{nbonds[j]}" for j in range(k)]
        E = np.einsum(f"{bonds}," + ",".join(terms) + f"->{nbonds}", E,
                      *[op[site] for op in ops])
    return complex(E.reshape(-1)[0])


class ProjMPS:
    """Environment blocks of <bra|[MPO]|ket> with a movable centre
    (projmps.jl:16-42, abstractprojmps.jl:33-81).  ``blocks[i]`` (1-based) is
    the left block through site i when i < centre, or the right block from
    site i when i > centre."""

    def __init__(self, bra, ket, mpo=None, center=1, coeff=1.0, squared=False):
        self.bra, self.ket, self.mpo = bra, ket, mpo
        self.squared = squared
        self.nobj = 2 if mpo is None else 3
        self.blocks = [_edge(self.nobj) for _ in range(len(bra))]
        self.center = 0
        self.coeff = coeff
        self.movecenter(center)

    def __len__(self):
        return len(self.bra)

    def block(self, idx):
        if idx < 1 or idx > len(self):
            return _edge(self.nobj)
        return self.blocks[idx - 1]

    def _W(self, i):
        return None if self.mpo is None else self.mpo[i]

    def buildleft(self, idx):
        self.blocks[idx - 1] = env_left(self.block(idx - 1), self.bra[idx], self._W(idx), self.ket[idx])

    def buildright(self, idx):
        self.blocks[idx - 1] = env_right(self.block(idx + 1), self.bra[idx], self._W(idx), self.ket[idx])

    def movecenter(self, idx):
        """abstractprojmps.jl:60-81"""
        if self.center == 0:
            for i in range(1, idx):
                self.buildleft(i)
            N = len(self)
            for i in range(1, N - idx + 1):
                self.buildright(N + 1 - i)
        elif idx > self.center:
            for i in range(1, idx - self.center + 1):
                self.buildleft(self.center - 1 + i)
        elif idx < self.center:
            for i in range(1, self.center - idx + 1):
                self.buildright(self.center + 1 - i)
        self.center = idx

    def product(self, theta, direction):
        """projmps.jl:103-145 with nsites=2: the MPO branch, or for a squared
        bra-ket projection coeff * (sum P theta) * conj(P), P = project()."""
        if self.mpo is None:
            P = self.project(direction)
            s = np.sum(P * theta)
            fac = np.conj(P) if self.squared else 1.0
            return s * fac * self.coeff
        site = self.center - 1 if direction else self.center
        out = heff2(self.block(site - 1), self.mpo[site], self.mpo[site + 1],
                    self.block(site + 2), theta)
        return out * self.coeff

    def project(self, direction):
        """projmps.jl:156-189 (no MPO, nsites=2): the bra's two sites
        contracted with the overlap blocks, P[b,s1,s2,c] = sum L[x,b]
        conj(bra1[x,s1,y]) conj(bra2[y,s2,z]) R[z,c]."""
        site = self.center - 1 if direction else self.center
        L, R = self.block(site - 1), self.block(site + 2)
        B1, B2 = np.conj(self.bra[site]), np.conj(self.bra[site + 1])
        return np.einsum("xb,xsy,ytz,zc->bstc", L, B1, B2, R, optimize=True)

    def calculate(self):
        """Full contraction at the centre (projmps.jl:192-216)."""
        site = self.center
        left = env_left(self.block(site - 1), self.bra[site], self._W(site), self.ket[site])
        right = self.block(site + 1)
        return self.coeff * np.sum(left * right)


def overlap(phi, psi):
    """<phi|psi> of two MPSs (inner(phi, psi), mpo.jl:181-250)."""
    L = _edge(2)
    for i in range(1, len(psi) + 1):
        L = env_left(L, phi[i], None, psi[i])
    return complex(L.reshape(-1)[0])


def scaled(psi, a):
    """*(psi, a) (abstractmps.jl:100-107): a copy with the centre tensor
    (site 1 without a centre) multiplied by a."""
    phi = psi.copy()
    site = phi.center if phi.center != 0 else 1
    phi[site] = phi[site] * a
    return phi


def mpo_mps_product(O, psi, cutoff=0.0, maxdim=0, mindim=1):
    """MPOMPSProduct(O, psi; kwargs) (mpo.jl:125-146): site tensors
    phi[(w, a), o, (w', b)] = sum_s O[w, o, s, w'] A[a, s, b] (w fastest in
    each pair), left-canonicalised by untruncated SVDs while they are built,
    then, the centre being unset, movecenter!(phi, 1; kwargs) sweeps from N."""
    N = len(psi)
    ts = []
    for i in range(1, N + 1):
        M, A = O[i], psi[i]
        B = np.einsum("wosv,asb->waovb", M, A)  # [w, a, o, w', b]
        wl, al, d, wr, ar = B.shape
        ts.append(B.reshape(wl * al, d, wr * ar, order="F"))
    phi = GMPS(1, psi.dim, ts, 0)
    for i in range(1, N):
        phi.moveright(i)
    phi.center = 0
    phi.movecenter(1, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
    return phi


class MPSProjector:
    """|right><left| / constant (projector.jl:1-47), constant = <left|right>
    unless given."""

    rank = 2

    def __init__(self, left, right=None, constant=0.0):
        self.left = left
        self.right = left if right is None else right
        self.constant = complex(constant) if constant != 0.0 else overlap(self.left, self.right)

    def apply(self, psi):
        return scaled(self.right, overlap(self.left, psi) / self.constant)


class ProjMPSSum:
    """A sum of projections (projmpssum.jl:1-108): movecenter, product and
    calculate add the terms'."""

    def __init__(self, projs, center=1):
        self.projs = list(projs)
        self.center = 0
        self.movecenter(center)

    def movecenter(self, idx):
        for p in self.projs:
            p.movecenter(idx)
        self.center = idx

    def product(self, theta, direction):
        out = self.projs[0].product(theta, direction)
        for p in self.projs[1:]:
            out = out + p.product(theta, direction)
        return out

    def calculate(self):
        return sum(p.calculate() for p in self.projs)


def inner(st, psi, oplist, phi):
    """Per-term expectation values <psi|term|phi> (mps.jl:87-134)."""
    proj = ProjMPS(psi, phi, None, center=1)
    out = np.zeros(len(oplist.sites), dtype=np.complex128)
    for site in range(1, len(psi) + 1):
        proj.movecenter(site)
        for idx in siteindexs(oplist, site):
            sites = oplist.sites[idx]
            rng = sites[-1] - sites[0] + 1
            left = proj.block(site - 1)
            right = proj.block(site + rng)
            for i in range(1, rng + 1):
                s = site - 1 + i
                B = phi[s]
                if s in sites:
                    O = st.op(oplist.ops[idx][sites.index(s)])
                    B = np.einsum("ts,asb->atb", O, B)
                left = env_left(left, psi[s], None, B)
            out[idx] = oplist.coeffs[idx] * np.sum(left * right)
    return out


def applyop(st, psi, ops, sites):
    """A <- O A on the physical index, no coefficient (mps.jl:141-151)."""
    for o, s in zip(ops, sites):
        psi[s] = np.einsum("ts,asb->atb", st.op(o), psi[s])
