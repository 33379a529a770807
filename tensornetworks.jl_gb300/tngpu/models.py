"""Model description on the host: site types, operator lists, the MPO built
from an operator list, and Trotter gates.  These run once per model and feed
the device kernels (src/sitetypes.jl, src/lattices/spinhalf.jl,
src/structures/mps/oplist.jl, mpo.jl:323-459, gatelist.jl:75-121).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def _f(x, shape):
    return np.reshape(x, shape, order="F")


class Sitetypes:
    """Named local states and operators (sitetypes.jl:1-135)."""

    def __init__(self, dim):
        self.dim = dim
        self._states = {}
        self._ops = {}
        self._dags = {}
        self._order = []
        self.temp = 0

    def add(self, name, A, dag="None"):
        """add!(st, name, A[, dag]) (sitetypes.jl:82-134)."""
        A = np.asarray(A, dtype=np.complex128)
        if A.ndim == 1:
            if A.shape[0] != self.dim:
                raise ValueError(f"The vector must be dimension {self.dim}.")
            if name in self._states:
                raise ValueError(f"The state name {name} already exists.")
            self._states[name] = A
        elif A.ndim == 2:
            if A.shape != (self.dim, self.dim):
                raise ValueError(f"The matrix must be dimensions ({self.dim}, {self.dim}).")
            if name in self._ops:
                raise ValueError(f"The operator name {name} already exists.")
            self._ops[name] = A
            self._dags[name] = dag
            self._order.append(name)
        else:
            raise ValueError("A is unsupported.")

    def state(self, name):
        if name not in self._states:
            raise KeyError(f"The state {name} is undefined.")
        return self._states[name].copy()

    def op(self, name):
        if name not in self._ops:
            raise KeyError(f"The operator {name} is undefined.")
        return self._ops[name].copy()

    def dag(self, name):
        if name not in self._ops:
            raise KeyError(f"The operator {name} is undefined.")
        return self._dags[name]

    def opprod(self, names):
        """Name of a product of operators, registering a new pair when no stored
        operator matches to 1e-12 in summed absolute difference
        (sitetypes.jl:144-166)."""
        m = self.op(names[0])
        for n in names[1:]:
            m = m @ self.op(n)
        for n in self._order:
            if np.sum(np.abs(m - self._ops[n])) < 1e-12:
                return n
        a, b = f"temp{self.temp}", f"temp{self.temp + 1}"
        self.add(a, m, b)
        self.add(b, m.conj().T, a)
        self.temp += 2
        return a


def spinhalf():
    """lattices/spinhalf.jl:1-23"""
    st = Sitetypes(2)
    st.add("up", [1, 0])
    st.add("dn", [0, 1])
    st.add("s", [0.5 ** 0.5, 0.5 ** 0.5])
    st.add("as", [0.5 ** 0.5, -0.5 ** 0.5])
    for name, m, dag in [("x", [[0, 1], [1, 0]], "x"), ("y", [[0, -1j], [1j, 0]], "y"),
                         ("z", [[1, 0], [0, -1]], "z"), ("id", [[1, 0], [0, 1]], "id"),
                         ("pu", [[1, 0], [0, 0]], "pu"), ("pd", [[0, 0], [0, 1]], "pd"),
                         ("n", [[1, 0], [0, 0]], "n"), ("s+", [[0, 1], [0, 0]], "s-"),
                         ("s-", [[0, 0], [1, 0]], "s+")]:
        st.add(name, m, dag)
    return st


class OpList:
    """Sum of local operator products with 1-based sites (oplist.jl:1-94)."""

    def __init__(self, length):
        self.length = length
        self.ops, self.sites, self.coeffs = [], [], []

    def add(self, ops, sites, coeff=1.0):
        if isinstance(ops, str):
            ops, sites = [ops], [sites]
        if len(ops) != len(sites):
            raise ValueError("The lists must be the same length.")
        order = sorted(range(len(sites)), key=lambda k: sites[k])
        sites = [int(sites[k]) for k in order]
        ops = [ops[k] for k in order]
        for k, s in enumerate(sites):
            if s < 0 or s > self.length:
                raise ValueError(f"The sites must be between 1 and {self.length}.")
            if sites.count(s) > 1:
                raise ValueError("There are two or more operators on the same site.")
            if k > 0 and s <= sites[k - 1]:
                raise ValueError("The site list must be ordered.")
        self.ops.append(ops)
        self.sites.append(sites)
        self.coeffs.append(complex(coeff))
        return self

    def __add__(self, other):
        o = OpList(max(self.length, other.length))
        o.ops = [list(x) for x in self.ops + other.ops]
        o.sites = [list(x) for x in self.sites + other.sites]
        o.coeffs = self.coeffs + other.coeffs
        return o

    def __rmul__(self, c):
        o = OpList(self.length)
        o.ops = [list(x) for x in self.ops]
        o.sites = [list(x) for x in self.sites]
        o.coeffs = [complex(c) * x for x in self.coeffs]
        return o

    __mul__ = __rmul__

    def __len__(self):
        return self.length

    def siterange(self):
        """oplist.jl:102-109"""
        return max([1] + [s[-1] - s[0] + 1 for s in self.sites])

    def siteindexs(self, site):
        return [k for k, s in enumerate(self.sites) if s[0] == site]


def term_tensor(st, H, k):
    """Term k as [o1,i1,o2,i2,...] padded with identities to the list's range
    and clipped at the chain end (oplist.jl:134-156)."""
    sites, ops = H.sites[k], H.ops[k]
    rng = min(H.siterange(), H.length - sites[0] + 1)
    mats = []
    for j in range(rng):
        s = sites[0] + j
        mats.append(st.op(ops[sites.index(s)]) if s in sites else st.op("id"))
    t = mats[0]
    for m in mats[1:]:
        t = np.multiply.outer(t, m)
    return H.coeffs[k] * t


def site_tensor(st, H, site):
    """Sum of the terms starting at ``site`` or None (oplist.jl:164-183)."""
    ks = H.siteindexs(site)
    if not ks:
        return None
    return sum(term_tensor(st, H, k) for k in ks)


# Free-function forms of the reference's OpList and Sitetypes functions
# (oplist.jl:102-183, sitetypes.jl:144-166); term and site indices 1-based
# as there.
def siterange(H):
    return H.siterange()


def siteindexs(H, site):
    """1-based indices of the terms starting at ``site`` (oplist.jl:117-125)."""
    return [k + 1 for k in H.siteindexs(site)]


def totensor(H, st, idx):
    """Term ``idx`` (1-based) as a tensor (oplist.jl:134-156)."""
    return term_tensor(st, H, idx - 1)


def sitetensor(H, st, site):
    return site_tensor(st, H, site)


def gatesize(gate):
    """The number of sites a gate acts on (gatelist.jl:28-32)."""
    n = np.ndim(gate)
    if n % 2 == 1:
        raise ValueError("The gate must have even number of dimensions.")
    return n // 2


def op(st, name):
    return st.op(name)


def dag(st, name):
    return st.dag(name)


def state(st, name):
    return st.state(name)


# ---------------------------------------------------------------------------
# MPO from an operator list
# ---------------------------------------------------------------------------
def _trunc_keep(S, cutoff):
    if cutoff == 0:
        return S.size
    S2 = S ** 2
    with np.errstate(invalid="ignore", divide="ignore"):
        tail = np.cumsum(S2[::-1])[::-1] / S2.sum()
    hit = np.nonzero(tail > cutoff)[0]
    return max(1, int(hit[-1]) + 1 if hit.size else 1)


def mpo_tensors(st, H, cutoff=1e-15):
    """MPO site tensors W[wl, d_out, d_in, wr] of an OpList.

    Assembly is a finite-state automaton with one channel per term crossing a
    bond plus 'not started' and 'done' channels; it is then compressed by the
    same left-to-right and right-to-left truncated SVD sweeps as
    mpo.jl:442-457 (cutoff 1e-15), which reduces every bond to the operator's
    Schmidt rank (3 for the Ising chain, 5 for XXZ)."""
    N, d = H.length, st.dim
    I = np.eye(d, dtype=np.complex128)
    # channel lists per bond b = 0..N
    chans = [dict() for _ in range(N + 1)]
    for b in range(1, N):
        chans[b] = {"start": 0, "done": 1}
    chans[0] = {"start": 0}
    chans[N] = {"done": 0}
    for k, s in enumerate(H.sites):
        for b in range(s[0], s[-1]):
            chans[b][("t", k)] = len(chans[b])
    W = [np.zeros((len(chans[i]), d, d, len(chans[i + 1])), dtype=np.complex128) for i in range(N)]
    for i in range(1, N + 1):
        L, R = chans[i - 1], chans[i]
        if "start" in L and "start" in R:
            W[i - 1][L["start"], :, :, R["start"]] = I
        if "done" in L and "done" in R:
            W[i - 1][L["done"], :, :, R["done"]] = I
    for k, (ops, sites, c) in enumerate(zip(H.ops, H.sites, H.coeffs)):
        a, b = sites[0], sites[-1]
        if a == b:
            W[a - 1][chans[a - 1]["start"], :, :, chans[a]["done"]] += c * st.op(ops[0])
            continue
        for i in range(a, b + 1):
            o = st.op(ops[sites.index(i)]) if i in sites else I
            lo = chans[i - 1]["start"] if i == a else chans[i - 1][("t", k)]
            hi = chans[i]["done"] if i == b else chans[i][("t", k)]
            W[i - 1][lo, :, :, hi] += (c if i == a else 1.0) * o
    for i in range(N - 1):
        M = W[i]
        a = M.shape[0]
        U, S, Vt = np.linalg.svd(_f(M, (a * d * d, -1)), full_matrices=False)
        k = _trunc_keep(S, cutoff)
        W[i] = _f(U[:, :k] * S[:k], (a, d, d, k))
        W[i + 1] = np.tensordot(Vt[:k], W[i + 1], axes=([1], [0]))
    for i in range(N - 1, 0, -1):
        M = W[i]
        b = M.shape[3]
        a = M.shape[0]
        U, S, Vt = np.linalg.svd(_f(M, (a, -1)), full_matrices=False)
        k = _trunc_keep(S, cutoff)
        W[i] = _f(Vt[:k], (k, d, d, b))
        W[i - 1] = np.tensordot(W[i - 1], U[:, :k] * S[:k], axes=([3], [0]))
    return W


# ---------------------------------------------------------------------------
# Trotter gates (gatelist.jl:75-121)
# ---------------------------------------------------------------------------
def gate_exp(gate, time):
    """exp(time * gate) with rows (o1,o2,...) and columns (i1,i2,...)
    (tensors.jl:319-334)."""
    n = gate.ndim // 2
    d = gate.shape[0]
    outs = list(range(0, 2 * n, 2))
    ins = list(range(1, 2 * n, 2))
    M = _f(np.transpose(time * gate, outs + ins), (d ** n, d ** n))
    E = _f(sla.expm(M), (d,) * (2 * n))
    back = np.argsort(outs + ins)
    return np.transpose(E, back)


def gate_exp_frechet(gate, dgate, time):
    """d/de exp(time * (gate + e dgate)) at e = 0, in the layout of gate_exp:
    the Frechet derivative of the matrix exponential (scipy expm_frechet)."""
    n = gate.ndim // 2
    d = gate.shape[0]
    outs = list(range(0, 2 * n, 2))
    ins = list(range(1, 2 * n, 2))
    M = _f(np.transpose(time * gate, outs + ins), (d ** n, d ** n))
    E = _f(np.transpose(time * dgate, outs + ins), (d ** n, d ** n))
    _, L = sla.expm_frechet(M, E)
    back = np.argsort(outs + ins)
    return np.transpose(_f(L, (d,) * (2 * n)), back)


def trotter_rows_dparam(st, H, H1, dt, order=2, evol="imag"):
    """Derivatives of the trotter_rows gates of H with respect to a parameter p
    when H(p + 1) = H1 and H is affine in p: each gate exp(tau g) changes by
    L(tau g, tau (g1 - g)) per unit p.  Rows and gates in trotter_rows order."""
    rng = H.siterange()
    order = 1 if rng == 1 else order
    t = -1j * dt if evol == "real" else dt
    rows = []
    for i in range(1, rng + 1):
        tau = t / 2 if (i < rng and order == 2) else t
        sites, dgates = [], []
        for site in range(i, H.length + 1, rng):
            g = site_tensor(st, H, site)
            if g is not None:
                g1 = site_tensor(st, H1, site)
                sites.append(site)
                dgates.append(gate_exp_frechet(g, g1 - g, tau))
        rows.append((sites, dgates))
    if order == 2:
        for i in range(1, rng):
            rows.append(rows[rng - i - 1])
    return rows


def trotter_rows(st, H, dt, order=2, evol="imag"):
    """Rows of non-overlapping gates: [(sites, gates), ...]; second order appends
    the first rng-1 rows in reverse (gatelist.jl:75-121)."""
    rng = H.siterange()
    order = 1 if rng == 1 else order
    if order < 0 or order > 2:
        raise ValueError("Only trotter order 1 and 2 are supported.")
    if evol not in ("imag", "real"):
        raise ValueError("evol must be real of imag.")
    t = -1j * dt if evol == "real" else dt
    rows = []
    for i in range(1, rng + 1):
        tau = t / 2 if (i < rng and order == 2) else t
        sites, gates = [], []
        for site in range(i, H.length + 1, rng):
            g = site_tensor(st, H, site)
            if g is not None:
                sites.append(site)
                gates.append(gate_exp(g, tau))
        rows.append((sites, gates))
    if order == 2:
        for i in range(1, rng):
            rows.append(rows[rng - i - 1])
    return rows
