"""Device-resident GMPS and MPO handles with the reference's operations
(structures/mps/gmps.jl, mps.jl, mpo.jl).  All arithmetic runs in
libtngpu.so on the GPU; the host only holds handles and small inputs."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .models import Sitetypes, mpo_tensors


def _f(x, shape):
    return np.reshape(x, shape, order="F")


class GMPS:
    """Rank-1 GMPS (an MPS) held on the GPU.  Sites and the orthogonality
    centre are 1-based; centre 0 means unset (gmps.jl:8-13)."""

    rank = 1

    def __init__(self, handle, N, dim, ctx):
        self._h = handle
        self.N = N
        self.dim = dim
        self.ctx = ctx

    # -- construction / transfer ------------------------------------------------
    @classmethod
    def from_tensors(cls, tensors, center=0, ctx=None):
        ctx = ctx or L.context()
        ts = [L.cplx_f(t) for t in tensors]
        N = len(ts)
        d = ts[0].shape[1]
        dims = [ts[0].shape[0]] + [t.shape[2] for t in ts]
        for i, t in enumerate(ts):
            if t.ndim != 3 or t.shape[1] != d or t.shape[0] != dims[i] or t.shape[2] != dims[i + 1]:
                raise ValueError("site tensors do not chain")
        dims_arr = (C.c_int64 * (N + 1))(*dims)
        h = C.c_void_p()
        ctx.check(ctx.lib.tn_mps_upload(ctx.h, N, d, dims_arr, L.ptr_array(ts), center, C.byref(h)))
        return cls(h, N, d, ctx)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and self.ctx.h:
            self.ctx.lib.tn_mps_destroy(h)
            self._h = None

    def __len__(self):
        return self.N

    def _query(self):
        buf = (C.c_int64 * (self.N + 1))()
        c = C.c_int32()
        self.ctx.check(self.ctx.lib.tn_mps_bonddims(self.ctx.h, self._h, buf, C.byref(c)))
        return [int(buf[i]) for i in range(self.N + 1)], int(c.value)

    def bonddims(self):
        """[1, chi_1, ..., chi_{N-1}, 1]"""
        return self._query()[0]

    @property
    def center(self):
        return self._query()[1]

    def tensors(self):
        """Download the site tensors as complex128 arrays [Dl, d, Dr]."""
        dims = self.bonddims()
        out = [np.zeros((dims[i], self.dim, dims[i + 1]), dtype=np.complex128, order="F")
               for i in range(self.N)]
        self.ctx.check(self.ctx.lib.tn_mps_download(self.ctx.h, self._h, L.ptr_array(out)))
        return out

    def __getitem__(self, i):
        return self.tensors()[i - 1]

    def copy(self):
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.tn_mps_copy(self.ctx.h, self._h, C.byref(h)))
        return GMPS(h, self.N, self.dim, self.ctx)

    deepcopy = copy

    def maxbonddim(self):
        """abstractmps.jl:75-81"""
        return max([1] + self.bonddims()[1:-1])

    # -- gauge / norm (gmps.jl:29-112) --------------------------------------------
    def movecenter(self, idx, cutoff=0.0, maxdim=0, mindim=1):
        t = L.trunc(cutoff, maxdim, mindim)
        self.ctx.check(self.ctx.lib.tn_mps_movecenter(self.ctx.h, self._h, idx, C.byref(t)))

    def norm(self):
        out = (C.c_double * 2)()
        self.ctx.check(self.ctx.lib.tn_mps_norm(self.ctx.h, self._h, out))
        return complex(out[0], out[1])

    def normalize(self):
        self.ctx.check(self.ctx.lib.tn_mps_normalize(self.ctx.h, self._h))

    def entropy(self, site):
        """gmps.jl:184-189"""
        out = C.c_double()
        self.ctx.check(self.ctx.lib.tn_mps_entropy(self.ctx.h, self._h, site, C.byref(out)))
        return out.value

    def singular_values(self, site):
        cap = max(self.bonddims()) * self.dim + 1
        buf = np.zeros(cap)
        n = C.c_int64(cap)
        self.ctx.check(self.ctx.lib.tn_mps_singular_values(self.ctx.h, self._h, site, L.as_dp(buf),
                                                           C.byref(n)))
        return buf[: n.value].copy()

    def scale(self, a):
        """psi <- a psi in place, the centre tensor scaled (abstractmps.jl:100-107)."""
        c = (C.c_double * 2)(complex(a).real, complex(a).imag)
        self.ctx.check(self.ctx.lib.tn_mps_scale(self.ctx.h, self._h, c))
        return self

    def __mul__(self, a):
        """*(psi, a): a scaled copy."""
        if isinstance(a, GMPS):
            return NotImplemented
        return self.copy().scale(a)

    __rmul__ = __mul__

    def applyop(self, st, ops, sites):
        """applyop! (mps.jl:141-151): A <- O A, no coefficient."""
        if isinstance(ops, str):
            ops, sites = [ops], [sites]
        for o, s in zip(ops, sites):
            m = L.cplx_f(st.op(o))
            self.ctx.check(self.ctx.lib.tn_mps_applyop(self.ctx.h, self._h, s, L.as_dp(m)))


def overlap(phi, psi):
    """<phi|psi> of two MPSs (inner(phi, psi), mpo.jl:181-250)."""
    out = (C.c_double * 2)()
    psi.ctx.check(psi.ctx.lib.tn_mps_overlap(psi.ctx.h, phi._h, psi._h, out))
    return complex(out[0], out[1])


def applyMPO(O, psi, cutoff=0.0, maxdim=0, mindim=1):
    """applyMPO(O, psi; kwargs) = MPOMPSProduct (mpo.jl:105-146): O|psi> as a
    new MPS, centred at site 1 after a truncating sweep.  An MPSProjector
    as O applies (<left|psi>/constant) right (projector.jl:41-47); with psi an
    MPO it is the MPO product O psi (MPOMPOProduct, mpo.jl:147-167)."""
    if isinstance(O, MPSProjector):
        return O.apply(psi)
    if getattr(psi, "rank", 1) == 2:  # an MPO times an MPO (mpo.jl:147-167)
        return mpo_product(O, psi, cutoff, maxdim, mindim)
    t = L.trunc(cutoff, maxdim, mindim)
    h = C.c_void_p()
    psi.ctx.check(psi.ctx.lib.tn_mpo_apply(psi.ctx.h, O._h, psi._h, C.byref(t), C.byref(h)))
    return GMPS(h, psi.N, psi.dim, psi.ctx)


class MPSProjector:
    """MPSProjector(left, right; constant) (projector.jl:1-47): the operator
    |right><left| / constant, constant = <left|right> unless given."""

    rank = 2

    def __init__(self, left, right=None, constant=0.0):
        right = left if right is None else right
        if left.dim != right.dim:
            raise ValueError("The MPS must share the same physical dimension.")
        if len(left) != len(right):
            raise ValueError("The MPS must be the same length.")
        self.left, self.right = left, right
        self.dim = left.dim
        self.constant = complex(constant) if constant != 0.0 else overlap(left, right)

    def __len__(self):
        return len(self.left)

    def apply(self, psi):
        """applyMPO(O, psi): (<left|psi> / constant) * copy(right)."""
        return self.right * (overlap(self.left, psi) / self.constant)


class MPOHandle:
    """Rank-2 GMPS (MPO) on the GPU with its host tensors."""

    rank = 2

    def __init__(self, tensors, ctx=None):
        self.ctx = ctx or L.context()
        ts = [L.cplx_f(t) for t in tensors]
        self.tensors = ts
        self.N = len(ts)
        self.dim = ts[0].shape[1]
        w = [ts[0].shape[0]] + [t.shape[3] for t in ts]
        self.wdims = w
        h = C.c_void_p()
        arr = (C.c_int64 * (self.N + 1))(*w)
        self.ctx.check(self.ctx.lib.tn_mpo_upload(self.ctx.h, self.N, self.dim, arr, L.ptr_array(ts), C.byref(h)))
        self._h = h

    def __len__(self):
        return self.N

    def __getitem__(self, i):
        return self.tensors[i - 1]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and self.ctx.h:
            self.ctx.lib.tn_mpo_destroy(h)
            self._h = None


class GMPO:
    """Rank-2 GMPS (an MPO) on the GPU in fused form: an MPS of physical
    dimension d^2 whose index is o + d*i, the column-major grouping of a site
    [Dl, o, i, Dr] and the grouping the reference's rank-2 SVDs use
    (gmps.jl:8-13, 199-267).  Gauge moves, truncated splits, norms and gate
    rows run through the MPS machinery on that form."""

    rank = 2

    def __init__(self, fused: GMPS, d):
        self.mps = fused
        self.d = self.dim = d
        self.N = fused.N
        self.ctx = fused.ctx

    @classmethod
    def from_tensors(cls, tensors, center=0, ctx=None):
        """Sites [Dl, d, d, Dr] (output index first, as the reference's)."""
        d = tensors[0].shape[1]
        fused = [np.reshape(L.cplx_f(t), (t.shape[0], d * d, t.shape[3]), order="F")
                 for t in tensors]
        return cls(GMPS.from_tensors(fused, center, ctx), d)

    def __len__(self):
        return self.N

    def tensors(self):
        d = self.d
        return [np.reshape(t, (t.shape[0], d, d, t.shape[2]), order="F")
                for t in self.mps.tensors()]

    def __getitem__(self, i):
        return self.tensors()[i - 1]

    def bonddims(self):
        return self.mps.bonddims()

    def maxbonddim(self):
        return self.mps.maxbonddim()

    @property
    def center(self):
        return self.mps.center

    def copy(self):
        return GMPO(self.mps.copy(), self.d)

    def movecenter(self, idx, cutoff=0.0, maxdim=0, mindim=1):
        self.mps.movecenter(idx, cutoff, maxdim, mindim)

    def norm(self):
        """The Frobenius norm sqrt(Tr(O^dag O)) (norm on the rank-2 GMPS, gmps.jl:29-37)."""
        return self.mps.norm()

    def normalize(self):
        self.mps.normalize()


def productMPO(st, names, ctx=None):
    """productMPO(st, names) (mpo.jl:85-93): a product MPO of named local
    operators, centre unset."""
    ts = [np.reshape(np.asarray(st.op(n), dtype=np.complex128), (1, st.dim, st.dim, 1), order="F")
          for n in names]
    return GMPO.from_tensors(ts, 0, ctx)


def as_gmpo(O, ctx=None):
    """An MPO handle (built from an OpList) or a GMPO as a GMPO."""
    if isinstance(O, GMPO):
        return O
    if isinstance(O, MPOHandle):
        return GMPO.from_tensors(O.tensors, 0, ctx or O.ctx)
    raise TypeError("expected an MPO")


def adjoint(O):
    """adjoint(O) (mpo.jl:32-39): every site conjugated, physical indices swapped."""
    O = as_gmpo(O)
    ts = [np.conj(np.transpose(t, (0, 2, 1, 3))) for t in O.tensors()]
    return GMPO.from_tensors(ts, O.center, O.ctx)


def mpo_product(O1, O2, cutoff=0.0, maxdim=0, mindim=1):
    """applyMPO(O1, O2; kwargs) = MPOMPOProduct (mpo.jl:147-167): O1 O2 as a
    new MPO, centred at site 1 after a truncating sweep."""
    A, B = as_gmpo(O1), as_gmpo(O2)
    if A.d != B.d or A.N != B.N:
        raise ValueError("GMPS must share the same physical dims and length.")
    t = L.trunc(cutoff, maxdim, mindim)
    h = C.c_void_p()
    A.ctx.check(A.ctx.lib.tn_mpo_mpo_apply(A.ctx.h, A.mps._h, B.mps._h, A.d, C.byref(t),
                                           C.byref(h)))
    return GMPO(GMPS(h, A.N, A.d * A.d, A.ctx), A.d)


def trace(*ops):
    """trace(O1, ..., Ok) = Tr(O1 ... Ok) (mpo.jl:229-252): Tr(O) as the
    overlap with the identity, Tr(A B) as <<A^dag|B>> of the fused forms, and
    longer products through untruncated MPO products first."""
    if not ops:
        raise ValueError("There must be at least 1 MPO argument (rank 2).")
    gs = [as_gmpo(o) for o in ops]
    d, N = gs[0].d, gs[0].N
    if any(g.d != d for g in gs):
        raise ValueError("GMPS must share the same physical dim.")
    if any(g.N != N for g in gs):
        raise ValueError("GMPS must share the same length.")
    if len(gs) == 1:
        eye = [np.reshape(np.eye(d, dtype=np.complex128), (1, d, d, 1), order="F")] * N
        return overlap(GMPO.from_tensors(eye, 0, gs[0].ctx).mps, gs[0].mps)
    X = gs[0]
    for g in gs[1:-1]:
        X = mpo_product(X, g)
    return overlap(adjoint(X).mps, gs[-1].mps)


def MPO(st: Sitetypes, H, cutoff=1e-15, ctx=None):
    """MPO(st, H::OpList) (mpo.jl:323-459), uploaded to the GPU."""
    return MPOHandle(mpo_tensors(st, H, cutoff), ctx)


def randomMPS(dim, length, bonddim, rng=None, draws=None, ctx=None):
    """randomGMPS (gmps.jl:276-291): normal site tensors (edges 1),
    movecenter!(N), movecenter!(1), site 1 replaced by a fresh normal
    [1, d, min(d, bonddim)] tensor, normalize!.  ``draws`` may give the N+1
    real arrays explicitly; otherwise they come from ``rng`` (numpy
    Generator), filled in column-major order."""
    N = length
    shapes = [((1 if i == 0 else bonddim), dim, (1 if i == N - 1 else bonddim)) for i in range(N)]
    first = (1, dim, min(dim, bonddim))
    if draws is None:
        rng = rng if rng is not None else np.random.default_rng()
        draws = [_f(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
        draws.append(_f(rng.standard_normal(int(np.prod(first))), first))
    psi = GMPS.from_tensors(draws[:N], 0, ctx)
    psi.movecenter(N)
    psi.movecenter(1)
    ts = psi.tensors()
    ts[0] = draws[N]
    c = psi.center
    psi2 = GMPS.from_tensors(ts, c, ctx)
    psi2.normalize()
    return psi2


def productMPS(st, names, ctx=None):
    """productMPS(st, names) (mps.jl:68-76); centre unset."""
    return GMPS.from_tensors([_f(st.state(n), (1, st.dim, 1)) for n in names], 0, ctx)


def _terms(st, oplist, d):
    firsts, lens, mats, coeffs = [], [], [], []
    for ops, sites, c in zip(oplist.ops, oplist.sites, oplist.coeffs):
        firsts.append(sites[0])
        n = sites[-1] - sites[0] + 1
        lens.append(n)
        for s in range(sites[0], sites[-1] + 1):
            m = st.op(ops[sites.index(s)]) if s in sites else np.eye(d, dtype=np.complex128)
            mats.append(L.cplx_f(m))
        coeffs.append(complex(c))
    return firsts, lens, mats, coeffs


def inner(st, psi, oplist, phi):
    """Per-term <psi|term|phi> (mps.jl:87-134), computed on the GPU."""
    ctx = psi.ctx
    firsts, lens, mats, coeffs = _terms(st, oplist, psi.dim)
    n = len(firsts)
    if n == 0:
        return np.zeros(0, dtype=np.complex128)
    f = np.asarray(firsts, dtype=np.int32)
    ln = np.asarray(lens, dtype=np.int32)
    ops = np.concatenate([m.ravel(order="F") for m in mats]).astype(np.complex128)
    co = np.asarray(coeffs, dtype=np.complex128)
    out = np.zeros(n, dtype=np.complex128)
    ctx.check(ctx.lib.tn_inner_terms(ctx.h, psi._h, phi._h, n, f.ctypes.data_as(L.i32p),
                                     ln.ctypes.data_as(L.i32p), L.as_dp(ops), L.as_dp(co), L.as_dp(out)))
    return out


# Free-function forms of the reference's accessors and gauge operations
# (abstractmps.jl:4-81, gmps.jl:29-127, mps.jl:141-151), for code written
# against the reference's function names; each calls the object's method.
def entropy(psi, site):
    return psi.entropy(site)


def normalize(psi):
    psi.normalize()


def movecenter(psi, idx, **kw):
    psi.movecenter(idx, **kw)


def norm(psi):
    return psi.norm()


def dim(psi):
    return psi.dim


def rank(psi):
    return psi.rank


def center(psi):
    return psi.center


def tensors(psi):
    return psi.tensors()


def bonddim(psi, site):
    """The bond dimension between site and site+1 (abstractmps.jl:64-67):
    None for a site outside 1..N; site N has no bond to its right."""
    if site < 1 or site > len(psi):
        return None
    if site == len(psi):
        raise IndexError("no bond to the right of the last site")
    return psi.bonddims()[site]


def maxbonddim(psi):
    return psi.maxbonddim()


def ismps(psi):
    return psi.rank == 1


def ismpo(psi):
    return psi.rank == 2


def truncate(psi, **kw):
    """truncate! (gmps.jl:121-127): a truncating sweep from the centre at
    one end to the other end.  With the centre elsewhere the reference's
    movecenter!(psi, 0) raises, and so does this."""
    N = len(psi)
    if psi.center != 1 and psi.center != N:
        raise ValueError("The index is out of range.")
    psi.movecenter(N if psi.center == 1 else 1, **kw)


def applyop(st, psi, ops, sites):
    """applyop!(st, psi, ops, sites) (mps.jl:141-151)."""
    psi.applyop(st, ops, sites)


# ---------------------------------------------------------------------------
# Checkpoints: the GMPS HDF5 group of gmps.jl:359-383 (attributes type="MPS"
# and version=1, datasets "length", "center" and "MPS[i]", 1-based, the site
# tensors complex [Dl, d, Dr] or [Dl, d, d, Dr]).  Paths ending in .h5 or
# .hdf5 are HDF5 files in HDF5.jl's layout (tngpu.h5); other paths hold the
# same group as entries of an .npz archive.
# ---------------------------------------------------------------------------
def mps_record(tensors, center, name="psi"):
    """The archive entries of one MPS group."""
    rec = {f"{name}/type": np.array("MPS"), f"{name}/version": np.array(1),
           f"{name}/length": np.array(len(tensors)), f"{name}/center": np.array(int(center))}
    for i, t in enumerate(tensors, start=1):
        rec[f"{name}/MPS[{i}]"] = np.asarray(t, dtype=np.complex128)
    return rec


def mps_from_record(rec, name="psi"):
    """(tensors, center) of one MPS group; the reference's read check."""
    key = f"{name}/type"
    if key not in rec or str(rec[key]) != "MPS":
        raise ValueError("HDF5 group of file does not contain MPS data.")
    N = int(rec[f"{name}/length"])
    return [np.asarray(rec[f"{name}/MPS[{i}]"]) for i in range(1, N + 1)], int(rec[f"{name}/center"])


def _is_hdf5(path):
    return str(path).lower().endswith((".h5", ".hdf5"))


def write_mps(path, psi, name="psi"):
    """Download psi (a GMPS or GMPO) and store it as the group ``name`` of
    an HDF5 file (a .h5/.hdf5 path) or of an .npz archive."""
    if _is_hdf5(path):
        from . import h5
        h5.write_gmps(path, psi.tensors(), psi.center, name)
    else:
        np.savez(path, **mps_record(psi.tensors(), psi.center, name))


def read_mps(path, name="psi", ctx=None):
    """Upload the group ``name`` written by write_mps (or, for an HDF5
    file, by the reference's HDF5.write): a GMPS, or a GMPO when the site
    tensors have two physical indices (the rank test of gmps.jl:380-382)."""
    if _is_hdf5(path):
        from . import h5
        tensors, center = h5.read_gmps(path, name)
    else:
        with np.load(path, allow_pickle=False) as z:
            tensors, center = mps_from_record({k: z[k] for k in z.files}, name)
    if np.ndim(tensors[0]) == 4:
        return GMPO.from_tensors(tensors, center, ctx)
    return GMPS.from_tensors(tensors, center, ctx)
