"""Oracle drivers: restarted Lanczos, two-site DMRG, Trotter gates, TEBD and
QJMC.  Test infrastructure only."""

from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

from .core import (MPSProjector, ProjMPSSum, mpo_mps_product, GMPS, OpList, ProjMPS, applyop, fr, inner, siterange,
                   sitetensor)

__all__ = [
    "lanczos_lowest", "dmrg", "trotterize", "applygate", "applygates", "tebd",
    "qjmc_gates", "qjmc_emission_rates", "qjmc_simulation", "dmrg_sweep_stats",
    "tebd_segments_objective", "vmps", "apply_op",
]


# ---------------------------------------------------------------------------
# Restarted Lanczos, lowest eigenpair
# ---------------------------------------------------------------------------
def lanczos_lowest(matvec, x0, krylovdim, maxiter, tol=1e-14, stats=None):
    """Lowest eigenpair by thick-restart Lanczos, restating the call
    ``eigsolve(Heff, A0, 1, :SR; krylovdim, maxiter=kryloviter,
    ishermitian=true, tol=1e-14)`` (algorithms/mps/dmrg.jl:51-53).

    KrylovKit is not vendored in the reference (Project.toml:6-13, no
    Manifest pins a version); this follows its published Lanczos eigsolve:
    x0 normalised; the basis grows one matvec at a time to ``krylovdim``
    vectors with full reorthogonalisation; the projected matrix is
    diagonalised only at full dimension (or on an invariant subspace,
    residual <= tol); Ritz pairs count as converged while |beta * u[K, j]| <=
    tol; otherwise, unless ``maxiter`` cycles have run, it restarts from the
    keep = (3*krylovdim + 2*converged) // 5 lowest Ritz vectors plus the
    normalised residual.  The projected matrix is assembled from the
    reorthogonalisation coefficients, which equals KrylovKit's Householder
    re-tridiagonalised form in exact arithmetic."""
    n = x0.size
    shape = x0.shape
    x = x0.reshape(-1).astype(np.complex128)
    V = [x / np.linalg.norm(x)]
    AV = []
    H = np.zeros((krylovdim + 1, krylovdim + 1), dtype=np.complex128)
    numops = 0
    numiter = 1
    K = 0  # vectors whose image is known

    def grow():
        nonlocal K, numops
        v = V[K]
        w = matvec(v.reshape(shape)).reshape(-1)
        numops += 1
        AV.append(w)
        Vm = np.array(V[:K + 1])
        h = Vm.conj() @ w
        r = w - Vm.T @ h
        h2 = Vm.conj() @ r
        r = r - Vm.T @ h2
        h = h + h2
        H[:K + 1, K] = h
        H[K, :K + 1] = h.conj()
        H[K, K] = h[K].real
        K += 1
        beta = np.linalg.norm(r)
        return r, beta

    while True:
        r, beta = grow()
        invariant = beta <= tol or K >= n
        if K < krylovdim and not invariant:
            V.append(r / beta)
            continue
        T = H[:K, :K]
        D, U = np.linalg.eigh(T)
        f = U[K - 1, :] * beta
        conv = 0
        while conv < K and abs(f[conv]) <= tol:
            conv += 1
        if invariant:
            conv = max(conv, 1)
        if conv >= 1 or numiter == maxiter:
            break
        keep = (3 * krylovdim + 2 * conv) // 5
        Vm, AVm = np.array(V[:K]), np.array(AV)
        Y = U[:, :keep].T @ Vm
        AY = U[:, :keep].T @ AVm
        V = [y for y in Y] + [r / beta]
        AV = [y for y in AY]
        H[:] = 0
        H[np.arange(keep), np.arange(keep)] = D[:keep]
        H[keep, :keep] = f[:keep]
        H[:keep, keep] = np.conj(f[:keep])
        # the residual's own column is filled by its matvec in grow()
        K = keep
        numiter += 1
    vec = U[:, 0] @ np.array(V[:K])
    if stats is not None:
        stats["numops"] = stats.get("numops", 0) + numops
        stats["numiter"] = numiter
    return D[0], vec.reshape(shape)


# ---------------------------------------------------------------------------
# DMRG (algorithms/mps/dmrg.jl)
# ---------------------------------------------------------------------------
def dmrg(psi, H, nsites=2, krylovdim=3, kryloviter=2, minsweeps=1, maxsweeps=1000,
         tol=1e-10, tolgrad=1e-5, numconverges=4.0, cutoff=1e-12, maxdim=1000,
         mindim=1, verbose=False, stats=None, energies=None, coeffs=None):
    """Two-site DMRG (dmrg.jl:1-99 and the entry point dmrg.jl:128-154).

    ``H`` is one MPO or a list of terms: MPOs (rank 2, ProjMPS(psi, H, psi))
    and MPSs (rank 1, ProjMPS(phi, psi; squared=true)), weighted by
    ``coeffs``, summed in a ProjMPSSum.  One directional pass is one sweep
    (dmrg.jl:63-66).  Returns (psi, cost) with cost the last local Lanczos
    eigenvalue (dmrg.jl:55,98)."""
    if nsites != 2:
        raise ValueError("only two-site DMRG is on this path")
    if psi.rank != 1:
        raise ValueError("Psi must be a GMPS of rank 1 (vector).")
    psi.movecenter(1)
    N = len(psi)
    if isinstance(H, (list, tuple)):
        cs = [1.0] * len(H) if coeffs is None else list(coeffs)
        terms = [ProjMPS(psi, psi, h, center=1, coeff=c) if h.rank == 2
                 else ProjMPS(h, psi, None, center=1, coeff=c, squared=True)
                 for h, c in zip(H, cs)]
        proj = ProjMPSSum(terms, center=1)
    else:
        proj = ProjMPS(psi, psi, H, center=1)
    cost = proj.calculate()
    lastcost = cost
    D = psi.maxbonddim()
    lastD = D
    grad = 0.0
    direction = False
    converged = False
    convsweeps = convgrad = 0
    sweeps = 0
    while not converged:
        for j in range(1, N + 2 - nsites):
            site = N + 1 - j if direction else j
            site1 = site + 1 - nsites if direction else site
            proj.movecenter(site)
            A0 = np.tensordot(psi[site1], psi[site1 + 1], axes=([2], [0]))
            eig, vec = lanczos_lowest(lambda x: proj.product(x, direction), A0,
                                      krylovdim, kryloviter, stats=stats)
            cost = eig
            psi.replacesites(vec, site1, direction, True, cutoff=cutoff,
                             maxdim=maxdim, mindim=mindim)
        proj.movecenter(1 if direction else N)
        direction = not direction
        sweeps += 1
        D = psi.maxbonddim()

        def diff(x, y):
            return abs(x - y) if abs(x) < 1e-10 else abs((x - y) / x)

        if sweeps >= minsweeps:
            dd = diff(cost, lastcost)
            convsweeps = convsweeps + 1 if (dd < tol and lastD == D) else 0
            with np.errstate(invalid="ignore", divide="ignore"):
                g = abs((dd - grad) / (dd + grad)) if (dd + grad) != 0 else float("nan")
            convgrad = convgrad + 1 if (g < tolgrad and lastD == D) else 0
            if max(convsweeps, convgrad) >= numconverges:
                converged = True
            if sweeps >= maxsweeps and maxsweeps != 0:
                converged = True
        grad = abs(diff(cost, lastcost))
        lastcost = cost
        lastD = D
        if energies is not None:
            energies.append(float(np.real(cost)))
        if verbose:
            print(f"Sweep={sweeps}, energy={np.real(cost):.12f}, maxbonddim={D}")
    return psi, cost


def dmrg_sweep_stats(bonddims, d, w, n_mv):
    """Algorithmic flops of one directional sweep with the given bond dims
    (list of N+1), MPO bond dim w and matvecs per bond."""
    total = 0.0
    for i in range(len(bonddims) - 2):
        cl, cr = bonddims[i], bonddims[i + 2]
        fmv = 8 * (w * d * d * cl * cl * cr + w * w * d ** 4 * cl * cr + w * d * d * cl * cr * cr)
        total += n_mv * fmv
    return total


# ---------------------------------------------------------------------------
# Trotter gates and gate application (structures/mps/gatelist.jl)
# ---------------------------------------------------------------------------
def _gate_exp(gate, time):
    """exp(time*gate, [2,4,..]) with rows (o1,o2,..) and columns (i1,i2,..)
    (gatelist.jl:100, tensors.jl:319-334)."""
    n = gate.ndim // 2
    d = gate.shape[0]
    perm = [2 * i for i in range(n)] + [2 * i + 1 for i in range(n)]
    M = fr(np.transpose(time * gate, perm), (d ** n, d ** n))
    E = sla.expm(M)
    inv = np.argsort(perm)
    return np.transpose(fr(E, (d,) * (2 * n)), inv)


def trotterize(st, ops, dt, order=2, evol="imag"):
    """Gate layers (gatelist.jl:75-121).  Returns list of (sites, gates) rows;
    2nd order adds the first rng-1 rows again in reverse."""
    rng = siterange(ops)
    order = 1 if rng == 1 else order
    if order < 0 or order > 2:
        raise ValueError("Only trotter order 1 and 2 are supported.")
    dt = -1j * dt if evol == "real" else dt
    rows = []
    for i in range(1, rng + 1):
        time = dt / 2 if (i < rng and order == 2) else dt
        sites, gates = [], []
        site = i
        while site <= ops.length:
            g = sitetensor(ops, st, site)
            if g is not None:
                gates.append(_gate_exp(g, time))
                sites.append(site)
            site += rng
        rows.append((sites, gates))
    if order == 2:
        for i in range(1, rng):
            rows.append(rows[rng - i - 1])
    return rows


def applygate(psi, site, gate, direction=False, cutoff=0.0, maxdim=0, mindim=1):
    """gatelist.jl:137-171 without the optional fidelity (off in applygates!).
    On an MPO (rank 2) the gate acts on each site's output index."""
    if psi.rank == 2:
        if gate.ndim == 2:
            theta = np.einsum("po,aoib->apib", gate, psi[site])
        else:
            prod = np.tensordot(psi[site], psi[site + 1], axes=([3], [0]))  # a o1 i1 o2 i2 b
            theta = np.einsum("pkql,akilmb->apiqmb", gate, prod, optimize=True)
        psi.replacesites(theta, site, direction, False, cutoff=cutoff, maxdim=maxdim,
                         mindim=mindim)
        return
    if gate.ndim == 2:
        theta = np.einsum("ts,asb->atb", gate, psi[site])
    else:
        theta = np.tensordot(psi[site], psi[site + 1], axes=([2], [0]))
        theta = np.einsum("aijb,piqj->apqb", theta, gate, optimize=True)
    psi.replacesites(theta, site, direction, False, cutoff=cutoff, maxdim=maxdim, mindim=mindim)


def applygates(psi, rows, cutoff=0.0, maxdim=0, mindim=1):
    """Row schedule with truncating gauge moves before every gate
    (gatelist.jl:191-227)."""
    for sites, gates in rows:
        first = sites[0]
        last = sites[-1] + gates[-1].ndim // 2 - 1
        direction = not (abs(psi.center - first) < abs(psi.center - last))
        n = len(gates)
        for i in range(n):
            g = n - 1 - i if direction else i
            size = gates[g].ndim // 2
            ctr = sites[g] + size - 1 if direction else sites[g]
            psi.movecenter(ctr, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
            applygate(psi, sites[g], gates[g], direction, cutoff, maxdim, mindim)


def vmps(*psis, coeffs=None, nsites=2, minsweeps=2, maxsweeps=200, tol=1e-10, numconverges=3,
         cutoff=1e-12, maxdim=1000, mindim=1, stats=None):
    """vmps(psis...; kwargs) (vmps.jl:1-105): psi0 = a copy of psis[0] centred
    at 1, fitted by two-site sweeps to sum_k coeffs[k] psis[k] (the reference
    weights by scaling a term's tensor: the same target).  At each bond the
    local target is sum_k c_k conj(project(ProjMPS(psi_k, psi0))) and
    replacesites! splits it without normalising; the cost is |psi0|^2 -
    2 |calculate| and converged sweeps accumulate as the reference's do."""
    psi0 = psis[0].copy()
    psi0.movecenter(1)
    N = len(psi0)
    cs = [1.0] * len(psis) if coeffs is None else list(coeffs)
    projs = [ProjMPS(p, psi0, None, center=1) for p in psis]

    def cost():
        nrm = abs(psi0.norm()) ** 2
        c = sum(np.conj(ck) * p.calculate() for ck, p in zip(cs, projs))
        return nrm - 2 * abs(c)

    def diff(x, y):
        return abs(x - y) if abs(x) < 1e-10 else abs((x - y) / x)

    lastcost = cost()
    lastD = psi0.maxbonddim()
    direction, converged, convsweeps, sweeps = False, False, 0, 0
    while not converged:
        for j in range(1, N + 2 - nsites):
            site = N + 1 - j if direction else j
            site1 = site + 1 - nsites if direction else site
            for p in projs:
                p.movecenter(site)
            vec = sum(ck * np.conj(p.project(direction)) for ck, p in zip(cs, projs))
            psi0.replacesites(vec, site1, direction, False, cutoff=cutoff, maxdim=maxdim,
                              mindim=mindim)
        for p in projs:
            p.movecenter(1 if direction else N)
        direction = not direction
        sweeps += 1
        D = psi0.maxbonddim()
        c = cost()
        if sweeps >= minsweeps:
            if diff(c, lastcost) < tol and lastD == D:
                convsweeps += 1  # never reset: vmps.jl:67 compares instead of assigning
            if convsweeps >= numconverges:
                converged = True
            if sweeps >= maxsweeps and maxsweeps != 0:
                converged = True
        lastcost, lastD = c, D
    if stats is not None:
        stats.update(cost=lastcost, sweeps=sweeps)
    return psi0


def apply_op(P, psi, **kw):
    """P * psi for an MPSProjector or an MPO (applyMPO, projector.jl:41-47,
    mpo.jl:105-146)."""
    if isinstance(P, MPSProjector):
        return P.apply(psi)
    return mpo_mps_product(P, psi, **kw)


def tebd(st, psi, H, dt, tmax, save, observers=None, cutoff=1e-12, maxdim=0,
         mindim=1, evol="imag", order=2, norm=0.0, record=None, projectors=None,
         projection_every=10, variational_cutoff=None):
    """TEBD step loop (tebd.jl:3-100).  ``projectors`` (MPS, MPO or
    MPSProjector) are projected out before the loop and after every
    ``projection_every`` steps by psi = vmps(psi, -P psi, ...) at
    ``variational_cutoff`` and ``maxdim`` (tebd.jl:23-41,67-73); the
    returned psi is then a new MPS.

    ``observers`` is a list of OpList; their expectations are appended to
    ``record`` (dict with 'times', 'ops', 'lognorm', 'energy') at t=0 and
    every nsave steps, as TEBDOperators/TEBDNorm/TEBDEnergy do
    (tebd.jl:132-219)."""
    if st.dim != psi.dim:
        raise ValueError("Sitetypes and MPS physical dimensions do not match.")
    if len(psi) != H.length:
        raise ValueError("OpList and MPS have different lengths.")
    rows = trotterize(st, H, dt, order=order, evol=evol)
    vcut = cutoff if variational_cutoff is None else variational_cutoff
    projs = [MPSProjector(p, p) if (hasattr(p, "rank") and p.rank == 1) else p
             for p in (projectors or [])]

    def project(p):
        terms = [p] + [apply_op(P, p) for P in projs]
        return vmps(*terms, coeffs=[1.0] + [-1.0] * len(projs), cutoff=vcut, maxdim=maxdim)

    if projs:
        psi = project(psi)
    nsteps = int(round(tmax / dt))
    save = dt if save < dt else save
    nsave = int(round(save / dt))
    normal = norm
    energy = float(np.real(np.sum(inner(st, psi, H, psi))))
    observers = observers or []

    def measure(t):
        if record is None:
            return
        record.setdefault("times", []).append(t)
        record.setdefault("lognorm", []).append(normal)
        record.setdefault("energy", []).append(energy)
        record.setdefault("ops", []).append([inner(st, psi, o, psi) for o in observers])

    measure(0.0)
    step = 0
    psi.norm()  # tebd.jl:61 evaluates log(norm(psi)), which canonicalises an unset centre
    while True:
        applygates(psi, rows, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
        if projs and (step + 1) % projection_every == 0:
            psi = project(psi)
        normal += math.log(float(np.real(psi.norm())))
        psi.normalize()
        step += 1
        done = step >= nsteps
        if step % nsave == 0:
            energy = float(np.real(np.sum(inner(st, psi, H, psi))))
            measure(step * dt)
        if done:
            break
    return psi, energy


def tebd_segments_objective(st, psi, Hs, dt, nsub, op, site, cutoff=1e-12, maxdim=0, mindim=1,
                            evol="real", order=2):
    """<op at site> of the normalised state after len(Hs) segments of nsub
    TEBD steps, segment k with Hamiltonian Hs[k]: the step loop of
    tebd.jl:61-84 (applygates! then normalize!) with the gates rebuilt per
    segment by trotterize (gatelist.jl:75-121).  The reference has no such
    driver; a user script composes it from these calls.  ``psi`` is
    modified."""
    psi.norm()  # tebd.jl:61 canonicalises an unset centre
    for H in Hs:
        rows = trotterize(st, H, dt, order=order, evol=evol)
        for _ in range(nsub):
            applygates(psi, rows, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
            psi.normalize()
    ob = OpList(len(psi))
    ob.add([op], [site], 1.0)
    num = complex(np.sum(inner(st, psi, ob, psi)))
    return float(np.real(num)) / float(np.real(psi.norm()) ** 2)


# ---------------------------------------------------------------------------
# QJMC (algorithms/mps/qjmc.jl)
# ---------------------------------------------------------------------------
def qjmc_gates(st, H, jumpops, dt, **kw):
    """Escape operators c^2 L^dag L and Heff = -iH - 1/2 sum escape, Trotterised
    with the default evol='imag' (qjmc.jl:9-26)."""
    esc = OpList(jumpops.length)
    for ops, sites, c in zip(jumpops.ops, jumpops.sites, jumpops.coeffs):
        names = [st.opprod([st.dag(o), o]) for o in ops]
        esc.add(names, sites, c ** 2)
    heff = H.scaled(-1j) + esc.scaled(-0.5)
    return heff, trotterize(st, heff, dt, **kw)


def qjmc_emission_rates(st, psi, jumpops):
    """rates_i = |c_i^2 <psi| L_i^dag L_i |psi>| via overlap blocks
    (qjmc.jl:170-220)."""
    proj = ProjMPS(psi, psi, None, center=1)
    rates = np.zeros(len(jumpops.ops), dtype=np.complex128)
    for i in range(1, len(psi) + 1):
        idxs = [k for k, s in enumerate(jumpops.sites) if s[0] == i]
        proj.movecenter(i)
        for idx in idxs:
            sites, ops = jumpops.sites[idx], jumpops.ops[idx]
            coeff = jumpops.coeffs[idx] ** 2
            rng = sites[-1] - sites[0] + 1
            prod = proj.block(sites[0] - 1)
            right = proj.block(sites[-1] + 1)
            for j in range(1, rng + 1):
                s = i + j - 1
                A = psi[s]
                O = st.op(ops[sites.index(s)]) if s in sites else st.op("id")
                OdO = np.conj(O).T @ O
                prod = np.einsum("ab,asc,st,btd->cd", prod, np.conj(A), OdO, A, optimize=True)
            rates[idx] = coeff * np.sum(prod * right)
    return np.abs(rates)


class UniformStream:
    """Explicit uniform draws consumed in order (stands in for Julia rand())."""

    def __init__(self, draws):
        self.draws = np.asarray(draws, dtype=np.float64)
        self.pos = 0

    def __call__(self):
        if self.pos >= self.draws.size:
            raise IndexError("uniform stream exhausted")
        u = self.draws[self.pos]
        self.pos += 1
        return float(u)


def qjmc_simulation(st, psi, H, jumpops, tmax, dt, rand, observers=None, save=0.0,
                    cutoff=1e-12, mindim=1, maxdim=0, classical=True, record=None,
                    entropies=False):
    """One trajectory (qjmc.jl:28-166).  ``rand`` is a callable returning the
    next uniform draw; per step the reference draws once unconditionally
    (qjmc.jl:64), once for the jump decision (:97) and once more on a jump
    (:99).  Returns (jumps, jumptimes) with 1-based jump indices.

    ``entropies=True`` also records, at every save, the entanglement entropy
    at every bond 1..N-1 as QJMCEntropy does (qjmc.jl:301-309): each
    entropy(psi, i) moves the centre to i (gmps.jl:184-189), so the
    measurement changes the gauge the next steps start from."""
    save = dt if save == 0 else save
    steps = math.ceil(round(tmax / dt, 5))
    savesteps = math.ceil(round(save / dt))
    jumps, jumptimes = [], []
    _, rows = qjmc_gates(st, H, jumpops, dt)
    t = 0.0
    observers = observers or []

    def measure(tt):
        if record is not None:
            record.setdefault("times", []).append(tt)
            record.setdefault("ops", []).append([inner(st, psi, o, psi) for o in observers])
            if entropies:
                record.setdefault("entropy", []).append(
                    [psi.entropy(b) for b in range(1, len(psi))])

    measure(t)
    N = len(psi)
    for i in range(1, steps + 1):
        applygates(psi, rows, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
        r = rand()
        if not classical:
            prob = float(np.real(psi.norm() ** 2))
            psi.normalize()
            if r > prob:
                rates = qjmc_emission_rates(st, psi, jumpops)
                r = rand()
                cum = np.cumsum(rates) / np.sum(rates)
                idx = int(np.nonzero(r < cum)[0][0])
                _jump(st, psi, jumpops, idx, N, cutoff, maxdim, mindim)
                jumps.append(idx + 1)
                jumptimes.append(t + dt)
        else:
            psi.normalize()
            rates = qjmc_emission_rates(st, psi, jumpops)
            er = np.sum(rates)
            prob = math.exp(-er * dt)
            if rand() > prob:
                r = rand()
                cum = np.cumsum(rates) / er
                idx = int(np.nonzero(r < cum)[0][0])
                _jump(st, psi, jumpops, idx, N, cutoff, maxdim, mindim)
                jumps.append(idx + 1)
                jumptimes.append(t + dt)
        t += dt
        if i % savesteps == 0:
            measure(t)
    return jumps, jumptimes


def _jump(st, psi, jumpops, idx, N, cutoff, maxdim, mindim):
    """qjmc.jl:103-107"""
    psi.movecenter(1)
    applyop(st, psi, jumpops.ops[idx], jumpops.sites[idx])
    psi.movecenter(N)
    psi.movecenter(1, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
    psi.normalize()
