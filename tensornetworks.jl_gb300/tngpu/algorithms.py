"""dmrg, trotterize/applygates!, tebd and qjmc_simulation with the reference's
arguments, keywords, return values and observers
(src/algorithms/mps/{dmrg,tebd,qjmc}.jl, structures/mps/gatelist.jl).

Each call hands whole algorithm stages to libtngpu.so; the host loop only
sequences steps and records observers.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .models import OpList, gatesize, trotter_rows, trotter_rows_dparam
from .mps import GMPS, MPOHandle, MPSProjector, applyMPO, inner


# ---------------------------------------------------------------------------
# DMRG (dmrg.jl:1-154)
# ---------------------------------------------------------------------------
def dmrg(psi: GMPS, *Hs, nsites=2, krylovdim=3, kryloviter=2, minsweeps=1,
         maxsweeps=1000, tol=1e-10, tolgrad=1e-5, numconverges=4, cutoff=1e-12, maxdim=1000,
         mindim=1, verbose=True, precision="fp64", stats=None, max_bond_updates=0,
         profile_from_sweep=-1, coeffs=None, refine=0, residuals=False):
    """Two-site DMRG; mutates ``psi`` and returns (psi, energy).

    ``Hs`` are the terms of dmrg(psi, Hs::GMPS...; coeffs) (dmrg.jl:128-154):
    MPOs (rank 2) and MPSs (rank 1, each the penalty coeff |phi><phi|, as
    ProjMPS(phi, psi; squared=true) gives), weighted by ``coeffs`` (default
    all 1).  ``precision``: "fp64", "mixed" (3xTF32 tensor-core H_eff,
    environments and projections) or "mixed-env64" (the same with FP64
    environment updates).  ``refine`` (mixed modes): refinement steps of each
    bond's Ritz vector against its FP64 residual, one Lanczos cycle each
    whose first product is FP64.  ``stats`` (a dict) receives sweeps,
    matvecs, per-sweep device seconds and energies, and with ``residuals``
    the FP64 residual norm of every bond's eigenvector before and after the
    refinement (``bond_resid_in``/``bond_resid_out``; one extra FP64 product
    per bond and value that a refinement step did not already make);
    ``max_bond_updates`` > 0 stops after that many bond optimisations (a
    bounded timing sample)."""
    if psi.rank != 1:
        raise ValueError("Psi must be a GMPS of rank 1 (vector).")
    if len(Hs) == 0:
        raise ValueError("You must provide atleast one MPS/MPO for the Hamiltonian.")
    coeffs = [1.0] * len(Hs) if coeffs is None else [float(c) for c in coeffs]
    if len(coeffs) != len(Hs):
        raise ValueError("one coefficient per Hamiltonian term")
    for H in Hs:
        if len(H) != len(psi) or H.dim != psi.dim:
            raise ValueError("GMPS must share the same properties.")
        if H.rank not in (1, 2):
            raise ValueError("Hamiltonian must be composed of MPOs (rank 2) or MPSs (rank 1).")
    if nsites != 2:
        raise ValueError("only two-site DMRG (nsites=2) is on this path")
    o = L.DmrgOpts(nsites, krylovdim, kryloviter, minsweeps, maxsweeps, tol, tolgrad,
                   float(numconverges), cutoff, maxdim, mindim, L.PREC[precision], int(bool(verbose)),
                   int(max_bond_updates), int(profile_from_sweep), int(refine))
    e = C.c_double()
    st = L.DmrgStats()
    cap = maxsweeps if maxsweeps > 0 else 1000
    secs, ens = np.zeros(cap), np.zeros(cap)
    mds = np.zeros(cap, dtype=np.int32)
    st.sweep_cap = cap
    st.sweep_seconds, st.sweep_energies = L.as_dp(secs), L.as_dp(ens)
    st.sweep_maxdim = mds.ctypes.data_as(L.i32p)
    bcap = max(1, (len(psi) - 1) * min(cap, 64))
    bsec = np.zeros(bcap)
    bchi = np.zeros(bcap, dtype=np.int32)
    st.bond_cap = bcap
    st.bond_seconds, st.bond_chi = L.as_dp(bsec), bchi.ctypes.data_as(L.i32p)
    rin, rout = np.zeros(bcap), np.zeros(bcap)
    if residuals:
        st.bond_resid_in, st.bond_resid_out = L.as_dp(rin), L.as_dp(rout)
    ctx = psi.ctx
    if len(Hs) == 1 and Hs[0].rank == 2 and coeffs[0] == 1.0:
        ctx.check(ctx.lib.tn_dmrg(ctx.h, psi._h, Hs[0]._h, C.byref(o), C.byref(e), C.byref(st)))
    else:
        mpos = [H for H in Hs if H.rank == 2]
        prjs = [H for H in Hs if H.rank == 1]
        mc = np.asarray([c for H, c in zip(Hs, coeffs) if H.rank == 2] or [0.0])
        pc = np.asarray([c for H, c in zip(Hs, coeffs) if H.rank == 1] or [0.0])
        mh = (L.P * max(len(mpos), 1))(*[H._h for H in mpos])
        ph = (L.P * max(len(prjs), 1))(*[H._h for H in prjs])
        ctx.check(ctx.lib.tn_dmrg_sum(ctx.h, psi._h, len(mpos), mh, L.as_dp(mc), len(prjs), ph,
                                      L.as_dp(pc), C.byref(o), C.byref(e), C.byref(st)))
    if stats is not None:
        stats.update(sweeps=st.sweeps, maxbonddim=st.maxbonddim, matvecs=st.matvecs,
                     seconds=st.seconds, energy_fp64=st.energy_fp64,
                     last_discarded=st.last_discarded, bond_updates=st.bond_updates,
                     sweep_seconds=secs[: min(st.sweeps, cap)].tolist(),
                     sweep_energies=ens[: min(st.sweeps, cap)].tolist(),
                     sweep_maxdim=mds[: min(st.sweeps, cap)].tolist(),
                     bond_seconds=bsec[: min(st.bond_updates, bcap)].tolist(),
                     bond_chi=bchi[: min(st.bond_updates, bcap)].tolist())
        if residuals:
            stats.update(bond_resid_in=rin[: min(st.bond_updates, bcap)].tolist(),
                         bond_resid_out=rout[: min(st.bond_updates, bcap)].tolist())
    return psi, e.value


def vmps(*psis, coeffs=None, nsites=2, minsweeps=2, maxsweeps=200, tol=1e-10, numconverges=3,
         cutoff=1e-12, maxdim=1000, mindim=1, verbose=False, stats=None):
    """vmps(psis...; kwargs) (vmps.jl:1-105): a new MPS, starting as a copy of
    psis[0] centred at site 1, fitted by two-site sweeps to the sum of the
    psis (each weighted by ``coeffs``, default 1).  ``stats`` receives the
    final cost |fit|^2 - 2 |<target|fit>| and the sweep count."""
    if len(psis) == 0:
        raise ValueError("vmps needs at least one MPS")
    ctx = psis[0].ctx
    cs = [1.0] * len(psis) if coeffs is None else list(coeffs)
    cbuf = np.zeros(2 * len(psis))
    for k, c in enumerate(cs):
        cbuf[2 * k], cbuf[2 * k + 1] = complex(c).real, complex(c).imag
    o = L.VmpsOpts(nsites, minsweeps, maxsweeps, tol, float(numconverges), cutoff, maxdim,
                   mindim, int(bool(verbose)))
    hs = (L.P * len(psis))(*[p._h for p in psis])
    h, cost, sw = C.c_void_p(), C.c_double(), C.c_int32()
    ctx.check(ctx.lib.tn_vmps(ctx.h, len(psis), hs, L.as_dp(cbuf), C.byref(o), C.byref(h),
                              C.byref(cost), C.byref(sw)))
    if stats is not None:
        stats.update(cost=cost.value, sweeps=sw.value)
    return GMPS(h, psis[0].N, psis[0].dim, ctx)


# ---------------------------------------------------------------------------
# Gates (gatelist.jl)
# ---------------------------------------------------------------------------
class GateList:
    """Rows of non-overlapping gates uploaded to the GPU (gatelist.jl:8-62)."""

    def __init__(self, length, rows, dim, ctx=None):
        self.length = length
        self.rows = rows
        self.ctx = ctx or L.context()
        row_len = np.asarray([len(s) for s, _ in rows], dtype=np.int32)
        sites = np.asarray([s for ss, _ in rows for s in ss], dtype=np.int32)
        nsites = np.asarray([gatesize(g) for _, gs in rows for g in gs], dtype=np.int32)
        mats = [L.cplx_f(g) for _, gs in rows for g in gs]
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.tn_gates_upload(
            self.ctx.h, length, dim, len(rows), row_len.ctypes.data_as(L.i32p),
            sites.ctypes.data_as(L.i32p), nsites.ctypes.data_as(L.i32p), L.ptr_array(mats),
            C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self.ctx.lib.tn_gates_destroy(h)
            self._h = None


def trotterize(st, ops: OpList, dt, order=2, evol="imag", ctx=None):
    """gatelist.jl:75-121"""
    return GateList(ops.length, trotter_rows(st, ops, dt, order, evol), st.dim, ctx)


def lift_to_output_index(gate, d):
    """A gate of the reference's layout (g[o', o] or g[o1', o1, o2', o2]) as
    the same gate on fused MPO sites (index o + d*i), acting on the output
    index and leaving the input index alone: applygate on a rank-2 GMPS
    contracts the gate with each site's first physical index
    (gatelist.jl:146-154 with r = 2)."""
    eye = np.eye(d, dtype=np.complex128)
    g = np.asarray(gate, dtype=np.complex128)
    if g.ndim == 2:
        return np.reshape(np.einsum("po,ab->paob", g, eye), (d * d, d * d), order="F")
    lifted = np.einsum("pkql,ab,cd->pakbqcld", g, eye, eye)
    return np.reshape(lifted, (d * d,) * 4, order="F")


def applygates(psi, gates: GateList, cutoff=0.0, maxdim=0, mindim=1):
    """applygates! (gatelist.jl:191-227) on an MPS, or on an MPO (GMPO) with
    every gate acting on the output index."""
    t = L.trunc(cutoff, maxdim, mindim)
    if getattr(psi, "rank", 1) == 2:
        lifted = getattr(gates, "_lifted", None)
        if lifted is None:
            rows = [(sites, [lift_to_output_index(g, psi.d) for g in gs]) for sites, gs in gates.rows]
            lifted = GateList(gates.length, rows, psi.d * psi.d, gates.ctx)
            gates._lifted = lifted
        psi.ctx.check(psi.ctx.lib.tn_applygates(psi.ctx.h, psi.mps._h, lifted._h, C.byref(t)))
        return
    psi.ctx.check(psi.ctx.lib.tn_applygates(psi.ctx.h, psi._h, gates._h, C.byref(t)))


applygates_ = applygates


# ---------------------------------------------------------------------------
# TEBD (tebd.jl:3-219)
# ---------------------------------------------------------------------------
class TEBDObserver:
    def measure(self, time, psi, norm, energy):
        return True

    def checkdone(self):
        return False


class TEBDNorm(TEBDObserver):
    """tebd.jl:132-159"""

    def __init__(self, tol=1e-10):
        self.times, self.measurements, self.tol = [], [], tol

    def measure(self, time, psi, norm, energy):
        self.times.append(time)
        self.measurements.append(norm)

    def checkdone(self):
        if len(self.times) < 3:
            return False
        m, t = self.measurements, self.times
        E1 = (m[-1] - m[-2]) / (t[-1] - t[-2])
        E2 = (m[-2] - m[-3]) / (t[-2] - t[-3])
        if abs(E2 + E1) < 1e-8:
            return abs(E2 - E1) < self.tol
        return abs((E2 - E1) / (0.5 * (E2 + E1))) < self.tol


class TEBDEnergy(TEBDObserver):
    """tebd.jl:168-193"""

    def __init__(self, tol=1e-10):
        self.times, self.measurements, self.tol = [], [], tol

    def measure(self, time, psi, norm, energy):
        self.times.append(time)
        self.measurements.append(energy)

    def checkdone(self):
        if len(self.times) < 3:
            return False
        E1, E2 = self.measurements[-1], self.measurements[-2]
        if 0.5 * abs(E2 + E1) < 1e-8:
            return abs(E2 - E1) < self.tol
        return abs(2 * (E2 - E1) / (E2 + E1)) < self.tol


class TEBDOperators(TEBDObserver):
    """tebd.jl:201-219"""

    def __init__(self, st, oplist):
        self.times, self.measurements, self.st, self.oplist = [], [], st, oplist

    def measure(self, time, psi, norm, energy):
        self.times.append(time)
        self.measurements.append(inner(self.st, psi, self.oplist, psi))


def tebd(st, psi: GMPS, H: OpList, dt, tmax, save, observers=(), projectors=(), cutoff=1e-12,
         maxdim=0, mindim=1, evol="imag", order=2, norm=0.0, verbose=False, precision="fp64",
         projection_every=10, variational_cutoff=None):
    """Time evolution (tebd.jl:3-100); returns (psi, energy).  ``projectors``
    (MPS, MPO handles or MPSProjector) are projected out before the loop and
    after every ``projection_every`` steps: psi is replaced by vmps(psi,
    -P_1 psi, ...) at ``variational_cutoff`` (default ``cutoff``) and
    ``maxdim`` (tebd.jl:23-41,67-73).  ``psi`` may then be a new MPS: use the
    returned one.  precision="mixed" runs the gate contractions and
    truncation projections as 3xTF32 tensor-core products (FP64 Gram
    eigensolver and norms)."""
    if st.dim != psi.dim:
        raise ValueError("Sitetypes and MPS physical dimensions do not match.")
    if len(psi) != H.length:
        raise ValueError("OpList and MPS have different lengths.")
    if evol not in ("imag", "real"):
        raise ValueError("evol must be real of imag.")
    if order not in (1, 2):
        raise ValueError("Only first or second order trotter supported.")
    gates = trotterize(st, H, dt, order=order, evol=evol, ctx=psi.ctx)
    vcut = cutoff if variational_cutoff is None else variational_cutoff
    projs = []
    for proj in projectors:
        if isinstance(proj, GMPS):
            projs.append(MPSProjector(proj, proj))
        elif isinstance(proj, (MPOHandle, MPSProjector)):
            projs.append(proj)
        else:
            raise ValueError("Only MPS, MPO and MPSProjectors are supported as projectors.")

    def project(p):
        terms = [p] + [applyMPO(P, p) for P in projs]
        return vmps(*terms, coeffs=[1.0] + [-1.0] * len(projs), cutoff=vcut, maxdim=maxdim)

    if projs:
        psi = project(psi)
    nsteps = int(round(tmax / dt))
    save = dt if save < dt else save
    nsave = int(round(save / dt))
    normal = float(norm)
    energy = float(np.real(np.sum(inner(st, psi, H, psi))))
    for ob in observers:
        ob.measure(0.0, psi, normal, energy)
    psi.norm()  # log(norm(psi)) at tebd.jl:61 canonicalises an unset centre
    t = L.trunc(cutoff, maxdim, mindim)
    step = 0
    converged = False
    while not converged:
        ln = C.c_double(0.0)
        if projs:
            # applygates!, the projection every projection_every steps, then
            # log(norm) and normalize! (tebd.jl:62-78)
            applygates(psi, gates, cutoff, maxdim, mindim)
            if (step + 1) % projection_every == 0:
                psi = project(psi)
            ln.value = math.log(abs(psi.norm()))
            psi.normalize()
        else:
            psi.ctx.check(psi.ctx.lib.tn_tebd_steps_prec(psi.ctx.h, psi._h, gates._h, 1,
                                                         C.byref(t), L.PREC[precision],
                                                         C.byref(ln)))
        normal += ln.value
        step += 1
        converged = step >= nsteps
        if step % nsave == 0:
            if verbose:
                print(f"time={step * dt:.4f}, energy={energy:.12f}, maxbonddim={psi.maxbonddim()} ")
            energy = float(np.real(np.sum(inner(st, psi, H, psi))))
            for ob in observers:
                ob.measure(step * dt, psi, normal, energy)
                converged = converged or ob.checkdone()
    return psi, energy


# ---------------------------------------------------------------------------
# Differentiated TEBD: hand-written adjoint behind an rrule-shaped interface
# ---------------------------------------------------------------------------
class TEBDGradProblem:
    """A TEBD evolution over parameter segments: segment k runs ``nsub`` steps
    of the Trotter gates of ``H_of(params[k])`` (H_of affine in its argument;
    the evolution of tebd.jl:61-84 with a Hamiltonian that changes per
    segment), then the objective f = <op at site> of the normalised state."""

    def __init__(self, st, H_of, dt, nsub, op, site, cutoff=1e-12, maxdim=0, mindim=1,
                 evol="real", order=2, checkpoint=10, broadening=1e-32):
        self.st, self.H_of, self.dt, self.nsub = st, H_of, float(dt), int(nsub)
        self.op, self.site = op, int(site)
        self.cutoff, self.maxdim, self.mindim = cutoff, maxdim, mindim
        self.evol, self.order = evol, order
        self.checkpoint, self.broadening = int(checkpoint), float(broadening)

    def _lists(self, params, ctx):
        rows = [trotter_rows(self.st, self.H_of(p), self.dt, self.order, self.evol) for p in params]
        return rows, [GateList(self.H_of(params[0]).length, r, self.st.dim, ctx) for r in rows]

    def _call(self, psi0, params, want):
        ctx = psi0.ctx
        params = np.asarray(params, dtype=float)
        rows, lists = self._lists(params, ctx)
        step_gate = np.repeat(np.arange(len(params), dtype=np.int32), self.nsub)
        sizes = [g.size for r in rows for _, gs in r for g in gs]
        grads = np.zeros(2 * sum(sizes)) if want else None
        handles = (C.c_void_p * len(lists))(*[gl._h.value for gl in lists])
        op = L.cplx_f(self.st.op(self.op)).astype(np.complex128)
        f = C.c_double(0.0)
        t = L.trunc(self.cutoff, self.maxdim, self.mindim)
        ctx.check(ctx.lib.tn_tebd_grad(
            ctx.h, psi0._h, len(lists), handles, len(step_gate), step_gate.ctypes.data_as(L.i32p),
            C.byref(t), self.checkpoint, self.site, L.as_dp(op), self.broadening, C.byref(f),
            L.as_dp(grads) if want else None))
        return f.value, rows, grads

    def value(self, psi0, params):
        """f(params) by the forward pass alone."""
        return self._call(psi0, params, False)[0]

    def rrule(self, psi0, params):
        """(f, pullback): pullback(fbar) = fbar * df/dparams, through the
        library's adjoint (the shape of a ChainRulesCore rrule)."""
        f, rows, grads = self._call(psi0, params, True)
        gz = grads.view(np.complex128)
        dfdp = np.zeros(len(params))
        off = 0
        for k, p in enumerate(np.asarray(params, dtype=float)):
            drows = trotter_rows_dparam(self.st, self.H_of(p), self.H_of(p + 1.0), self.dt,
                                        self.order, self.evol)
            acc = 0.0
            for (_, gs), (_, dgs) in zip(rows[k], drows):
                for g, dg in zip(gs, dgs):
                    gb = gz[off:off + g.size].reshape(g.shape, order="F")
                    acc += float(np.real(np.vdot(gb, dg)))  # Re sum conj(gbar) dG
                    off += g.size
            dfdp[k] = acc
        return f, (lambda fbar=1.0: fbar * dfdp)


def tebd_grad(st, psi0, H_of, params, dt, nsub, op, site, **kw):
    """f and df/dparams of the segment-wise TEBD objective (TEBDGradProblem)."""
    prob = TEBDGradProblem(st, H_of, dt, nsub, op, site, **kw)
    f, back = prob.rrule(psi0, params)
    return f, back()


# ---------------------------------------------------------------------------
# QJMC (qjmc.jl:9-310)
# ---------------------------------------------------------------------------
def qjmc_gates(st, H: OpList, jumpops: OpList, dt, **kw):
    """Escape operators c^2 L^dag L and Heff = -iH - 1/2 sum escape (qjmc.jl:9-26)."""
    esc = OpList(jumpops.length)
    for ops, sites, c in zip(jumpops.ops, jumpops.sites, jumpops.coeffs):
        esc.add([st.opprod([st.dag(o), o]) for o in ops], sites, c ** 2)
    heff = (-1j) * H + (-0.5) * esc
    return heff, trotter_rows(st, heff, dt, **kw)


def qjmc_ensemble(st, psi: GMPS, H: OpList, jumpops: OpList, tmax, dt, obs: OpList, ntraj,
                  draws=None, rand=None, save=0.0, cutoff=1e-12, mindim=1, maxdim=0, workers=64,
                  seed=None, first_traj=0, engine="auto", blocks_per_sm=4, records=False,
                  stats=None, classical=True, tune_cache=None, probe_steps=8):
    """``ntraj`` independent trajectories of qjmc_simulation from ``psi``
    (left unchanged), advanced concurrently on the GPU.  Returns (times,
    averaged single-site observables [rows x terms], jump counts), and with
    ``records`` also the per-trajectory jump channels (1-based) and times.
    ``draws`` is an (ntraj x m) array of uniforms consumed per trajectory in
    the reference's order; with ``seed`` trajectory t draws from its own
    counter-based stream philox_uniforms(seed, first_traj + t); otherwise
    the draws come from ``rand``.

    engine="device" runs the whole ensemble as one persistent launch
    (tn_qjmc_ensemble: every block runs whole trajectories, ``blocks_per_sm``
    blocks per SM; needs maxdim >= 1 with d * maxdim <= 256);
    blocks_per_sm="auto" takes the width the autotuner picked for this
    workload's (maxdim, d, ntraj, N) bucket (tngpu.autotune), probing the
    first ``probe_steps`` steps of this ensemble at every candidate width on
    a cache miss (``tune_cache``: a WidthCache or a JSON path; default
    $TNGPU_TUNE_CACHE or ~/.cache/tngpu/engine_widths.json);
    engine="workers" runs ``workers`` host threads, each driving one
    trajectory at a time on its own stream (tn_qjmc_batch); "auto" takes the
    device engine whenever it applies.  ``stats`` (a dict) receives the
    device engine's algorithmic FP64 flops, launch time (CUDA events) and
    trajectory-steps.  ``classical=False`` selects the norm-based jump
    decision (qjmc.jl:65-86; device engine)."""
    save = dt if save == 0 else save
    steps = math.ceil(round(tmax / dt, 5))
    savesteps = math.ceil(round(save / dt))
    _, rows = qjmc_gates(st, H, jumpops, dt)
    gates = GateList(H.length, rows, st.dim, psi.ctx)
    if any(len(s) != 1 for s in jumpops.sites) or any(len(s) != 1 for s in obs.sites):
        raise NotImplementedError("single-site jump operators and observables only")
    fits = maxdim >= 1 and st.dim <= 4 and st.dim * max(maxdim, max(psi.bonddims())) <= 256
    if engine == "auto":
        engine = "device" if fits else "workers"
    if engine not in ("device", "workers"):
        raise ValueError("engine must be 'auto', 'device' or 'workers'")
    if engine == "device" and not fits:
        raise ValueError("the device engine needs maxdim >= 1, d <= 4 and d * maxdim <= 256")
    if draws is None and seed is None:
        g = rand if rand is not None else np.random.default_rng()
        draws = g.random((ntraj, 3 * steps + 3))
    if draws is None and first_traj != 0 and engine == "workers":
        # the worker engine numbers its streams from 0: draw shifted ones here
        draws = np.stack([philox_uniforms(seed, first_traj + t, 3 * steps + 3)
                          for t in range(ntraj)])
    if draws is not None:
        draws = np.ascontiguousarray(draws, dtype=np.float64)
        if draws.shape[0] != ntraj:
            raise ValueError("draws must have one row per trajectory")
        ndraws, dptr, sd = draws.shape[1], L.as_dp(draws), 0
    else:
        ndraws, dptr, sd = 3 * steps + 3, None, int(seed)
    jsites = np.asarray([s[0] for s in jumpops.sites], dtype=np.int32)
    jops = np.concatenate([L.cplx_f(st.op(o[0])).ravel(order="F") for o in jumpops.ops]).astype(np.complex128)
    jco = np.asarray(jumpops.coeffs, dtype=np.complex128)
    osites = np.asarray([s[0] for s in obs.sites], dtype=np.int32)
    oops = np.concatenate([L.cplx_f(complex(c) * st.op(o[0])).ravel(order="F")
                           for o, c in zip(obs.ops, obs.coeffs)]).astype(np.complex128)
    nrows = steps // savesteps + 1
    out = np.zeros((nrows, len(osites)), dtype=np.complex128)
    nj = np.zeros(ntraj, dtype=np.int32)
    t = L.trunc(cutoff, maxdim, mindim)
    ctx = psi.ctx
    if engine == "device" and blocks_per_sm == "auto":
        blocks_per_sm, timings, key = tune_qjmc_width(
            st, psi, H, jumpops, dt, obs, ntraj, probe_steps=min(steps, int(probe_steps)),
            cache=tune_cache, draws=draws, seed=seed, first_traj=first_traj, cutoff=cutoff,
            mindim=mindim, maxdim=maxdim, classical=classical)
        if stats is not None:
            stats.update(tune_key=key, tune_seconds_per_traj_step=timings)
    if engine == "device":
        mj = steps + 1 if records else 0
        jch = np.zeros((ntraj, max(mj, 1)), dtype=np.int32)
        jtm = np.zeros((ntraj, max(mj, 1)))
        sb = np.zeros(4)
        ctx.check(ctx.lib.tn_qjmc_ensemble(
            ctx.h, psi._h, gates._h, len(jsites), jsites.ctypes.data_as(L.i32p), L.as_dp(jops),
            L.as_dp(jco), steps, float(dt), ntraj, dptr, ndraws, sd, int(first_traj),
            C.byref(t), savesteps, len(osites), osites.ctypes.data_as(L.i32p), L.as_dp(oops),
            L.as_dp(out), nj.ctypes.data_as(L.i32p), mj, jch.ctypes.data_as(L.i32p),
            L.as_dp(jtm), int(blocks_per_sm), L.as_dp(sb), 1 if classical else 0))
        if stats is not None:
            stats.update(flops=float(sb[0]), kernel_ms=float(sb[1]), traj_steps=float(sb[2]),
                         blocks=int(sb[3]), blocks_per_sm=int(blocks_per_sm))
    else:
        if records:
            raise ValueError("jump records come from the device engine")
        if not classical:
            raise ValueError("the worker engine runs the escape-rate unraveling only")
        ctx.check(ctx.lib.tn_qjmc_batch(
            ctx.h, psi._h, gates._h, len(jsites), jsites.ctypes.data_as(L.i32p), L.as_dp(jops),
            L.as_dp(jco), steps, float(dt), ntraj, dptr, ndraws, sd, C.byref(t), savesteps,
            len(osites), osites.ctypes.data_as(L.i32p), L.as_dp(oops), L.as_dp(out),
            nj.ctypes.data_as(L.i32p), int(workers)))
    tt, times = 0.0, [0.0]
    for i in range(1, steps + 1):
        tt += dt
        if i % savesteps == 0:
            times.append(tt)
    if records:
        return (times, out, nj, [list(jch[r, :nj[r]]) for r in range(ntraj)],
                [list(jtm[r, :nj[r]]) for r in range(ntraj)])
    return times, out, nj


def tune_qjmc_width(st, psi, H, jumpops, dt, obs, ntraj, probe_steps=8, cache=None, **kw):
    """The trajectory engine's launch width (blocks per SM) for this
    ensemble, from the autotuner (tngpu.autotune): the cached width of the
    workload's (maxdim, d, ntraj, N) bucket, or on a miss the fastest width
    over the first ``probe_steps`` steps of this ensemble (``kw``: the
    draws or seed and truncation of qjmc_ensemble), timed by the engine's
    CUDA events per trajectory-step and then cached.  ``cache``: a
    WidthCache or a JSON path (None: the default path).  Returns (width,
    {width: seconds per trajectory-step} -- empty on a cache hit, key)."""
    from . import autotune as AT
    cache = cache if isinstance(cache, AT.WidthCache) else AT.WidthCache(cache)
    pk = max(1, int(probe_steps))
    kw = {k: v for k, v in kw.items()
          if k not in ("save", "engine", "blocks_per_sm", "stats", "records")}

    def probe(w):
        s = {}
        qjmc_ensemble(st, psi, H, jumpops, pk * dt, dt, obs, ntraj, save=dt, engine="device",
                      blocks_per_sm=w, stats=s, **kw)
        return s["kernel_ms"] * 1e-3 / max(s["traj_steps"], 1.0)

    key = AT.bucket(kw.get("maxdim", 0), st.dim, ntraj, H.length)
    width, timings = AT.tune(key, probe, cache=cache)
    return width, timings, key


def philox_uniforms(seed, trajectory, n):
    """The uniform stream of one trajectory under ``seed`` (tn_philox_uniforms:
    Philox4x32-10, Salmon et al. 2011), n values in [0, 1)."""
    out = np.zeros(int(n))
    lib = L.load()
    rc = lib.tn_philox_uniforms(int(seed), int(trajectory), int(n), L.as_dp(out))
    if rc != L.TN_OK:
        raise L.TNError(rc, "tn_philox_uniforms failed")
    return out


def shard_range(ntraj, rank, world):
    """Contiguous block of trajectory indices [lo, hi) for one rank: the
    first ntraj % world ranks take one extra trajectory."""
    base, extra = divmod(int(ntraj), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


_HOST_GROUPS = {}


def _host_group(group):
    """A gloo process group over the ranks of ``group`` for the host-tensor
    reduction (an NCCL group carries device tensors only); created once,
    collectively, the first time a non-gloo group asks."""
    import torch.distributed as dist
    if dist.get_backend(group) == "gloo":
        return group
    key = "world" if group is None else id(group)
    if key not in _HOST_GROUPS:
        ranks = None if group is None else dist.get_process_group_ranks(group)
        _HOST_GROUPS[key] = dist.new_group(ranks=ranks, backend="gloo")
    return _HOST_GROUPS[key]


def qjmc_ensemble_sharded(st, psi, H, jumpops, tmax, dt, obs, ntraj, draws=None, group=None,
                          run=None, seed=None, **kw):
    """qjmc_ensemble with the trajectories sharded over the ranks of a
    torch.distributed process group (one process per GPU).  Each rank runs
    its block of trajectories [lo, hi) -- draw rows lo:hi, or with ``seed``
    the streams philox_uniforms(seed, lo..hi-1), the same trajectories one
    process would run -- with no data-path collective; the
    trajectory-summed observables and the per-trajectory jump counts are
    combined once at the end (all_reduce / all_gather on the host, over a
    gloo group when ``group`` is an NCCL group).  Returns what qjmc_ensemble
    returns for all ntraj trajectories.  ``run`` replaces qjmc_ensemble (same
    signature), for host-only tests."""
    import torch
    import torch.distributed as dist
    run = run or qjmc_ensemble
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = shard_range(ntraj, rank, world)
    if draws is None and seed is None:
        raise ValueError("give draws or a seed")

    def block(a, b):
        if draws is not None:
            return dict(draws=np.asarray(draws)[a:b])
        return dict(seed=seed, first_traj=a)

    if hi > lo:
        times, avg, nj = run(st, psi, H, jumpops, tmax, dt, obs, hi - lo, **block(lo, hi), **kw)
        part = np.asarray(avg, dtype=np.complex128) * (hi - lo)
    else:
        times, avg, nj = run(st, psi, H, jumpops, tmax, dt, obs, 1, **block(0, 1), **kw)
        part = np.zeros_like(np.asarray(avg, dtype=np.complex128))
        nj = np.zeros(0, dtype=np.int32)
    if world == 1:
        return times, part / ntraj, np.asarray(nj, dtype=np.int32)
    hg = _host_group(group)
    buf = torch.from_numpy(np.ascontiguousarray(part.view(np.float64)))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=hg)
    total = buf.numpy().view(np.complex128).reshape(part.shape)
    # equal-size gather (padded to the largest block), trimmed per rank
    m = -(-int(ntraj) // world)
    mine = np.full(m, -1, dtype=np.int32)
    mine[:hi - lo] = np.asarray(nj, dtype=np.int32)[:hi - lo]
    counts = [torch.zeros(m, dtype=torch.int32) for _ in range(world)]
    dist.all_gather(counts, torch.from_numpy(mine), group=hg)
    sizes = [shard_range(ntraj, r, world)[1] - shard_range(ntraj, r, world)[0] for r in range(world)]
    return times, total / ntraj, np.concatenate([c.numpy()[:k] for c, k in zip(counts, sizes)])


class QJMCOperators:
    """qjmc.jl:238-260"""

    def __init__(self, oplist, st, save=False, savefile=""):
        self.times, self.measurements, self.oplist, self.st = [], [], oplist, st

    def measure(self, time, psi, jumps, jumptimes):
        self.times.append(time)
        self.measurements.append(inner(self.st, psi, self.oplist, psi))


class QJMCActivity:
    """qjmc.jl:264-285: the time and jump count of the last measurement;
    with ``save`` each measurement rewrites the HDF5 file ``savefile`` with
    the datasets "time" (Float64) and "jumps" (Int64), as h5open(savefile,
    "w") does there."""

    def __init__(self, save=False, savefile=""):
        self.time, self.jumps = 0.0, 0
        self.save, self.savefile = bool(save), savefile

    def measure(self, time, psi, jumps, jumptimes):
        self.time = time
        self.jumps = len(jumps)
        if self.save:
            from . import h5
            h5.write_file(self.savefile, h5.Group({"time": float(self.time),
                                                   "jumps": int(self.jumps)}))


class QJMCEntropy:
    """qjmc.jl:293-310"""

    def __init__(self):
        self.times, self.measurements = [], []

    def measure(self, time, psi, jumps, jumptimes):
        self.times.append(time)
        self.measurements.append([psi.entropy(i) for i in range(1, len(psi))])


def qjmc_simulation(st, psi: GMPS, H: OpList, jumpops: OpList, tmax, dt, observers=(), save=0.0,
                    cutoff=1e-12, mindim=1, maxdim=0, classical=True, verbose=False, rand=None,
                    draws=None):
    """One trajectory (qjmc.jl:28-166); mutates ``psi`` and returns (jumps,
    jumptimes) with 1-based jump indices.

    Uniform draws come from ``draws`` (an explicit array consumed in the
    reference's order) or ``rand`` (a numpy Generator).  ``classical=False``
    decides jumps from the norm of the unnormalised state (qjmc.jl:65-86).
    Single-site jump operators and single-site observables run the whole
    trajectory inside the library; other observers are sampled from the host
    between steps."""
    save = dt if save == 0 else save
    steps = math.ceil(round(tmax / dt, 5))
    savesteps = math.ceil(round(save / dt))
    _, rows = qjmc_gates(st, H, jumpops, dt)
    gates = GateList(H.length, rows, st.dim, psi.ctx)
    if any(len(s) != 1 for s in jumpops.sites):
        raise NotImplementedError("multi-site jump operators are not on this path")
    if draws is None:
        g = rand if rand is not None else np.random.default_rng()
        draws = g.random(3 * steps + 3)
    draws = np.ascontiguousarray(draws, dtype=np.float64)
    jsites = np.asarray([s[0] for s in jumpops.sites], dtype=np.int32)
    jops = np.concatenate([L.cplx_f(st.op(o[0])).ravel(order="F") for o in jumpops.ops]).astype(np.complex128)
    jco = np.asarray(jumpops.coeffs, dtype=np.complex128)
    fast_obs = all(isinstance(o, QJMCOperators) and all(len(s) == 1 for s in o.oplist.sites)
                   for o in observers)
    ctx = psi.ctx
    t = L.trunc(cutoff, maxdim, mindim)
    cap = steps + 1
    jumps = np.zeros(cap, dtype=np.int32)
    jtimes = np.zeros(cap)
    nj = C.c_int32(cap)
    used = C.c_int64(0)
    if fast_obs:
        obs_sites, obs_ops, owner = [], [], []
        for k, o in enumerate(observers):
            for ops, sites, c in zip(o.oplist.ops, o.oplist.sites, o.oplist.coeffs):
                obs_sites.append(sites[0])
                obs_ops.append(complex(c) * st.op(ops[0]))
                owner.append(k)
        nobs = len(obs_sites)
        nrows = steps // savesteps + 1
        out = np.zeros((nrows, max(nobs, 1)), dtype=np.complex128)
        osites = np.asarray(obs_sites or [1], dtype=np.int32)
        oops = (np.concatenate([L.cplx_f(m).ravel(order="F") for m in obs_ops])
                if nobs else np.zeros(4, dtype=np.complex128)).astype(np.complex128)
        ctx.check(ctx.lib.tn_qjmc_run(
            ctx.h, psi._h, gates._h, len(jsites), jsites.ctypes.data_as(L.i32p), L.as_dp(jops),
            L.as_dp(jco), steps, float(dt), L.as_dp(draws), draws.size, C.byref(t), savesteps,
            nobs, osites.ctypes.data_as(L.i32p), L.as_dp(oops), L.as_dp(out),
            jumps.ctypes.data_as(L.i32p), L.as_dp(jtimes), C.byref(nj), C.byref(used),
            1 if classical else 0))
        times = [0.0] + [dt * savesteps * (r + 1) for r in range(nrows - 1)]
        # reproduce the reference's accumulated time values
        tt, acc = 0.0, [0.0]
        for i in range(1, steps + 1):
            tt += dt
            if i % savesteps == 0:
                acc.append(tt)
        times = acc
        for k, o in enumerate(observers):
            cols = [j for j, w in enumerate(owner) if w == k]
            for r in range(nrows):
                o.times.append(times[r])
                o.measurements.append(out[r, cols].copy())
        n = nj.value
        return [int(x) for x in jumps[:n]], [float(x) for x in jtimes[:n]]
    # host-sequenced trajectory for general observers
    jl, jt = [], []
    pos = 0

    def nxt():
        nonlocal pos
        if pos >= draws.size:
            raise IndexError("uniform draw stream exhausted")
        pos += 1
        return float(draws[pos - 1])

    time = 0.0
    for o in observers:
        o.measure(time, psi, jl, jt)
    rates = np.zeros(len(jsites))
    N = len(psi)
    for i in range(1, steps + 1):
        applygates(psi, gates, cutoff, maxdim, mindim)
        r0 = nxt()
        prob = abs(psi.norm()) ** 2
        psi.normalize()
        ctx.check(ctx.lib.tn_qjmc_rates(ctx.h, psi._h, len(jsites), jsites.ctypes.data_as(L.i32p),
                                        L.as_dp(jops), L.as_dp(jco), L.as_dp(rates)))
        er = float(np.sum(rates))
        if (r0 > prob) if not classical else (nxt() > math.exp(-er * dt)):
            r = nxt()
            idx = int(np.nonzero(r < np.cumsum(rates) / er)[0][0])
            psi.movecenter(1)
            psi.applyop(st, jumpops.ops[idx], jumpops.sites[idx])
            psi.movecenter(N)
            psi.movecenter(1, cutoff=cutoff, maxdim=maxdim, mindim=mindim)
            psi.normalize()
            jl.append(idx + 1)
            jt.append(time + dt)
        time += dt
        if i % savesteps == 0:
            if verbose:
                print(f"time={time:.5f}, jumps={len(jl)}, maxbonddim={psi.maxbonddim()}")
            for o in observers:
                o.measure(time, psi, jl, jt)
    return jl, jt
