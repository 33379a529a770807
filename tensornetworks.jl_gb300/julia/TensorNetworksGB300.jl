"""
    TensorNetworksGB300

Drop-in GPU backend for the finite-MPS hot path of TensorNetworks.jl.  The
methods below keep the reference's names, argument types, keywords and return
values (`dmrg`, `tebd`, `applygates!`, `qjmc_simulation`) and forward the work
to libtngpu.so through `ccall`.  Model construction (`spinhalf`, `OpList`,
`MPO(st, H)`, `trotterize`) stays in TensorNetworks.jl; only tensors cross the
boundary, as column-major `ComplexF64` arrays.

Usage:
    using TensorNetworks, TensorNetworksGB300
    psi, energy = TensorNetworksGB300.dmrg(psi, H; maxdim=1024, precision=:mixed)
"""
module TensorNetworksGB300

using TensorNetworks
import TensorNetworks: GMPS, OpList, Sitetypes, GateList

const libtngpu = get(ENV, "TNGPU_LIB", joinpath(@__DIR__, "..", "tngpu", "libtngpu.so"))

const TN_PREC_FP64 = Int32(0)
const TN_PREC_MIXED = Int32(1)
const TN_PREC_MIXED_ENV64 = Int32(2)
prec_code(p::Symbol) = p === :mixed ? TN_PREC_MIXED : p === :mixed_env64 ? TN_PREC_MIXED_ENV64 : TN_PREC_FP64

struct TruncOpts
    cutoff::Float64
    maxdim::Int64
    mindim::Int64
end

struct DmrgOpts
    nsites::Int32
    krylovdim::Int32
    kryloviter::Int32
    minsweeps::Int32
    maxsweeps::Int32
    tol::Float64
    tolgrad::Float64
    numconverges::Float64
    cutoff::Float64
    maxdim::Int64
    mindim::Int64
    precision::Int32
    verbose::Int32
    max_bond_updates::Int32
    profile_from_sweep::Int32
    refine::Int32
end

mutable struct DmrgStats
    sweeps::Int32
    maxbonddim::Int32
    matvecs::Int64
    seconds::Float64
    energy_fp64::Float64
    last_discarded::Float64
    sweep_cap::Int32
    sweep_seconds::Ptr{Float64}
    sweep_energies::Ptr{Float64}
    sweep_maxdim::Ptr{Int32}
    bond_updates::Int32
    bond_cap::Int32
    bond_seconds::Ptr{Float64}
    bond_chi::Ptr{Int32}
    bond_resid_in::Ptr{Float64}
    bond_resid_out::Ptr{Float64}
end
DmrgStats() = DmrgStats(0, 0, 0, 0.0, 0.0, 0.0, 0, C_NULL, C_NULL, C_NULL, 0, 0, C_NULL, C_NULL,
                        C_NULL, C_NULL)

mutable struct Context
    h::Ptr{Cvoid}
end

const _ctx = Ref{Union{Nothing,Context}}(nothing)

function context(device::Integer=0)
    if _ctx[] === nothing
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:tn_ctx_create, libtngpu), Int32, (Int32, Ref{Ptr{Cvoid}}), device, h)
        rc == 0 || error(unsafe_string(ccall((:tn_last_error, libtngpu), Cstring, (Ptr{Cvoid},), C_NULL)))
        _ctx[] = Context(h[])
        atexit(() -> ccall((:tn_ctx_destroy, libtngpu), Int32, (Ptr{Cvoid},), _ctx[].h))
    end
    return _ctx[]
end

# The reference raises Julia errors (error("...")); status codes become the same.
function check(ctx::Context, rc::Integer)
    rc == 0 && return nothing
    error(unsafe_string(ccall((:tn_last_error, libtngpu), Cstring, (Ptr{Cvoid},), ctx.h)))
end

# ---- MPS / MPO transfer ------------------------------------------------------
function upload(ctx::Context, psi::GMPS)
    N = length(psi)
    ts = [convert(Array{ComplexF64,3}, psi[i]) for i = 1:N]
    dims = Int64[size(ts[1], 1); [size(t, 3) for t in ts]]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve ts begin
        ptrs = [Ptr{Float64}(pointer(t)) for t in ts]
        check(ctx, ccall((:tn_mps_upload, libtngpu), Int32,
                         (Ptr{Cvoid}, Int32, Int32, Ptr{Int64}, Ptr{Ptr{Float64}}, Int32, Ref{Ptr{Cvoid}}),
                         ctx.h, N, dim(psi), dims, ptrs, center(psi), h))
    end
    return h[]
end

function download!(ctx::Context, psi::GMPS, h::Ptr{Cvoid})
    N = length(psi)
    dims = zeros(Int64, N + 1)
    c = Ref{Int32}(0)
    check(ctx, ccall((:tn_mps_bonddims, libtngpu), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ref{Int32}),
                     ctx.h, h, dims, c))
    ts = [zeros(ComplexF64, dims[i], dim(psi), dims[i+1]) for i = 1:N]
    GC.@preserve ts begin
        ptrs = [Ptr{Float64}(pointer(t)) for t in ts]
        check(ctx, ccall((:tn_mps_download, libtngpu), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Float64}}),
                         ctx.h, h, ptrs))
    end
    for i = 1:N
        psi[i] = ts[i]
    end
    psi.center = c[]
    return psi
end

destroy_mps(h) = ccall((:tn_mps_destroy, libtngpu), Int32, (Ptr{Cvoid},), h)

function upload_mpo(ctx::Context, H::GMPS)
    N = length(H)
    ts = [convert(Array{ComplexF64,4}, H[i]) for i = 1:N]
    wd = Int64[size(ts[1], 1); [size(t, 4) for t in ts]]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve ts begin
        ptrs = [Ptr{Float64}(pointer(t)) for t in ts]
        check(ctx, ccall((:tn_mpo_upload, libtngpu), Int32,
                         (Ptr{Cvoid}, Int32, Int32, Ptr{Int64}, Ptr{Ptr{Float64}}, Ref{Ptr{Cvoid}}),
                         ctx.h, N, dim(H), wd, ptrs, h))
    end
    return h[]
end

# ---- dmrg (src/algorithms/mps/dmrg.jl:128-154) -------------------------------
function dmrg(psi::GMPS, H::GMPS; nsites::Int=2, krylovdim::Int=3, kryloviter::Int=2,
              minsweeps::Int=1, maxsweeps::Int=1000, tol::Float64=1e-10, tolgrad::Float64=1e-5,
              numconverges::Real=4, cutoff::Float64=1e-12, maxdim::Int=1000, mindim::Int=1,
              verbose::Bool=true, precision::Symbol=:fp64, refine::Int=0, kwargs...)
    rank(psi) != 1 && error("Psi must be a GMPS of rank 1 (vector).")
    (length(H) != length(psi) || dim(H) != dim(psi)) && error("GMPS must share the same properties.")
    ctx = context()
    hpsi = upload(ctx, psi)
    hH = upload_mpo(ctx, H)
    opts = DmrgOpts(nsites, krylovdim, kryloviter, minsweeps, maxsweeps, tol, tolgrad,
                    Float64(numconverges), cutoff, maxdim, mindim,
                    prec_code(precision), verbose, 0, -1, refine)
    energy = Ref{Float64}(0.0)
    stats = Ref(DmrgStats())
    try
        check(ctx, ccall((:tn_dmrg, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DmrgOpts}, Ref{Float64}, Ref{DmrgStats}),
                         ctx.h, hpsi, hH, opts, energy, stats))
        download!(ctx, psi, hpsi)
    finally
        destroy_mps(hpsi)
        ccall((:tn_mpo_destroy, libtngpu), Int32, (Ptr{Cvoid},), hH)
    end
    return psi, energy[]
end

# dmrg(psi, Hs::GMPS...; coeffs) over a sum of terms (dmrg.jl:128-154,
# projmpssum.jl): rank-2 terms are MPOs, rank-1 terms MPS projectors
# coeff |phi><phi| (ProjMPS(phi, psi; squared=true)).
function dmrg(psi::GMPS, Hs::GMPS...; coeffs=ones(length(Hs)), nsites::Int=2,
              krylovdim::Int=3, kryloviter::Int=2, minsweeps::Int=1, maxsweeps::Int=1000,
              tol::Float64=1e-10, tolgrad::Float64=1e-5, numconverges::Real=4,
              cutoff::Float64=1e-12, maxdim::Int=1000, mindim::Int=1, verbose::Bool=true,
              precision::Symbol=:fp64, refine::Int=0, kwargs...)
    length(Hs) == 1 && rank(Hs[1]) == 2 && coeffs == [1] &&
        return dmrg(psi, Hs[1]; nsites, krylovdim, kryloviter, minsweeps, maxsweeps, tol,
                    tolgrad, numconverges, cutoff, maxdim, mindim, verbose, precision, refine)
    ctx = context()
    hpsi = upload(ctx, psi)
    mpos = Ptr{Cvoid}[]; mc = Float64[]; projs = Ptr{Cvoid}[]; pc = Float64[]
    try
        for (H, c) in zip(Hs, coeffs)
            if rank(H) == 2
                push!(mpos, upload_mpo(ctx, H)); push!(mc, Float64(c))
            else
                push!(projs, upload(ctx, H)); push!(pc, Float64(c))
            end
        end
        opts = DmrgOpts(nsites, krylovdim, kryloviter, minsweeps, maxsweeps, tol, tolgrad,
                        Float64(numconverges), cutoff, maxdim, mindim, prec_code(precision),
                        verbose, 0, -1, refine)
        energy = Ref{Float64}(0.0)
        stats = Ref(DmrgStats())
        check(ctx, ccall((:tn_dmrg_sum, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Float64}, Int32,
                          Ptr{Ptr{Cvoid}}, Ptr{Float64}, Ref{DmrgOpts}, Ref{Float64}, Ref{DmrgStats}),
                         ctx.h, hpsi, length(mpos), mpos, mc, length(projs), projs, pc, opts,
                         energy, stats))
        download!(ctx, psi, hpsi)
        return psi, energy[]
    finally
        destroy_mps(hpsi)
        foreach(h -> ccall((:tn_mpo_destroy, libtngpu), Int32, (Ptr{Cvoid},), h), mpos)
        foreach(destroy_mps, projs)
    end
end

# ---- vmps, applyMPO, inner (vmps.jl:1-105, mpo.jl:105-250) ---------------------
struct VmpsOpts
    nsites::Int32
    minsweeps::Int32
    maxsweeps::Int32
    tol::Float64
    numconverges::Float64
    cutoff::Float64
    maxdim::Int64
    mindim::Int64
    verbose::Int32
end

function new_gmps(ctx::Context, h::Ptr{Cvoid}, like::GMPS)
    out = GMPS(1, dim(like), [zeros(ComplexF64, 1, dim(like), 1) for _ in 1:length(like)], 0)
    download!(ctx, out, h)
    destroy_mps(h)
    return out
end

function vmps(psis::GMPS...; coeffs=ones(length(psis)), nsites::Int=2, minsweeps::Int=2,
              maxsweeps::Int=200, tol::Real=1e-10, numconverges::Real=3, cutoff::Real=1e-12,
              maxdim::Int=1000, mindim::Int=1, verbose::Bool=false, kwargs...)
    ctx = context()
    hs = [upload(ctx, p) for p in psis]
    cs = ComplexF64.(coeffs)
    out = Ref{Ptr{Cvoid}}(C_NULL); cost = Ref{Float64}(0.0); sw = Ref{Int32}(0)
    try
        check(ctx, ccall((:tn_vmps, libtngpu), Int32,
                         (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{ComplexF64}, Ref{VmpsOpts},
                          Ref{Ptr{Cvoid}}, Ref{Float64}, Ref{Int32}),
                         ctx.h, length(hs), hs, cs,
                         VmpsOpts(nsites, minsweeps, maxsweeps, tol, numconverges, cutoff, maxdim,
                                  mindim, verbose), out, cost, sw))
        return new_gmps(ctx, out[], psis[1])
    finally
        foreach(destroy_mps, hs)
    end
end

function applyMPO(O::GMPS, psi::GMPS; cutoff::Real=0.0, maxdim::Int=0, mindim::Int=1, kwargs...)
    ctx = context()
    hO = upload_mpo(ctx, O); hp = upload(ctx, psi)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    try
        check(ctx, ccall((:tn_mpo_apply, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{TruncOpts}, Ref{Ptr{Cvoid}}),
                         ctx.h, hO, hp, TruncOpts(cutoff, maxdim, mindim), out))
        return new_gmps(ctx, out[], psi)
    finally
        ccall((:tn_mpo_destroy, libtngpu), Int32, (Ptr{Cvoid},), hO)
        destroy_mps(hp)
    end
end

# MPOMPOProduct (mpo.jl:147-167) through tn_mpo_mpo_apply: each rank-2 site
# [Dl, o, i, Dr] is uploaded as an MPS site [Dl, o + d*i, Dr] (the same
# column-major memory), and the fused product is reshaped back.
function fused(O::GMPS)
    d = dim(O)
    return GMPS(1, d^2, [reshape(O[i], size(O[i], 1), d^2, size(O[i], 4)) for i in 1:length(O)],
                center(O))
end

function applyMPO(O1::GMPS, O2::GMPS; cutoff::Real=0.0, maxdim::Int=0, mindim::Int=1, kwargs...)
    (rank(O1) == 2 && rank(O2) == 2) || error("applyMPO of two GMPS here takes two MPOs")
    ctx = context()
    d = dim(O1)
    ha = upload(ctx, fused(O1)); hb = upload(ctx, fused(O2))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    try
        check(ctx, ccall((:tn_mpo_mpo_apply, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ref{TruncOpts}, Ref{Ptr{Cvoid}}),
                         ctx.h, ha, hb, d, TruncOpts(cutoff, maxdim, mindim), out))
        f = new_gmps(ctx, out[], fused(O1))
        return GMPS(2, d, [reshape(f[i], size(f[i], 1), d, d, size(f[i], 3)) for i in 1:length(f)],
                    center(f))
    finally
        destroy_mps(ha); destroy_mps(hb)
    end
end

function inner(phi::GMPS, psi::GMPS)
    ctx = context()
    ha = upload(ctx, phi); hb = upload(ctx, psi)
    v = zeros(Float64, 2)
    try
        check(ctx, ccall((:tn_mps_overlap, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}), ctx.h, ha, hb, v))
        return complex(v[1], v[2])
    finally
        destroy_mps(ha); destroy_mps(hb)
    end
end

# ---- gates, applygates!, tebd (gatelist.jl:191-227, tebd.jl:3-100) -----------
function upload_gates(ctx::Context, gl::GateList, d::Integer)
    rows = length(gl.gates)
    row_len = Int32[length(r) for r in gl.gates]
    sites = Int32[s for r in gl.sites for s in r]
    gs = [convert(Array{ComplexF64}, g) for r in gl.gates for g in r]
    ns = Int32[ndims(g) ÷ 2 for g in gs]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve gs begin
        ptrs = [Ptr{Float64}(pointer(g)) for g in gs]
        check(ctx, ccall((:tn_gates_upload, libtngpu), Int32,
                         (Ptr{Cvoid}, Int32, Int32, Int32, Ptr{Int32}, Ptr{Int32}, Ptr{Int32},
                          Ptr{Ptr{Float64}}, Ref{Ptr{Cvoid}}),
                         ctx.h, length(gl), d, rows, row_len, sites, ns, ptrs, h))
    end
    return h[]
end

function applygates!(psi::GMPS, gates::GateList; cutoff::Real=0.0, maxdim::Int=0, mindim::Int=1, kwargs...)
    ctx = context()
    hpsi = upload(ctx, psi)
    hg = upload_gates(ctx, gates, dim(psi))
    t = TruncOpts(cutoff, maxdim, mindim)
    try
        check(ctx, ccall((:tn_applygates, libtngpu), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{TruncOpts}),
                         ctx.h, hpsi, hg, t))
        download!(ctx, psi, hpsi)
    finally
        destroy_mps(hpsi)
        ccall((:tn_gates_destroy, libtngpu), Int32, (Ptr{Cvoid},), hg)
    end
    return 1
end

function tebd(st::Sitetypes, psi::GMPS, H::OpList, dt::Number, tmax::Number, save::Number,
              observers::Vector=[]; cutoff::Float64=1e-12, maxdim::Int=0, mindim::Int=1,
              evol::String="imag", order::Int=2, norm::Real=0.0, precision::Symbol=:fp64, kwargs...)
    st.dim != dim(psi) && error("Sitetypes and MPS physical dimensions do not match.")
    length(psi) != length(H) && error("OpList and MPS have different lengths.")
    gates = trotterize(st, H, dt; evol=evol, order=order)
    nsteps = Int(round(tmax / dt))
    save = save < dt ? dt : save
    nsave = Int(round(save / dt))
    normal = Float64(norm)
    energy = real(sum(inner(st, psi, H, psi)))
    for observer in observers
        TensorNetworks.measure!(observer, 0.0, psi, normal, energy)
    end
    ctx = context()
    TensorNetworks.norm(psi)
    hpsi = upload(ctx, psi)
    hg = upload_gates(ctx, gates, dim(psi))
    t = TruncOpts(cutoff, maxdim, mindim)
    step = 0
    converged = false
    try
        while !converged
            ln = Ref{Float64}(0.0)
            check(ctx, ccall((:tn_tebd_steps_prec, libtngpu), Int32,
                             (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ref{TruncOpts}, Int32, Ref{Float64}),
                             ctx.h, hpsi, hg, 1, t,
                             precision == :mixed ? TN_PREC_MIXED : TN_PREC_FP64, ln))
            normal += ln[]
            step += 1
            converged = step >= nsteps
            if step % nsave == 0
                download!(ctx, psi, hpsi)
                energy = real(sum(inner(st, psi, H, psi)))
                for observer in observers
                    TensorNetworks.measure!(observer, step * dt, psi, normal, energy)
                    converged = converged || TensorNetworks.checkdone!(observer)
                end
            end
        end
        download!(ctx, psi, hpsi)
    finally
        destroy_mps(hpsi)
        ccall((:tn_gates_destroy, libtngpu), Int32, (Ptr{Cvoid},), hg)
    end
    return psi, energy
end

# ---- qjmc_simulation (qjmc.jl:28-166), one trajectory, explicit draws --------
function qjmc_simulation(st::Sitetypes, psi::GMPS, H::OpList, jumpops::OpList, tmax::Real, dt::Real,
                         observers=[]; save::Real=0, cutoff::Real=1e-12, mindim::Int=1, maxdim::Int=0,
                         draws::Vector{Float64}=rand(3 * (ceil(Int, tmax / dt) + 1)),
                         classical::Bool=true, kwargs...)
    save = save == 0 ? dt : save
    steps = Int(ceil(round(tmax / dt, digits=5)))
    savesteps = Int(ceil(round(save / dt)))
    escapeops, gates = TensorNetworks.qjmc_gates(st, H, jumpops, dt)
    all(length(s) == 1 for s in jumpops.sites) || error("multi-site jump operators are not on this path")
    ctx = context()
    hpsi = upload(ctx, psi)
    hg = upload_gates(ctx, gates, dim(psi))
    jsites = Int32[s[1] for s in jumpops.sites]
    jops = reduce(vcat, [vec(op(st, o[1])) for o in jumpops.ops])
    jco = ComplexF64.(jumpops.coeffs)
    cap = steps + 1
    jumps = zeros(Int32, cap)
    jtimes = zeros(Float64, cap)
    nj = Ref{Int32}(cap)
    used = Ref{Int64}(0)
    t = TruncOpts(cutoff, maxdim, mindim)
    try
        check(ctx, ccall((:tn_qjmc_run, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{ComplexF64}, Ptr{ComplexF64},
                          Int32, Float64, Ptr{Float64}, Int64, Ref{TruncOpts}, Int32, Int32, Ptr{Int32},
                          Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Int32}, Ptr{Float64}, Ref{Int32}, Ref{Int64}, Int32),
                         ctx.h, hpsi, hg, length(jsites), jsites, jops, jco, steps, dt, draws, length(draws),
                         t, savesteps, 0, C_NULL, C_NULL, C_NULL, jumps, jtimes, nj, used,
                         Int32(classical)))
        download!(ctx, psi, hpsi)
    finally
        destroy_mps(hpsi)
        ccall((:tn_gates_destroy, libtngpu), Int32, (Ptr{Cvoid},), hg)
    end
    return Int.(jumps[1:nj[]]), jtimes[1:nj[]]
end

# An ensemble of ntraj trajectories of qjmc_simulation in one persistent
# launch (tn_qjmc_ensemble); trajectory t draws from the Philox stream
# (seed, first_traj + t).  Returns the save times, the trajectory-averaged
# single-site observables and the jump counts.
function qjmc_ensemble(st::Sitetypes, psi::GMPS, H::OpList, jumpops::OpList, tmax::Real, dt::Real,
                       obs::OpList, ntraj::Integer; seed::Integer=0, first_traj::Integer=0,
                       save::Real=0, cutoff::Real=1e-12, mindim::Int=1, maxdim::Int=64,
                       blocks_per_sm::Integer=4)
    save = save == 0 ? dt : save
    steps = Int(ceil(round(tmax / dt, digits=5)))
    savesteps = Int(ceil(round(save / dt)))
    escapeops, gates = TensorNetworks.qjmc_gates(st, H, jumpops, dt)
    ctx = context()
    hpsi = upload(ctx, psi)
    hg = upload_gates(ctx, gates, dim(psi))
    jsites = Int32[s[1] for s in jumpops.sites]
    jops = reduce(vcat, [vec(op(st, o[1])) for o in jumpops.ops])
    jco = ComplexF64.(jumpops.coeffs)
    osites = Int32[s[1] for s in obs.sites]
    oops = reduce(vcat, [vec(c * op(st, o[1])) for (o, c) in zip(obs.ops, obs.coeffs)])
    nrows = steps ÷ savesteps + 1
    avg = zeros(ComplexF64, length(osites), nrows)   # row-major rows x terms in C order
    nj = zeros(Int32, ntraj)
    try
        check(ctx, ccall((:tn_qjmc_ensemble, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{ComplexF64},
                          Ptr{ComplexF64}, Int32, Float64, Int32, Ptr{Float64}, Int64, UInt64, UInt32,
                          Ref{TruncOpts}, Int32, Int32, Ptr{Int32}, Ptr{ComplexF64}, Ptr{ComplexF64},
                          Ptr{Int32}, Int32, Ptr{Int32}, Ptr{Float64}, Int32, Ptr{Float64}, Int32),
                         ctx.h, hpsi, hg, length(jsites), jsites, jops, jco, steps, dt, ntraj,
                         C_NULL, 0, UInt64(seed), UInt32(first_traj),
                         TruncOpts(cutoff, maxdim, mindim), savesteps, length(osites), osites,
                         oops, avg, nj, 0, C_NULL, C_NULL, blocks_per_sm, C_NULL, Int32(1)))
    finally
        destroy_mps(hpsi)
        ccall((:tn_gates_destroy, libtngpu), Int32, (Ptr{Cvoid},), hg)
    end
    return collect(0:savesteps:steps) .* dt, permutedims(avg), Int.(nj)
end

# ---- differentiated TEBD: value and gradient for an rrule ---------------------
# Segment k runs nsub TEBD steps with the Trotter gates of H_of(hs[k]) (H_of
# affine in its argument); the objective is <op at site> of the final state.
# The library returns df/dconj(G) for every uploaded gate; the chain to h
# uses the Frechet derivative of exp, the upper-right block of
# exp([A E; 0 A]) with A = tau * g and E = tau * dg/dh.
function frechet_exp(g::Array{ComplexF64}, dg::Array{ComplexF64}, tau::Number)
    n = ndims(g) ÷ 2
    d = size(g, 1)
    perm = vcat(collect(1:2:2n), collect(2:2:2n))
    A = reshape(permutedims(tau .* g, perm), d^n, d^n)
    E = reshape(permutedims(tau .* dg, perm), d^n, d^n)
    L = exp([A E; zero(A) A])[1:d^n, d^n+1:end]
    return permutedims(reshape(L, ntuple(_ -> d, 2n)), invperm(perm))
end

function tebd_objective_grad(st::Sitetypes, psi0::GMPS, H_of, hs::Vector{Float64}, dt::Real,
                             nsub::Integer, opname::String, site::Integer; cutoff::Real=1e-12,
                             maxdim::Int=0, mindim::Int=1, evol::String="real", checkpoint::Int=10,
                             broadening::Real=1e-32)
    ctx = context()
    lists = [trotterize(st, H_of(h), dt; evol=evol, order=2) for h in hs]
    handles = [upload_gates(ctx, gl, dim(psi0)) for gl in lists]
    hpsi = upload(ctx, psi0)
    steps = Int32.(repeat(0:length(hs)-1, inner=nsub))
    ngate = sum(length(g) for gl in lists for r in gl.gates for g in r)
    gbar = zeros(Float64, 2 * ngate)
    f = Ref{Float64}(0.0)
    o = convert(Array{ComplexF64}, op(st, opname))
    try
        check(ctx, ccall((:tn_tebd_grad, libtngpu), Int32,
                         (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Int32, Ptr{Int32},
                          Ref{TruncOpts}, Int32, Int32, Ptr{ComplexF64}, Float64, Ref{Float64},
                          Ptr{Float64}),
                         ctx.h, hpsi, length(handles), handles, length(steps), steps,
                         TruncOpts(cutoff, maxdim, mindim), checkpoint, site, o, broadening, f, gbar))
    finally
        destroy_mps(hpsi)
        for h in handles
            ccall((:tn_gates_destroy, libtngpu), Int32, (Ptr{Cvoid},), h)
        end
    end
    gz = reinterpret(ComplexF64, gbar)
    dh = zeros(length(hs))
    off = 0
    tfac = evol == "real" ? -im * dt : dt
    for (k, h) in enumerate(hs)
        H0, H1 = H_of(h), H_of(h + 1.0)
        gl = lists[k]
        rng = TensorNetworks.siterange(H0)
        for (r, (sites, gates)) in enumerate(zip(gl.sites, gl.gates))
            tau = (r == rng || length(gl.gates) == 1) ? tfac : tfac / 2  # 2nd order: half steps on the outer rows
            for (s, G) in zip(sites, gates)
                g0 = TensorNetworks.sitetensor(H0, st, s)
                g1 = TensorNetworks.sitetensor(H1, st, s)
                dG = frechet_exp(convert(Array{ComplexF64}, g0), convert(Array{ComplexF64}, g1 .- g0), tau)
                gb = reshape(gz[off+1:off+length(G)], size(G))
                dh[k] += real(sum(conj.(gb) .* dG))
                off += length(G)
            end
        end
    end
    return f[], dh
end

end # module
