/*
 * tngpu.h — C ABI of libtngpu.so, the GB300 (sm_103a) implementation of the
 * finite-MPS hot path of TensorNetworks.jl (two-site DMRG, TEBD gate
 * application, quantum-jump Monte Carlo).
 *
 * Conventions (the reference's, in its structures/mps sources):
 *   - every tensor is complex double, passed as interleaved (re, im) pairs in
 *     column-major (Julia) order;
 *   - MPS site  A[Dl, d, Dr]            (structures/mps/gmps.jl:8-13)
 *   - MPO site  W[wl, d_out, d_in, wr]  (structures/mps/mpo.jl:6-12)
 *   - gate      G[o1, i1, o2, i2] for two sites, G[o, i] for one site
 *                                       (structures/mps/oplist.jl:134-156)
 *   - sites and orthogonality centres are 1-based; centre 0 means "unset"
 *     (structures/mps/abstractmps.jl:43-48).
 *
 * Every entry point returns an int32 status: TN_OK (0) or a negative code.
 * tn_last_error() gives the message of the last failure on a context.  Host
 * arrays are caller-owned and copied synchronously; handles own their device
 * memory.  A context is used by one host thread at a time and owns one CUDA
 * stream; every call has completed on the device when it returns.
 */
#ifndef TNGPU_H
#define TNGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TN_OK                 0
#define TN_ERR_INVALID       -1  /* bad argument (the reference's error("...")) */
#define TN_ERR_CUDA          -2  /* CUDA runtime / library failure             */
#define TN_ERR_OOM           -3  /* device allocation failed                   */
#define TN_ERR_TIMEOUT       -4  /* a bounded device wait ran out              */
#define TN_ERR_NUMERIC       -5  /* eigensolver / decomposition failure        */

#define TN_PREC_FP64   0   /* plain FP64 (parity mode)                          */
#define TN_PREC_MIXED  1   /* 3xTF32 tcgen05 products, FP64 Lanczos/truncation */
#define TN_PREC_MIXED_ENV64 2 /* tn_dmrg / tn_dmrg_sum only: as TN_PREC_MIXED for
                                 the H_eff products and truncation projections,
                                 with the environment blocks updated in FP64
                                 (their 3xTF32 rounding otherwise compounds
                                 along the chain into a ~1e-5 scale error of
                                 H_eff)                                       */

typedef struct tn_ctx tn_ctx;
typedef struct tn_mps tn_mps;     /* GMPS of rank 1 on the device */
typedef struct tn_mpo tn_mpo;     /* GMPS of rank 2 on the device */
typedef struct tn_gates tn_gates; /* GateList on the device       */

/* Truncation keywords of svd(x, idx; cutoff, maxdim, mindim) (src/tensors.jl:168-215). */
typedef struct tn_trunc_opts {
    double cutoff;   /* 0 = no cutoff          */
    int64_t maxdim;  /* 0 = no cap             */
    int64_t mindim;  /* default 1              */
} tn_trunc_opts;

/* Keywords of dmrg (src/algorithms/mps/dmrg.jl:3-19). */
typedef struct tn_dmrg_opts {
    int32_t nsites;        /* must be 2                                   */
    int32_t krylovdim;     /* default 3                                   */
    int32_t kryloviter;    /* default 2                                   */
    int32_t minsweeps;     /* default 1                                   */
    int32_t maxsweeps;     /* default 1000; 0 = unlimited                 */
    double tol;            /* default 1e-10                               */
    double tolgrad;        /* default 1e-5                                */
    double numconverges;   /* default 4 (Inf disables early stopping)     */
    double cutoff;         /* default 1e-12                               */
    int64_t maxdim;        /* default 1000                                */
    int64_t mindim;        /* default 1                                   */
    int32_t precision;     /* TN_PREC_FP64, _MIXED or _MIXED_ENV64        */
    int32_t verbose;       /* print the reference's per-sweep line        */
    int32_t max_bond_updates; /* 0 = run the sweeps; n > 0 = stop after n bond
                                 optimisations (a bounded timing sample)  */
    int32_t profile_from_sweep; /* >= 0: enable the kernel profiler (see
                                   tn_profile_read) from this sweep index on */
    int32_t refine;        /* mixed modes only, default 0: after each bond's
                              Lanczos, `refine` refinement steps of the Ritz
                              vector against its FP64 residual, each one
                              Lanczos cycle (krylovdim products) whose first
                              product is FP64 and fixes the projected
                              matrix's first row; no reference counterpart
                              (the reference's eigsolve is FP64 throughout) */
} tn_dmrg_opts;

typedef struct tn_dmrg_stats {
    int32_t sweeps;
    int32_t maxbonddim;
    int64_t matvecs;
    double seconds;
    double energy_fp64;    /* FP64 <psi|H|psi> at the final centre (mixed mode) */
    double last_discarded; /* discarded weight of the last truncation */
    /* optional caller-owned per-sweep records (NULL to skip), capacity sweep_cap:
     * device-timeline seconds between CUDA events recorded at sweep boundaries
     * on the context's stream, the sweep's final local energy and max bond dim */
    int32_t sweep_cap;
    double* sweep_seconds;
    double* sweep_energies;
    int32_t* sweep_maxdim;
    int32_t bond_updates;  /* bond optimisations performed */
    int32_t bond_cap;      /* optional per-bond records, capacity bond_cap */
    double* bond_seconds;  /* host wall seconds of each bond optimisation */
    int32_t* bond_chi;     /* max(chi_l, chi_r) of each optimised bond */
    /* optional, capacity bond_cap: the FP64 residual ||H x - <x|H|x> x|| of
     * each bond's unit eigenvector x before the refinement steps (the
     * Lanczos output) and after them (the vector that is split); each costs
     * one FP64 product unless a refinement step already made it */
    double* bond_resid_in;
    double* bond_resid_out;
} tn_dmrg_stats;

/* ---- kernel profiler ---------------------------------------------------------
 * CUDA events on the context's stream around each launch of a kernel class;
 * algorithmic flops and bytes are accumulated per class.  Classes:
 * 0 tensor-core GEMM (tcgen05), 1 FP64 GEMM, 2 Hermitian eigensolver,
 * 3 FP64 operator legs, 4 mixed operator leg, 5 operand conversion,
 * 6 Lanczos vector ops; class 7 holds only a launch count: every kernel this
 * library launched while the profiler was on. */
#define TN_PROF_CLASSES 8
int32_t tn_profile_enable(tn_ctx* ctx, int32_t on);
int32_t tn_profile_reset(tn_ctx* ctx);
int32_t tn_profile_read(tn_ctx* ctx, int64_t* launches, double* ms, double* flops, double* bytes);
/* Host wall seconds of the DMRG bond phases while the profiler was on (the
 * stream is synchronised at each phase end): [0] environment update,
 * [1] two-site tensor and operand preparation, [2] Lanczos, [3] truncation
 * and gauge move.  No reference counterpart (instrumentation). */
int32_t tn_profile_phases(tn_ctx* ctx, double* seconds4);

/* ---- context -------------------------------------------------------------- */
int32_t tn_ctx_create(int32_t device, tn_ctx** out);
int32_t tn_ctx_destroy(tn_ctx* ctx);
const char* tn_last_error(tn_ctx* ctx);
int32_t tn_version(void);
/* Number of kernels this library launched on ctx since creation. */
int64_t tn_kernel_launches(tn_ctx* ctx);

/* ---- MPS / MPO handles (structures/mps/gmps.jl:8-21, mps.jl:6-12, mpo.jl:6-12) */
/* bonddims has N+1 entries (bonddims[0] = bonddims[N] = 1 for a finite MPS);
 * site_ptrs[i] points at the interleaved tensor [bonddims[i], d, bonddims[i+1]]. */
int32_t tn_mps_upload(tn_ctx* ctx, int32_t N, int32_t d, const int64_t* bonddims,
                      const double* const* site_ptrs, int32_t center, tn_mps** out);
int32_t tn_mps_download(tn_ctx* ctx, const tn_mps* mps, double* const* site_ptrs);
int32_t tn_mps_bonddims(tn_ctx* ctx, const tn_mps* mps, int64_t* bonddims, int32_t* center);
int32_t tn_mps_copy(tn_ctx* ctx, const tn_mps* src, tn_mps** out);
int32_t tn_mps_destroy(tn_mps* mps);
/* wdims has N+1 entries; site_ptrs[i] is [wdims[i], d, d, wdims[i+1]]. */
int32_t tn_mpo_upload(tn_ctx* ctx, int32_t N, int32_t d, const int64_t* wdims,
                      const double* const* site_ptrs, tn_mpo** out);
int32_t tn_mpo_destroy(tn_mpo* mpo);

/* ---- gauge, norm, entropy (structures/mps/gmps.jl:29-112,184-189) -------- */
int32_t tn_mps_movecenter(tn_ctx* ctx, tn_mps* mps, int32_t site, const tn_trunc_opts* trunc);
int32_t tn_mps_norm(tn_ctx* ctx, tn_mps* mps, double* out_re_im);
int32_t tn_mps_normalize(tn_ctx* ctx, tn_mps* mps);
int32_t tn_mps_entropy(tn_ctx* ctx, tn_mps* mps, int32_t site, double* out);
/* Singular values across bond (site, site+1) after movecenter!(site); *n in:
 * capacity, out: count. */
int32_t tn_mps_singular_values(tn_ctx* ctx, tn_mps* mps, int32_t site, double* out, int64_t* n);
/* A <- op A on one site, op a d x d matrix (structures/mps/mps.jl:141-151). */
int32_t tn_mps_applyop(tn_ctx* ctx, tn_mps* mps, int32_t site, const double* op);

/* ---- expectation values (structures/mps/mps.jl:87-134) -------------------- */
/* Per-term <bra|term|ket>.  Term t covers sites term_first[t] .. +term_len[t]-1;
 * term_ops holds, term after term, term_len[t] interleaved d x d matrices (one
 * per covered site; identity where the term has no operator); coeffs are
 * complex (re, im).  out gets ntermsx(re, im). */
int32_t tn_inner_terms(tn_ctx* ctx, const tn_mps* bra, const tn_mps* ket, int32_t nterms,
                       const int32_t* term_first, const int32_t* term_len,
                       const double* term_ops, const double* coeffs, double* out);

/* ---- DMRG (src/algorithms/mps/dmrg.jl:1-154) ------------------------------ */
int32_t tn_dmrg(tn_ctx* ctx, tn_mps* psi, const tn_mpo* H, const tn_dmrg_opts* opts,
                double* energy, tn_dmrg_stats* stats);

/* dmrg(psi, Hs::GMPS...; coeffs) over a sum of terms (dmrg.jl:128-154,
 * projmpssum.jl:51-108): nmpo MPOs with coefficients mpo_coeffs (NULL: all
 * 1), each ProjMPS(psi, H, psi; rank=2), and nproj MPS terms with
 * coefficients proj_coeffs (NULL: all 1), each ProjMPS(phi, psi; rank=2,
 * squared=true), whose product is coeff |phi><phi|psi> on the two sites
 * (projmps.jl:103-145) -- the penalty that targets excited states.  The
 * initial cost is the terms' calculate (a projector contributes coeff
 * <phi|psi>, as projmps.jl:192-216 does); energy_fp64 in the stats is
 * sum_t c_t <psi|H_t|psi> + sum_p c_p |<phi_p|psi>|^2 of the final state.
 * The projector states are read, not modified. */
int32_t tn_dmrg_sum(tn_ctx* ctx, tn_mps* psi, int32_t nmpo, const tn_mpo* const* mpos,
                    const double* mpo_coeffs, int32_t nproj, const tn_mps* const* projs,
                    const double* proj_coeffs, const tn_dmrg_opts* opts, double* energy,
                    tn_dmrg_stats* stats);

/* ---- variational fitting and MPO products (vmps.jl, mpo.jl, projector.jl) -- */
/* Keywords of vmps (src/algorithms/mps/vmps.jl:2-13). */
typedef struct tn_vmps_opts {
    int32_t nsites;        /* must be 2                                   */
    int32_t minsweeps;     /* default 2                                   */
    int32_t maxsweeps;     /* default 200; 0 = unlimited                  */
    double tol;            /* default 1e-10                               */
    double numconverges;   /* default 3                                   */
    double cutoff;         /* default 1e-12                               */
    int64_t maxdim;        /* default 1000                                */
    int64_t mindim;        /* default 1                                   */
    int32_t verbose;
} tn_vmps_opts;
/* vmps(psis...) (vmps.jl:1-105): a new MPS, initially a copy of terms[0]
 * centred at site 1, fitted by two-site sweeps to sum_k coeffs[k] |terms[k]>
 * (coeffs: nterms complex (re, im) pairs, NULL = all 1; the reference
 * carries a weight inside the term's scaled tensor).  *cost receives the
 * final |fit|^2 - 2 |<target|fit>| (vmps.jl:18-25), *sweeps the count. */
int32_t tn_vmps(tn_ctx* ctx, int32_t nterms, const tn_mps* const* terms, const double* coeffs,
                const tn_vmps_opts* opts, tn_mps** out, double* cost, int32_t* sweeps);
/* applyMPO(O, psi; kwargs) = MPOMPSProduct (mpo.jl:125-146): a new MPS with
 * bond dimensions w_i * D_i, left-canonicalised, then its centre moved to
 * site 1 with the truncation trunc (NULL: none). */
int32_t tn_mpo_apply(tn_ctx* ctx, const tn_mpo* O, const tn_mps* psi, const tn_trunc_opts* trunc,
                     tn_mps** out);
/* applyMPO(O1, O2; kwargs) = MPOMPOProduct (mpo.jl:147-167) on MPOs held as
 * fused MPS handles: physical dimension d^2 with index o + d*i (the
 * column-major grouping of a rank-2 site [Dl, o, i, Dr], the grouping the
 * reference's rank-2 SVDs use).  The product O1 O2 (O1's input index summed
 * with O2's output index) is left-canonicalised, then its centre moved to
 * site 1 with the truncation trunc (NULL: none). */
int32_t tn_mpo_mpo_apply(tn_ctx* ctx, const tn_mps* O1, const tn_mps* O2, int32_t d,
                         const tn_trunc_opts* trunc, tn_mps** out);
/* psi <- a psi, a complex (re, im): the centre tensor is scaled (site 1
 * without a centre), as *(psi, a) does (abstractmps.jl:100-107). */
int32_t tn_mps_scale(tn_ctx* ctx, tn_mps* psi, const double* a);
/* <bra|ket> (inner(phi, psi), mpo.jl:181-250 with two MPSs); out = (re, im). */
int32_t tn_mps_overlap(tn_ctx* ctx, const tn_mps* bra, const tn_mps* ket, double* out);

/* ---- gates (structures/mps/gatelist.jl) ----------------------------------- */
/* nrows rows; row r has row_len[r] gates; sites/gate_nsites/gate_ptrs list all
 * gates row after row.  gate_ptrs[g] is [o1,i1,o2,i2] (2 sites) or [o,i]. */
int32_t tn_gates_upload(tn_ctx* ctx, int32_t N, int32_t d, int32_t nrows, const int32_t* row_len,
                        const int32_t* sites, const int32_t* gate_nsites,
                        const double* const* gate_ptrs, tn_gates** out);
int32_t tn_gates_destroy(tn_gates* gates);
/* applygates! (gatelist.jl:191-227). */
int32_t tn_applygates(tn_ctx* ctx, tn_mps* psi, const tn_gates* gates, const tn_trunc_opts* trunc);
/* nsteps x (applygates!, lognorm += log(norm), normalize!) (tebd.jl:61-84). */
int32_t tn_tebd_steps(tn_ctx* ctx, tn_mps* psi, const tn_gates* gates, int32_t nsteps,
                      const tn_trunc_opts* trunc, double* lognorm_accum);
/* tn_tebd_steps with a precision mode: TN_PREC_MIXED runs the two-site
 * contraction and the truncation projections as 3xTF32 tensor-core products
 * (the Gram matrix, its eigensolver, norms and normalisation stay FP64). */
int32_t tn_tebd_steps_prec(tn_ctx* ctx, tn_mps* psi, const tn_gates* gates, int32_t nsteps,
                           const tn_trunc_opts* trunc, int32_t precision, double* lognorm_accum);
/* Hand-written adjoint of a TEBD evolution with step-dependent gates (the
 * differentiated-TEBD form of the hot path; the reference has no counterpart:
 * a ChainRulesCore rrule around its tebd step loop, tebd.jl:61-84, would call
 * this).  Step s applies gates[step_gate[s]] as applygates! does
 * (gatelist.jl:191-227), then normalize!.  The objective is
 * f = <psi|O|psi>/<psi|psi> with the d x d Hermitian obs_op at obs_site,
 * evaluated after non-truncating gauge moves to that site.  psi0 is not
 * modified.  gate_grads == NULL: forward only.  Otherwise gate_grads receives
 * df/dconj(G) (df = Re sum conj(gbar) dG) for every gate of every list, in
 * list order and in each gate's upload layout ([o1,i1,o2,i2] or [o,i]),
 * interleaved re/im.  The state is checkpointed every checkpoint_every
 * steps and each segment recomputed for the reverse pass.  broadening eta:
 * inverse Gram gaps x become x / (x^2 + eta lmax^2). */
int32_t tn_tebd_grad(tn_ctx* ctx, const tn_mps* psi0, int32_t ngates, const tn_gates* const* gates,
                     int32_t nsteps, const int32_t* step_gate, const tn_trunc_opts* trunc,
                     int32_t checkpoint_every, int32_t obs_site, const double* obs_op,
                     double broadening, double* f, double* gate_grads);

/* ---- QJMC (src/algorithms/mps/qjmc.jl) ------------------------------------ */
/* Emission rates |c_j^2 <psi|L_j^dag L_j|psi>| of single-site jump operators
 * (qjmc.jl:170-220); ops are d x d interleaved, coeffs complex. */
int32_t tn_qjmc_rates(tn_ctx* ctx, tn_mps* psi, int32_t njump, const int32_t* sites,
                      const double* ops, const double* coeffs, double* rates);
/* One trajectory of qjmc_simulation (qjmc.jl:28-166).  classical != 0: the
 * escape-rate unraveling (the reference's default: one unused draw per step,
 * one for the jump decision, one more on a jump); classical == 0: the jump
 * decision compares the step's first draw with the squared norm of the
 * unnormalised state (qjmc.jl:65-86: one draw per step, one more on a jump).
 * Observables (single-site ops) are evaluated at t=0 and every save_every
 * steps into obs_out[(nsave_rows) x nobs] (re, im).  Jump indices are
 * 1-based.  *njumps in: capacity, out: count; *ndraws_used out. */
int32_t tn_qjmc_run(tn_ctx* ctx, tn_mps* psi, const tn_gates* gates, int32_t njump,
                    const int32_t* jump_sites, const double* jump_ops, const double* jump_coeffs,
                    int32_t nsteps, double dt, const double* draws, int64_t ndraws,
                    const tn_trunc_opts* trunc, int32_t save_every, int32_t nobs,
                    const int32_t* obs_sites, const double* obs_ops, double* obs_out,
                    int32_t* jumps, double* jumptimes, int32_t* njumps, int64_t* ndraws_used,
                    int32_t classical);

/* ntraj independent trajectories of the run above from the same initial MPS,
 * advanced concurrently by nworkers host threads, each with its own CUDA
 * stream.  Uniform draws: with draws != NULL trajectory t consumes
 * draws[t*ndraws_per_traj ...] (the parity mode: explicit streams); with
 * draws == NULL trajectory t draws from its own counter-based stream under
 * `seed` (tn_philox_uniforms(seed, t, ...)), ndraws_per_traj values long
 * (3*nsteps + 3 always suffices).  obs_avg gets the trajectory-averaged
 * observables (rows = t=0 and every save_every steps, nobs columns, re/im);
 * njumps_per_traj (optional) the jump counts.  The reference runs one
 * trajectory per qjmc_simulation call (qjmc.jl:28) with Julia's rand()
 * (qjmc.jl:64,97,99); ensembles are this loop. */
int32_t tn_qjmc_batch(tn_ctx* ctx, const tn_mps* psi0, const tn_gates* gates, int32_t njump,
                      const int32_t* jump_sites, const double* jump_ops, const double* jump_coeffs,
                      int32_t nsteps, double dt, int32_t ntraj, const double* draws,
                      int64_t ndraws_per_traj, uint64_t seed, const tn_trunc_opts* trunc,
                      int32_t save_every, int32_t nobs, const int32_t* obs_sites,
                      const double* obs_ops, double* obs_avg, int32_t* njumps_per_traj,
                      int32_t nworkers);
/* The same ensemble as one persistent device launch: every block of the
 * launch runs whole trajectories on the device (gates, truncated splits with
 * a one-block FP64 eigensolver, norm, emission rates, draws, jumps,
 * observables) with no host round trip per gate, each in a slot of fixed
 * capacity: trunc->maxdim >= 1 bounds every bond (with the initial state's
 * bonds), d <= 4, d x bond dimension <= 256, at most 1024 sites, one- and
 * two-site gates.  Draws as tn_qjmc_batch; with draws == NULL trajectory t
 * uses the stream tn_philox_uniforms(seed, first_traj + t, ...), unbounded.
 * jumps/jumptimes (optional, ntraj x max_jumps) receive the 1-based jump
 * channels and times of each trajectory (max_jumps = 0: none returned, one
 * per step allowed).  blocks_per_sm (1..8) sets the launch width: blocks =
 * min(ntraj, SMs x blocks_per_sm).  stats (optional, 4 values): the
 * algorithmic FP64 flops of all trajectories (contractions, Gram products,
 * the LAPACK count 16/3 n^3 + 8 n^2 k of each eigensolve), the launch's
 * device time in ms (CUDA events on the context's stream), the
 * trajectory-steps and the blocks launched.  classical as in tn_qjmc_run.
 * Replaces the loop of qjmc_simulation calls (qjmc.jl:28-166) over an
 * ensemble. */
int32_t tn_qjmc_ensemble(tn_ctx* ctx, const tn_mps* psi0, const tn_gates* gates, int32_t njump,
                         const int32_t* jump_sites, const double* jump_ops,
                         const double* jump_coeffs, int32_t nsteps, double dt, int32_t ntraj,
                         const double* draws, int64_t ndraws_per_traj, uint64_t seed,
                         uint32_t first_traj, const tn_trunc_opts* trunc, int32_t save_every,
                         int32_t nobs, const int32_t* obs_sites, const double* obs_ops,
                         double* obs_avg, int32_t* njumps_per_traj, int32_t max_jumps,
                         int32_t* jumps, double* jumptimes, int32_t blocks_per_sm,
                         double* stats, int32_t classical);
/* The per-trajectory uniform stream of tn_qjmc_batch: out[k] in [0, 1) is the
 * top 53 bits of 64-bit word k % 2 of Philox4x32-10 (Salmon et al., SC 2011)
 * at counter (k / 2 low 32 bits, trajectory, k / 2 high 32 bits, 0) under the
 * key (seed low 32 bits, seed high 32 bits).  Host only; no reference
 * counterpart (the reference draws from Julia's global RNG). */
int32_t tn_philox_uniforms(uint64_t seed, uint32_t trajectory, int64_t n, double* out);

/* ---- unit-level kernels on host buffers (for parity tests) --------------- */
/* out[a,s1',s2',c'] = sum L[a,w,b] W1[w,s1',s1,w'] W2[w',s2',s2,w''] th[b,s1,s2,c] R[c',w'',c]
 * (structures/mps/projmps.jl:103-145). */
int32_t tn_heff2_apply(tn_ctx* ctx, int64_t chil, int64_t chir, int32_t d, int64_t wl, int64_t wm,
                       int64_t wr, const double* L, const double* W1, const double* W2,
                       const double* R, const double* theta, double* out, int32_t precision);
/* The same product as tn_heff2_apply (FP64) for callers that cannot allocate
 * device memory: a host that owns the GPU's memory through its own arena and
 * budget and hands the library buffers from it, or a long run that must not
 * stop on an out-of-memory error halfway.  Every pointer (L, W1, W2, R,
 * theta, out) is a DEVICE pointer on the context's GPU that the caller owns;
 * nothing is allocated.  Intermediates live in one static 64 MiB device
 * array that the library holds on every GPU that loads it, until exit;
 * problems needing more (16*chil*chir*d^2*(wl+wr) bytes plus the merged
 * operator), or a merged operator (wl*d^2)*(d^2*wr) above 4096 entries, are
 * rejected with TN_ERR_INVALID.  All calls share that array and it keeps the
 * last call's contents: calls whose GPU work overlaps race and must be
 * serialised by the caller.  As every entry point, the call returns after its
 * work has finished.  The first call on a device resolves the array's
 * address; make it before any stream capture.
 * No counterpart in the reference: an addition for allocation-free callers. */
int32_t tn_heff2_apply_noalloc(tn_ctx* ctx, int64_t chil, int64_t chir, int32_t d, int64_t wl,
                               int64_t wm, int64_t wr, const double* L, const double* W1,
                               const double* W2, const double* R, const double* theta,
                               double* out);
/* L'[a',w',b'] = sum L[a,w,b] conj(A[a,s',a']) W[w,s',s,w'] A[b,s,b'] (projmps.jl:50-66). */
int32_t tn_env_left(tn_ctx* ctx, int64_t chil, int64_t chir, int32_t d, int64_t wl, int64_t wr,
                    const double* L, const double* A, const double* W, double* out, int32_t precision);
/* R[a,w,b] = sum A[b,s,b'] R'[a',w',b'] W[w,s',s,w'] conj(A[a,s',a']) (projmps.jl:74-95). */
int32_t tn_env_right(tn_ctx* ctx, int64_t chil, int64_t chir, int32_t d, int64_t wl, int64_t wr,
                     const double* R, const double* A, const double* W, double* out, int32_t precision);
/* Theta'[Dl,o1,o2,Dr] = sum G[o1,i1,o2,i2] A1[Dl,i1,k] A2[k,i2,Dr] (gatelist.jl:137-154). */
int32_t tn_gate2_apply(tn_ctx* ctx, int64_t chil, int64_t chim, int64_t chir, int32_t d,
                       const double* A1, const double* A2, const double* G, double* out);
/* C[m x n] = op(A) B with A column-major (m x k, or k x m when conj_a, where
 * op(A) = A^H), B column-major k x n; precision TN_PREC_FP64 runs the FP64
 * SIMT GEMM, TN_PREC_MIXED the 3xTF32 tcgen05 GEMM.  No reference
 * counterpart: the contraction primitive under tensors.jl:13-18 exposed for
 * tests and callers. */
int32_t tn_gemm(tn_ctx* ctx, int64_t m, int64_t n, int64_t k, const double* A, int32_t conj_a,
                const double* B, double* C, int32_t precision);
/* Truncated split of theta[m x n] (tensors.jl:168-227 keep rule).  direction 0:
 * X isometric, Y = S Vt; direction 1: X = U S, Y co-isometric.  X gets m x k,
 * Y k x n, S the k kept singular values; *k in: capacity, out: kept count. */
int32_t tn_truncate(tn_ctx* ctx, int64_t m, int64_t n, const double* theta,
                    const tn_trunc_opts* trunc, int32_t direction, double* X, double* Y,
                    double* S, int64_t* k);

/* Top `want` eigenpairs of the Hermitian n x n matrix G (host, interleaved,
 * column-major; the lower triangle is read): lam[g] is the g-th largest
 * eigenvalue, V[:, g] (n x want) its unit eigenvector.  The library's own
 * FP64 eigensolver (Householder tridiagonalisation, bisection, inverse
 * iteration, QR re-orthonormalisation, back-transformation), which sets the
 * cut of every truncated split in place of LAPACK's SVD at tensors.jl:191-195;
 * exposed for tests and callers.  n <= 4096. */
int32_t tn_eigh_top(tn_ctx* ctx, int64_t n, const double* G, int64_t want, double* lam, double* V);

#ifdef __cplusplus
}
#endif
#endif /* TNGPU_H */
