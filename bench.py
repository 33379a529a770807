#!/usr/bin/env python
"""Two-site DMRG sweeps/s at chi=1024 on the Heisenberg XXZ chain (N=100,
J=Delta=1, open boundaries, MPO bond dimension 5), mixed precision:
3xTF32 tcgen05 tensor-core H_eff products, FP64 Lanczos, environments and
truncation.

Workload: seeded random MPS of bond dimension 16 (numpy PCG64 seed 2),
ramped with maxdim 64 (2 sweeps) and 256 (2 sweeps), then W warm-up and K
timed sweeps at maxdim=1024, cutoff 1e-12, krylovdim=3, kryloviter=2.  A
sweep is one directional pass (dmrg.jl:66).  Inputs (MPS 2.7 GB, environment
blocks up to 80 MB each) are far larger than L2; no flush needed.

Reported beside it: an FP64 bond-update sample of the same state (plain FP64
path), an end-to-end run through the C ABI from pinned host buffers, the
kernel roofline from the library's CUDA-event profiler, and a CPU baseline
(the numpy FP64 restatement of the reference, one bond update at chi=1024).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tensornetworks.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "DMRG sweeps/s at chi=1024 (mixed vs FP64, |dE|<1e-9); QJMC trajectory-steps/s"
UNIT = "sweeps/s"
N_SITES, CHI, D0, SEED = 100, 1024, 16, 2


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=N_SITES)
    p.add_argument("--chi", type=int, default=CHI)
    p.add_argument("--mode", default="mixed-env64", choices=["mixed", "mixed-env64"],
                   help="precision mode of the timed sweeps: 3xTF32 H_eff and projections with "
                        "FP64 environment updates (mixed-env64, the mode that holds "
                        "|dE/E| <= 1e-9), or 3xTF32 environments as well (mixed)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-side", action="store_true", help="skip the QJMC and TEBD samples")
    p.add_argument("--kernel-sample", action="store_true",
                   help="only three mixed H_eff products at the bulk shape (kernel captures)")
    p.add_argument("--workload", default="dmrg", choices=["dmrg", "tebd-grad", "tebd", "qjmc"],
                   help="tebd-grad: the differentiated-TEBD gradient; tebd: the quench in FP64 "
                        "and mixed precision; qjmc: the batched trajectory ensemble (each its "
                        "own JSON line)")
    p.add_argument("--qjmc-traj", type=int, default=1024, help="qjmc: trajectories")
    p.add_argument("--qjmc-steps", type=int, default=500, help="qjmc: steps per trajectory")
    p.add_argument("--qjmc-single", type=int, default=2,
                   help="qjmc: trajectories of the one-at-a-time arm")
    p.add_argument("--blocks-per-sm", default="4",
                   help="qjmc: engine blocks per SM (1, 2, 4, 8), or 'auto' for the autotuner's "
                        "pick, tuned before the timed run")
    p.add_argument("--qjmc-pre", type=int, default=0,
                   help="qjmc: start every trajectory from one trajectory evolved this many "
                        "steps (untimed) instead of the all-up state")
    p.add_argument("--tebd-steps", type=int, default=60, help="tebd: steps of the quench")
    p.add_argument("--segments", type=int, default=100, help="tebd-grad: h segments")
    p.add_argument("--fd-coords", type=int, default=2,
                   help="tebd-grad: coordinates checked by central differences")
    p.add_argument("--fd-k", default="", help="tebd-grad: explicit coordinates (comma list)")
    p.add_argument("--fd-eps", default="1e-6",
                   help="tebd-grad: central-difference steps (comma list)")
    return p.parse_args()


def config(args):
    return {"workload": f"XXZ chain N={args.n} J=Delta=1 OBC, two-site DMRG at chi={args.chi} "
                        f"(maxdim=mindim={args.chi}; the 1e-12 cutoff alone settles near chi 220 "
                        f"for this chain) after a 64/256 ramp, cutoff 1e-12, krylovdim 3, kryloviter 2",
            "model": "Heisenberg XXZ MPO (w=5)", "n_sites": args.n, "chi": args.chi,
            "initial_state": f"random MPS D={D0}, numpy PCG64 seed {SEED}",
            "l2": "working set > L2 (MPS 2.7 GB, environments up to 80 MB each); no flush",
            "parallelism": "replicas only (bond-sequential sweeps)"}


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def xxz(mod, N):
    H = mod.OpList(N)
    for i in range(1, N):
        for o in "xyz":
            H.add([o, o], [i, i + 1], 1.0)
    return H


def draws(N, D, seed):
    rng = np.random.default_rng(seed)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    out = [np.reshape(rng.standard_normal(int(np.prod(s))), s, order="F") for s in shapes]
    out.append(np.reshape(rng.standard_normal(2 * min(2, D)), (1, 2, min(2, D)), order="F"))
    return out


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples (200 ms) while a region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={device}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 9]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        util = [float(r[4]) for r in rows if r[4].strip().replace(".", "").isdigit()]
        loaded = [s for s, u in zip(sm, util) if u >= 20] or sm
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[6:10]) if "Active" in v and "Not" not in v})
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ---------------------------------------------------------------------------
def cpu_bond_sample(chi, w=5, d=2, seed=0):
    """One two-site bond update of the FP64 CPU restatement at chi: Lanczos
    (krylovdim 3, 2 cycles: 5 matvecs), truncated SVD to chi, one environment
    update.  The matvecs use the reference's contraction order (left block
    and MPO tensors first, projmps.jl:103-145), as its CPU path runs them.
    Environment blocks are Hermitian per channel, synthetic."""
    import oracle as O
    rng = np.random.default_rng(seed)

    def herm_env(c):
        X = rng.standard_normal((c, w, c)) + 1j * rng.standard_normal((c, w, c))
        return X + np.conj(np.transpose(X, (2, 1, 0)))

    L, R = herm_env(chi), herm_env(chi)
    st = O.spinhalf()
    W = O.mpo_from_oplist(st, xxz(O, 8))[4]  # a bulk tensor, w = 5 on both sides
    theta = rng.standard_normal((chi, d, d, chi)) + 1j * rng.standard_normal((chi, d, d, chi))
    t0 = time.perf_counter()
    _, vec = O.lanczos_lowest(lambda x: O.core.heff2_reference_order(L, W, W, R, x), theta, 3, 2)
    M = O.fr(vec, (chi * d, d * chi))
    U, S, Vt = O.trunc_svd(M, 1e-12, chi, 1)
    A = O.fr(U, (chi, d, U.shape[1]))
    O.core.env_left(L, A, W, A)
    return time.perf_counter() - t0


def blas_threads():
    """The BLAS thread setting of the CPU restatement: the environment's
    OPENBLAS/OMP variables, else OpenBLAS's default of one thread per core."""
    for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
        if os.environ.get(k):
            return f"{k}={os.environ[k]}"
    return f"OpenBLAS default ({os.cpu_count()} threads, one per core)"


def reference_arm(args):
    """The reference's CPU path on the host cores: Julia is not installed, so
    this times the numpy FP64 restatement (the oracle) with all host BLAS
    threads, one bond update at chi per step, reported as sweeps/s."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_bond_sample(min(args.chi, 256))
    ts = [cpu_bond_sample(args.chi, seed=i) for i in range(args.steps)]
    t = float(np.mean(ts))
    value = 1.0 / (t * (args.n - 1))
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "blas_threads": blas_threads(),
                             "sample": f"one bond update at chi={args.chi} per step (5 Lanczos "
                                       f"matvecs in the reference's contraction order, SVD, env "
                                       f"update), extrapolated x{args.n - 1} bonds; Julia absent, "
                                       "numpy FP64 restatement"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def sweep_flops(dims, d=2, w=5, n_mv=5):
    """Algorithmic flops of one directional sweep over the bonds of an MPS
    with bond dimensions `dims` (N+1 entries): per bond n_mv two-site H_eff
    products, one environment update and the truncation products (the
    eigensolver excluded), 8 flops per complex multiply-add."""
    tot = 0.0
    for i in range(len(dims) - 2):
        cl, cr, k = dims[i], dims[i + 2], dims[i + 1]
        f_mv = 8.0 * (w * d * d * cl * cl * cr + 2 * w * w * d ** 3 * cl * cr + w * d * d * cl * cr * cr)
        f_env = 8.0 * (w * d * cl * cl * cr + w * w * d * d * cl * cr + w * d * cl * cr * cr)
        f_tr = 8.0 * ((d * cl) ** 2 * (d * cr) + (d * cl) * (d * cr) * k)
        tot += n_mv * f_mv + f_env + f_tr
    return tot


def ours(args):
    import ctypes as C

    import tngpu as tn
    from tngpu import _lib as L

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    ctx = tn.Context(local)
    W_mpo = tn.MPO(tn.spinhalf(), xxz(tn, args.n), ctx=ctx)
    psi = tn.randomMPS(2, args.n, D0, draws=draws(args.n, D0, SEED), ctx=ctx)
    ramp = {}
    for md in (64, 256):
        t0 = time.perf_counter()
        tn.dmrg(psi, W_mpo, maxdim=md, cutoff=1e-12, minsweeps=2, maxsweeps=2, numconverges=np.inf,
                verbose=False, precision=args.mode)
        ramp[md] = time.perf_counter() - t0

    Wu, K = args.warmup, args.steps
    if dist:
        dist.barrier()
    clk = Clocks(local)
    st = {}
    t0 = time.perf_counter()
    # the timed sweeps run with the profiler off; one profiled sweep follows
    # them.  An even total leaves the centre at site 1 for the end-to-end run
    # (a padding sweep joins the warm-ups).
    pad = (Wu + K + 1) % 2
    Wu_eff = Wu + pad
    total = Wu_eff + K + 1
    kw = dict(maxdim=args.chi, mindim=args.chi, cutoff=1e-12, numconverges=np.inf, verbose=False)
    _, E = tn.dmrg(psi, W_mpo, minsweeps=total, maxsweeps=total, precision=args.mode, stats=st,
                   profile_from_sweep=Wu_eff + K, **kw)
    wall_main = time.perf_counter() - t0
    clocks = clk.stop()
    log(f"main: {wall_main:.1f} s, sweeps {['%.2f' % s for s in st['sweep_seconds']]}, "
        f"maxdim {st['sweep_maxdim']}, E={E:.12f}, E64={st['energy_fp64']:.12f}, ramp {ramp}")
    timed = st["sweep_seconds"][Wu_eff:Wu_eff + K]
    t_timed = float(sum(timed))
    if dist:
        import torch
        tt = torch.tensor([t_timed], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_timed = float(tt.item())
    value = world * K / t_timed

    # kernel profile of the profiled sweep (CUDA events on the library's
    # stream around every launch)
    n = 8
    la, ms, fl, by = (C.c_int64 * n)(), (C.c_double * n)(), (C.c_double * n)(), (C.c_double * n)()
    ctx.check(ctx.lib.tn_profile_read(ctx.h, la, ms, fl, by))
    prof = [{"kernel": L.PROF_CLASSES[i], "launches": int(la[i]), "ms": ms[i], "flops": fl[i],
             "bytes": by[i]} for i in range(n)]
    gpu_launches = int(la[7]) * K  # launches of the profiled sweep, per timed sweep
    ph = (C.c_double * 4)()
    ctx.check(ctx.lib.tn_profile_phases(ctx.h, ph))
    phases = dict(zip(("environment", "two_site_prep", "lanczos", "truncation"), list(ph)))
    log("profile (one sweep): " + json.dumps(prof))

    pk, pk_src = peaks()
    tf32_peak = 0.5 * pk.get("bf16_tflops_sustained", pk["bf16_tflops"])
    z_peak = cublas_zgemm_tflops(local)
    tc = prof[0]
    tc_achieved = 3.0 * tc["flops"] / (tc["ms"] * 1e-3) / 1e12 if tc["ms"] > 0 else 0.0
    roof_tc = {"kernel": tc["kernel"], "bound": "tensor", "achieved": tc_achieved, "peak": tf32_peak,
               "unit": "TFLOP/s", "frac": tc_achieved / tf32_peak,
               "launches": tc["launches"], "avg_launch_ms": tc["ms"] / max(tc["launches"], 1),
               "note": "achieved counts the three TF32 passes the tensor pipe executes "
                       "(3 x 8 flops per complex multiply-add); peak = 0.5 x "
                       f"{pk_src} sustained bf16 dense: TF32 runs at half the BF16 rate"}
    own = [p for i, p in enumerate(prof) if i != 7]
    dom = max(own, key=lambda p: p["ms"])
    kern_ms = sum(p["ms"] for p in own)
    if dom is tc:
        roof = dict(roof_tc)
    else:
        ach = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
        roof = {"kernel": dom["kernel"], "bound": "fp64-pipe", "achieved": ach, "peak": z_peak,
                "unit": "TFLOP/s", "frac": ach / z_peak if z_peak else None,
                "launches": dom["launches"], "avg_launch_ms": dom["ms"] / max(dom["launches"], 1),
                "note": "FP64 SIMT kernels: peak = cuBLAS ZGEMM 4096^3 timed in this run (the "
                        "measured-peaks file has no FP64 figure); achieved = the class's "
                        "algorithmic flops (eigensolver: 16/3 n^3 + 8 n^2 k per call, the "
                        "LAPACK count) over its event time"}
    roof["share_of_kernel_time"] = dom["ms"] / kern_ms if kern_ms else None
    roof["traffic"] = None
    f_sweep = sweep_flops(psi.bonddims())
    sweep_roof = {"algorithmic_tflops_per_s": f_sweep / (t_timed / K) / 1e12, "peak_tf32": tf32_peak,
                  "frac": f_sweep / (t_timed / K) / 1e12 / tf32_peak, "sweep_flops": f_sweep,
                  "note": "per bond 5 H_eff products + environment update + truncation products "
                          "(eigensolver excluded) at the actual bond dims, over ms_per_step"}

    acc = accuracy_arms(tn, psi, W_mpo, kw)
    log("accuracy: " + json.dumps(acc))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": Wu, "ms_per_step": 1e3 * t_timed / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": f"{args.mode} (tf32x3 tensor-core H_eff and projections, f64 "
                     f"{'environments, ' if args.mode == 'mixed-env64' else ''}"
                     "Lanczos and eigensolver)",
            "data": "synthetic", "config": config(args), "clocks": clocks,
            "gpu_launches": gpu_launches, "roofline": roof, "roofline_tensor_core": roof_tc,
            "roofline_sweep": sweep_roof, "mode": args.mode,
            "energy": {"returned": E, "fp64_rayleigh": st["energy_fp64"],
                       "last_sweep_lanczos": st["sweep_energies"][total - 1]},
            "accuracy": acc, "rel_err_vs_fp64": acc[args.mode]["rel_err_vs_fp64"],
            "fp64": {"sweeps_per_s": acc["fp64_sweeps_per_s"], "sweep_s": acc["fp64_sweep_s"],
                     "method": "one plain-FP64 sweep at maxdim=mindim=chi from the same state, "
                               "device events at the sweep boundaries"},
            "mixed_vs_fp64": value / world / acc["fp64_sweeps_per_s"],
            "sweeps": {"seconds": st["sweep_seconds"], "maxdim": st["sweep_maxdim"],
                       "energies": st["sweep_energies"], "ramp_seconds": ramp,
                       "main_wall_s": wall_main, "profiled_sweep": Wu_eff + K},
            "kernel_profile": prof, "phase_seconds": phases}
    if not args.no_e2e:
        line["e2e"] = e2e_run(tn, ctx, psi, W_mpo, args, world)
        log("e2e: " + json.dumps(line["e2e"]))
    if rank == 0 and not args.no_side:
        try:
            line["qjmc"] = qjmc_sample(tn, ctx)
            log("qjmc: " + json.dumps(line["qjmc"]))
        except Exception as e:  # a side measurement never voids the headline line
            line["qjmc"] = {"error": str(e)}
        try:
            line["tebd"] = tebd_sample(tn, ctx)
            log("tebd: " + json.dumps(line["tebd"]))
        except Exception as e:
            line["tebd"] = {"error": str(e)}
    if rank == 0 and not args.no_cpu:
        try:
            t = cpu_bond_sample(args.chi)
            line["cpu_baseline"] = {"value": 1.0 / (t * (args.n - 1)), "unit": UNIT,
                                    "cores": os.cpu_count(), "kind": "port",
                                    "blas_threads": blas_threads(),
                                    "sample": f"one bond update at chi={args.chi} ({t:.1f} s: 5 "
                                              f"Lanczos matvecs in the reference's contraction "
                                              f"order, SVD, env update), x{args.n - 1} bonds; "
                                              "numpy FP64 restatement (Julia absent)"}
        except Exception as e:  # the CPU baseline never voids the headline line
            line["cpu_baseline"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def accuracy_arms(tn, psi, W_mpo, kw, modes=("mixed", "mixed-env64")):
    """From copies of the same state: one plain-FP64 sweep (its last local
    Lanczos eigenvalue, as dmrg.jl:55,98 returns, and the FP64 <psi|H|psi> of
    its final state) and one sweep in each mixed mode (whose returned energy
    is the FP64 <psi|H|psi> of its final state).  |dE/E| compares the final
    states' FP64 energies; each mixed arm's in-sweep Lanczos value is
    reported beside them."""
    pf, sf = psi.copy(), {}
    _, Ef = tn.dmrg(pf, W_mpo, minsweeps=1, maxsweeps=1, precision="fp64", stats=sf, **kw)
    E64, t64 = sf["energy_fp64"], sf["sweep_seconds"][0]
    out = {"fp64_energy": E64, "fp64_last_lanczos": Ef, "fp64_sweep_s": t64,
           "fp64_sweeps_per_s": 1.0 / t64, "fp64_maxdim": pf.maxbonddim()}
    for mode in modes:
        pm, sm = psi.copy(), {}
        _, Em = tn.dmrg(pm, W_mpo, minsweeps=1, maxsweeps=1, precision=mode, stats=sm, **kw)
        out[mode] = {"energy_fp64": Em, "rel_err_vs_fp64": abs(Em - E64) / abs(E64),
                     "last_lanczos": sm["sweep_energies"][0],
                     "lanczos_rel_dev_from_its_fp64": abs(sm["sweep_energies"][0] - Em) / abs(Em),
                     "sweep_s": sm["sweep_seconds"][0], "maxdim": pm.maxbonddim(),
                     "bonddims_identical_to_fp64": pm.bonddims() == pf.bonddims()}
        del pm
    return out


def qjmc_sample(tn, ctx, steps=200, ntraj=304):
    """Batched-QJMC sample on the DMRG line: the workload of --workload qjmc
    (N=32 Ising chain, L_i = sqrt(0.1) s-_i, all-up, dt=0.01, maxdim 64,
    cutoff 1e-10, Philox seed 2024) for `steps` steps: `ntraj` trajectories
    in one persistent engine launch against trajectory 0 alone through the
    single-trajectory driver on the same stream."""
    N, dt, seed = 32, 0.01, 2024
    H, Lj, Z = qjmc_model(tn, N)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up"] * N, ctx=ctx)
    kw = dict(cutoff=1e-10, maxdim=64, save=10 * dt)
    tn.qjmc_ensemble(st, psi, H, Lj, 2 * dt, dt, Z, 8, seed=seed, engine="device", **kw)
    stt = {}
    t0 = time.perf_counter()
    _, zav, nj = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, seed=seed,
                                  engine="device", stats=stt, **kw)
    batched = ntraj * steps / (time.perf_counter() - t0)
    draws = tn.philox_uniforms(seed, 0, 3 * steps + 3)[None, :]
    t0 = time.perf_counter()
    _, _, n1 = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 1, draws=draws,
                                engine="workers", workers=1, **kw)
    single = steps / (time.perf_counter() - t0)
    return {"traj_steps_per_s_single": single, "traj_steps_per_s_batched": batched,
            "batched_vs_single": batched / single, "jumps_traj0": {"engine": int(nj[0]),
                                                                   "single": int(n1[0])},
            "engine_fp64_tflops": stt["flops"] / (stt["kernel_ms"] * 1e-3) / 1e12,
            "z_avg_final": float(np.real(zav[-1]).mean()),
            "sample": f"{ntraj} trajectories x {steps} steps in one engine launch vs trajectory 0 "
                      f"alone through the single-trajectory driver; N=32, dt=0.01, maxdim 64, "
                      f"from the all-up state (the full run is --workload qjmc)"}


def tebd_sample(tn, ctx, pre_steps=20, steps=4):
    """TEBD quench shapes: N=64 XXZ (J=1, Delta=0.5) + staggered field
    0.2(-1)^i, Neel start, real time, 2nd order, dt=0.05, maxdim 256, cutoff
    1e-10; `steps` timed TEBD steps after `pre_steps` untimed ones."""
    import ctypes as C

    from tngpu import _lib as L
    N, dt = 64, 0.05
    H = tn.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], 1.0)
        H.add(["y", "y"], [i, i + 1], 1.0)
        H.add(["z", "z"], [i, i + 1], 0.5)
    for i in range(1, N + 1):
        H.add("z", i, 0.2 * (-1) ** i)
    st = tn.spinhalf()
    psi = tn.productMPS(st, ["up" if i % 2 else "dn" for i in range(1, N + 1)], ctx=ctx)
    gates = tn.trotterize(st, H, dt, order=2, evol="real", ctx=ctx)
    psi.norm()
    t = L.trunc(1e-10, 256, 1)
    ln = C.c_double(0.0)
    t0 = time.perf_counter()
    ctx.check(ctx.lib.tn_tebd_steps(ctx.h, psi._h, gates._h, pre_steps, C.byref(t), C.byref(ln)))
    pre_s = time.perf_counter() - t0
    chi0 = psi.maxbonddim()
    t0 = time.perf_counter()
    ctx.check(ctx.lib.tn_tebd_steps(ctx.h, psi._h, gates._h, steps, C.byref(t), C.byref(ln)))
    dt_s = time.perf_counter() - t0
    return {"steps_per_s": steps / dt_s, "chi_start": chi0, "chi_end": psi.maxbonddim(),
            "pre_steps_s": pre_s,
            "sample": f"{steps} steps after {pre_steps} untimed (t={pre_steps * dt:.2f}); N=64, "
                      "dt=0.05, maxdim 256, cutoff 1e-10, 3 gate rows per step"}


def cublas_zgemm_tflops(device):
    try:
        import torch
        a = torch.randn(4096, 4096, dtype=torch.complex128, device=f"cuda:{device}")
        b = torch.randn_like(a)
        a @ b
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(2):
            a @ b
        e1.record()
        torch.cuda.synchronize()
        return 2 * 8 * 4096 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12
    except Exception:
        return None


def e2e_run(tn, ctx, psi, W_mpo, args, world):
    """Sweeps through the C ABI from pinned host buffers: upload the MPS,
    tn_dmrg (min(K, 2) sweeps in the bench's mode), download the MPS, all
    inside the timed region (the sweep count is bounded to keep the run
    within minutes)."""
    import ctypes as C

    import torch
    from tngpu import _lib as L
    K = min(args.steps, 2)
    ts = psi.tensors()
    pinned = [torch.empty(t.size * 2, dtype=torch.float64, pin_memory=True) for t in ts]
    views = []
    for t, pbuf in zip(ts, pinned):
        v = pbuf.numpy().view(np.complex128).reshape(t.shape, order="F")
        v[...] = t
        views.append(v)
    dims = (C.c_int64 * (len(ts) + 1))(*psi.bonddims())
    nbytes = sum(t.nbytes for t in ts)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h = C.c_void_p()
    ctx.check(ctx.lib.tn_mps_upload(ctx.h, len(ts), 2, dims, L.ptr_array(views), psi.center, C.byref(h)))
    g = tn.GMPS(h, len(ts), 2, ctx)
    t_up = time.perf_counter() - t0
    st = {}
    tn.dmrg(g, W_mpo, maxdim=args.chi, mindim=args.chi, cutoff=1e-12, minsweeps=K, maxsweeps=K,
            numconverges=np.inf,
            verbose=False, precision=args.mode, stats=st)
    t_dmrg = time.perf_counter() - t0 - t_up
    out = g.bonddims()
    outs = []
    for i in range(len(ts)):
        nb = out[i] * 2 * out[i + 1] * 2
        outs.append(torch.empty(nb, dtype=torch.float64, pin_memory=True))
    ctx.check(ctx.lib.tn_mps_download(ctx.h, g._h, (L.dp * len(outs))(*[
        C.cast(o.data_ptr(), L.dp) for o in outs])))
    t = time.perf_counter() - t0
    dbytes = sum(o.numel() * 8 for o in outs)
    return {"value": world * K / t, "unit": UNIT, "h2d_bytes_per_step": nbytes // K,
            "d2h_bytes_per_step": dbytes // K,
            "breakdown_s": {"upload": t_up, "tn_dmrg": t_dmrg, "sweeps": float(sum(st["sweep_seconds"])),
                            "download": t - t_up - t_dmrg},
            "note": "upload + tn_dmrg(K sweeps; builds the environments, and at the end rebuilds "
                    "them in FP64 for the returned energy) + download, pinned host buffers"}


def kernel_sample(args):
    """Three mixed-precision H_eff products at the bulk bond shape of the
    workload (chi x chi, w = 5): the small case for detailed kernel captures.
    Operand planes (L 84 MB, theta 67 MB) exceed L2."""
    import ctypes as C

    import tngpu as tn
    ctx = tn.context()
    chi, w, d = args.chi, 5, 2
    rng = np.random.default_rng(0)

    def cr(*s):
        return np.asfortranarray(rng.standard_normal(s) + 1j * rng.standard_normal(s))

    L, R, W1, W2, th = cr(chi, w, chi), cr(chi, w, chi), cr(w, d, d, w), cr(w, d, d, w), cr(chi, d, d, chi)
    out = np.zeros_like(th)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    t = []
    for _ in range(3):
        t0 = time.perf_counter()
        ctx.check(ctx.lib.tn_heff2_apply(ctx.h, chi, chi, d, w, w, w, dp(L), dp(W1), dp(W2), dp(R),
                                         dp(th), dp(out), 1))
        t.append(time.perf_counter() - t0)
    # one FP64 truncated split of a bulk two-site tensor: lower-triangle Gram
    # (zgemm), top-half eigensolver, projection (zgemm)
    th2 = np.asfortranarray(th.reshape(2 * chi, 2 * chi, order="F"))
    X = np.zeros((2 * chi, chi), dtype=np.complex128, order="F")
    Y = np.zeros((chi, 2 * chi), dtype=np.complex128, order="F")
    S = np.zeros(chi)
    k = C.c_int64(chi)
    tr = tn._lib.trunc(0.0, chi, chi)
    t0 = time.perf_counter()
    ctx.check(ctx.lib.tn_truncate(ctx.h, 2 * chi, 2 * chi, dp(th2), C.byref(tr), 0, dp(X), dp(Y),
                                  dp(S), C.byref(k)))
    t.append(time.perf_counter() - t0)
    print(json.dumps({"kernel_sample": f"mixed H_eff chi={chi} w={w}; FP64 split {2 * chi}^2 -> {chi}",
                      "seconds": t}))


def tebd_grad_run(args):
    """Differentiated TEBD: N=32 chain, H(t) = sum Z Z + h(t) sum X with h
    piecewise constant over `segments` segments of 5 steps (values uniform in
    [0, 1], numpy PCG64 seed 5), dt=0.02, real time, 2nd order, maxdim 128,
    cutoff 1e-10, all-up start; objective <Z_16>(T).  Times the forward alone
    and the adjoint gradient (checkpoint every 10 steps); checks `fd_coords`
    coordinates (or --fd-k) by central differences (steps --fd-eps, default
    1e-6) of the same forward."""
    import tngpu as tn
    N, nsub, dt, chi, site = 32, 5, 0.02, 128, 16
    h = np.random.default_rng(5).uniform(0.0, 1.0, args.segments)

    def H_of(x):
        H = tn.OpList(N)
        for i in range(1, N):
            H.add(["z", "z"], [i, i + 1], 1.0)
        for i in range(1, N + 1):
            H.add("x", i, float(x))
        return H

    st = tn.spinhalf()
    psi0 = tn.productMPS(st, ["up"] * N)
    prob = tn.TEBDGradProblem(st, H_of, dt, nsub, "z", site, cutoff=1e-10, maxdim=chi,
                              checkpoint=10)
    clk = Clocks(0)
    t0 = time.perf_counter()
    f = prob.value(psi0, h)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    f2, back = prob.rrule(psi0, h)
    g = back()
    t_grad = time.perf_counter() - t0
    clocks = clk.stop()
    log(f"tebd-grad: forward {t_fwd:.1f} s, gradient {t_grad:.1f} s, f={f:.12f}")
    fd = []
    if args.fd_k:
        ks = [int(x) for x in args.fd_k.split(",")]
    else:
        ks = np.linspace(0, args.segments - 1, args.fd_coords).astype(int) if args.fd_coords else []
    for k in ks:
        for eps in [float(x) for x in args.fd_eps.split(",")]:
            hp, hm = h.copy(), h.copy()
            hp[k] += eps
            hm[k] -= eps
            d = (prob.value(psi0, hp) - prob.value(psi0, hm)) / (2 * eps)
            fd.append({"k": int(k), "eps": eps, "adjoint": float(g[k]), "central_difference": d,
                       "rel_err": abs(g[k] - d) / max(np.max(np.abs(g)), 1e-300)})
            log(f"tebd-grad fd: {fd[-1]}")
    line = {"metric": "differentiated TEBD gradient wall time", "value": t_grad, "unit": "s",
            "n_gpus": 1, "higher_is_better": False, "dtype": "c128 (f64)", "data": "synthetic",
            "config": {"workload": f"N={N} chain, H = sum ZZ + h_k sum X, {args.segments} segments x "
                                   f"{nsub} steps, dt={dt}, maxdim {chi}, cutoff 1e-10, all-up, "
                                   f"objective <Z_{site}>(T), checkpoint every 10 steps"},
            "forward_s": t_fwd, "gradient_over_forward": t_grad / t_fwd, "f": f,
            "f_from_gradient_pass": f2, "grad_norm": float(np.linalg.norm(g)),
            "fd_check": fd, "clocks": clocks,
            "note": "gradient = checkpoint pass + per-segment recompute with tape + reverse pass"}
    print(json.dumps(line))


def qjmc_model(tn, N=32):
    """The batched-QJMC workload: N-site Ising chain H = sum Z_i Z_i+1 + 0.8
    sum X_i, decay jumps L_i = sqrt(0.1) s-_i, <Z_i> observed."""
    H, Lj, Z = tn.OpList(N), tn.OpList(N), tn.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
        Lj.add("s-", i, np.sqrt(0.1))
        Z.add("z", i)
    return H, Lj, Z


def qjmc_run(args):
    """Batched QJMC: N=32, dt=0.01, all-up start, maxdim 64, cutoff 1e-10,
    --qjmc-traj trajectories of --qjmc-steps steps, trajectory t drawing from
    Philox stream (seed 2024, t).  The persistent device engine
    (tn_qjmc_ensemble) runs the whole ensemble; the one-trajectory-at-a-time
    arm runs the first --qjmc-single trajectories through the single-
    trajectory driver (tn_qjmc_run, one host loop per trajectory, the same
    streams).  Both report trajectory-steps/s; the engine's jump counts must
    equal the single arm's for the trajectories both ran.  With --qjmc-pre P
    every trajectory starts from one trajectory evolved P steps (the grown
    bond dimensions of the late run; the profiling case)."""
    import tngpu as tn
    N, dt, seed = 32, 0.01, 2024
    ntraj, steps = args.qjmc_traj, args.qjmc_steps
    H, Lj, Z = qjmc_model(tn, N)
    st = tn.spinhalf()
    ctx = tn.context()
    psi = tn.productMPS(st, ["up"] * N, ctx=ctx)
    kw = dict(cutoff=1e-10, maxdim=64, save=10 * dt)
    if args.qjmc_pre > 0:
        tn.qjmc_simulation(st, psi, H, Lj, args.qjmc_pre * dt, dt, [], cutoff=1e-10, maxdim=64,
                           draws=tn.philox_uniforms(seed + 1, 0, 3 * args.qjmc_pre + 3))
        psi.normalize()
    start_chi = psi.maxbonddim()
    fp64_peak = cublas_zgemm_tflops(ctx.device)
    # warm-up: a short ensemble (module load, pools)
    tn.qjmc_ensemble(st, psi, H, Lj, 2 * dt, dt, Z, 8, seed=seed, engine="device", **kw)
    tune = None
    if args.blocks_per_sm == "auto":
        width, timings, key = tn.tune_qjmc_width(st, psi, H, Lj, dt, Z, ntraj, seed=seed, **kw)
        tune = {"bucket": key, "width": width,
                "probe_seconds_per_traj_step": {str(w): t for w, t in timings.items()},
                "probe": "the first 8 steps of this ensemble at each width (empty: cached)"}
        log(f"qjmc autotune: {tune}")
    else:
        width = int(args.blocks_per_sm)
    clk = Clocks(ctx.device)
    stt = {}
    t0 = time.perf_counter()
    times, zav, nj = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, ntraj, seed=seed,
                                      engine="device", blocks_per_sm=width,
                                      stats=stt, **kw)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    rate = ntraj * steps / wall
    log(f"qjmc engine: {ntraj} x {steps} in {wall:.1f} s = {rate:.1f} traj-steps/s; {stt}")
    # one trajectory at a time: the single-trajectory driver on the same streams
    k = min(args.qjmc_single, ntraj)
    single, nj1 = None, []
    if k > 0:
        draws = np.stack([tn.philox_uniforms(seed, t, 3 * steps + 3) for t in range(k)])
        t0 = time.perf_counter()
        for t in range(k):
            _, _, n1 = tn.qjmc_ensemble(st, psi, H, Lj, steps * dt, dt, Z, 1,
                                        draws=draws[t:t + 1], engine="workers", workers=1, **kw)
            nj1.append(int(n1[0]))
        single = k * steps / (time.perf_counter() - t0)
        log(f"qjmc single: {single:.2f} traj-steps/s; jumps {nj1} vs engine {nj[:k].tolist()}")
    cpu = None
    if not args.no_cpu:
        # CPU restatement: one trajectory of the oracle, early steps from the
        # start state and late steps from a grown state (the device state of
        # one trajectory evolved to 80 % of the run)
        import oracle as Ocpu
        Ho, Lo, _ = qjmc_model(Ocpu, N)
        u = tn.philox_uniforms(seed, 0, 3 * steps + 3)
        po = Ocpu.GMPS(1, 2, psi.tensors(), psi.center)
        ce = min(steps, 30)
        t0 = time.perf_counter()
        Ocpu.qjmc_simulation(Ocpu.spinhalf(), po, Ho, Lo, ce * dt, dt,
                             Ocpu.algorithms.UniformStream(u), cutoff=1e-10, maxdim=64)
        early = ce / (time.perf_counter() - t0)
        pg = psi.copy()
        late_at = int(0.8 * steps)
        tn.qjmc_simulation(st, pg, H, Lj, late_at * dt, dt, [], cutoff=1e-10, maxdim=64,
                           draws=u)
        pl = Ocpu.GMPS(1, 2, pg.tensors(), pg.center)
        cl = 3
        t0 = time.perf_counter()
        Ocpu.qjmc_simulation(Ocpu.spinhalf(), pl, Ho, Lo, cl * dt, dt,
                             Ocpu.algorithms.UniformStream(tn.philox_uniforms(seed, 1, 12)),
                             cutoff=1e-10, maxdim=64)
        late = cl / (time.perf_counter() - t0)
        cpu = {"value": late, "unit": "traj-steps/s", "cores": os.cpu_count(), "kind": "port",
               "early_value": early,
               "sample": f"one trajectory of the numpy restatement: {cl} steps from a state "
                         f"evolved {late_at} steps (chi {pg.maxbonddim()}; value) and {ce} steps "
                         f"from the start state (chi {start_chi}; early_value)"}
        log(f"qjmc cpu: {cpu}")
    achieved = stt["flops"] / (stt["kernel_ms"] * 1e-3) / 1e12
    line = {"metric": "QJMC trajectory-steps/s", "value": ntraj * steps / (stt["kernel_ms"] * 1e-3),
            "unit": "traj-steps/s", "n_gpus": 1, "steps": steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)", "data": "synthetic",
            "config": {"workload": f"batched QJMC N={N} Ising chain H=sum ZZ + 0.8 sum X, L_i = "
                                   f"sqrt(0.1) s-_i, dt={dt}, {steps} steps, {ntraj} trajectories "
                                   f"(Philox seed {seed}), maxdim 64, cutoff 1e-10, start "
                                   + (f"state of one trajectory after {args.qjmc_pre} steps "
                                      f"(chi {start_chi})" if args.qjmc_pre else "all-up"),
                       "engine": f"persistent launch, {stt['blocks']} blocks "
                                 f"({width} per SM)", "autotune": tune},
            "wall_traj_steps_per_s": rate, "wall_s": wall,
            "single_trajectory_traj_steps_per_s": single,
            "batched_vs_single": rate / single if single else None,
            "single_arm": f"{k} trajectories one at a time through tn_qjmc_run (same streams)",
            "jumps_single_vs_engine": {"single": nj1, "engine": nj[:k].tolist()},
            "jumps_total": int(nj.sum()), "jumps_per_traj_mean": float(nj.mean()),
            "z_avg_final": float(np.real(zav[-1]).mean()),
            "z_final_sites": np.real(zav[-1]).round(6).tolist(),
            "roofline": {"kernel": "qjmc_engine_kernel", "bound": "fp64-pipe",
                         "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak if fp64_peak else None,
                         "algorithmic_flops": stt["flops"], "kernel_ms": stt["kernel_ms"],
                         "note": "achieved = the engine's own count of algorithmic FP64 flops "
                                 "(contractions, Gram products, the LAPACK count of each "
                                 "eigensolve, reduced density matrices) over the launch's CUDA-"
                                 "event time; peak = cuBLAS ZGEMM 4096^3 timed in this run"},
            "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": 2}
    print(json.dumps(line))


def tebd_step_flops(dims0, dims1, d=2):
    """Algorithmic FP64 flops of one TEBD step on an N-site chain, counted
    per bond with the larger of the bond dimensions before and after the
    step: each bond takes a two-site gate split and a truncating centre move
    in the 2nd-order schedule's three rows (1.5 gate applications and about
    as many moves per bond): the two-site tensor (8 Dl d^2 Dr Dm), the gate
    leg (8 Dl Dr d^4), the Gram matrix of order n = d D (4 n^2 (n + 1)),
    the eigensolve (16/3 n^3 + 8 n^2 k) and the projection (8 n^2 k)."""
    total = 0.0
    N = len(dims0) - 1
    for b in range(1, N):
        D = max(dims0[b], dims1[b])
        Dl = max(dims0[b - 1], dims1[b - 1])
        Dr = max(dims0[b + 1], dims1[b + 1])
        n, k = d * max(Dl, Dr), D
        split = 4.0 * n * n * (n + 1) + 16.0 / 3.0 * n ** 3 + 8.0 * n * n * k + 8.0 * n * n * k
        gate = 8.0 * Dl * d * d * Dr * D + 8.0 * Dl * Dr * d ** 4
        total += 1.5 * (gate + split) + 1.5 * split
    return total


def tebd_run(args):
    """TEBD quench: N=64 XXZ (J=1, Delta=0.5) + 0.2(-1)^i Z_i, Neel start, real
    time, 2nd order, dt=0.05, maxdim 256, cutoff 1e-10, <Z_i> and S(N/2) after
    every step; the same run in FP64 and in mixed precision (3xTF32 gate
    contractions and projections).  Reports steps/s of each and the largest
    deviation of the mixed observables from FP64 over the run."""
    import ctypes as C

    import tngpu as tn
    from tngpu import _lib as L
    N, dt, steps = 64, 0.05, args.tebd_steps
    H, Z = tn.OpList(N), tn.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], 1.0)
        H.add(["y", "y"], [i, i + 1], 1.0)
        H.add(["z", "z"], [i, i + 1], 0.5)
    for i in range(1, N + 1):
        H.add("z", i, 0.2 * (-1) ** i)
        Z.add("z", i)
    st = tn.spinhalf()
    ctx = tn.context()
    gates = tn.trotterize(st, H, dt, order=2, evol="real", ctx=ctx)
    t = L.trunc(1e-10, 256, 1)
    rec = {}
    clk = Clocks(0)
    for prec in ("fp64", "mixed"):
        psi = tn.productMPS(st, ["up" if i % 2 else "dn" for i in range(1, N + 1)], ctx=ctx)
        psi.norm()
        zs, ss, step_s, flops = [], [], 0.0, 0.0
        ln = C.c_double(0.0)
        for _ in range(steps):
            dims0 = psi.bonddims()
            t0 = time.perf_counter()
            ctx.check(ctx.lib.tn_tebd_steps_prec(ctx.h, psi._h, gates._h, 1, C.byref(t),
                                                 L.PREC[prec], C.byref(ln)))
            step_s += time.perf_counter() - t0
            flops += tebd_step_flops(dims0, psi.bonddims())
            zs.append(np.real(tn.inner(st, psi, Z, psi)))
            ss.append(psi.entropy(N // 2))
        rec[prec] = {"steps_per_s": steps / step_s, "chi_end": psi.maxbonddim(),
                     "z": np.asarray(zs), "s": np.asarray(ss), "flops": flops, "seconds": step_s}
        if prec == "fp64":
            final = psi.tensors(), psi.center
        log(f"tebd {prec}: {steps / step_s:.3f} steps/s, chi_end {psi.maxbonddim()}")
    clocks = clk.stop()
    fp64_peak = cublas_zgemm_tflops(ctx.device)
    achieved = rec["fp64"]["flops"] / rec["fp64"]["seconds"] / 1e12
    cpu = None
    if not args.no_cpu:
        # one step of the numpy restatement from the FP64 run's final state
        import oracle as Ocpu
        Ho = Ocpu.OpList(N)
        for ops, sites, c in zip(H.ops, H.sites, H.coeffs):
            Ho.add(ops, sites, c)
        rows = Ocpu.trotterize(Ocpu.spinhalf(), Ho, dt, order=2, evol="real")
        po = Ocpu.GMPS(1, 2, final[0], final[1])
        t0 = time.perf_counter()
        Ocpu.applygates(po, rows, cutoff=1e-10, maxdim=256)
        cs = time.perf_counter() - t0
        cpu = {"value": 1.0 / cs, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "blas_threads": blas_threads(),
               "sample": f"one TEBD step of the numpy restatement from the FP64 run's final "
                         f"state (chi {max(b for b in po.bonddims())}), {cs:.1f} s"}
        log(f"tebd cpu: {cpu}")
    dz = float(np.max(np.abs(rec["mixed"]["z"] - rec["fp64"]["z"])))
    ds = float(np.max(np.abs(rec["mixed"]["s"] - rec["fp64"]["s"])))
    line = {"metric": "TEBD steps/s", "value": rec["fp64"]["steps_per_s"], "unit": "steps/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "c128 (f64)", "data": "synthetic",
            "config": {"workload": f"N=64 XXZ J=1 Delta=0.5 + 0.2(-1)^i Z_i, Neel, dt=0.05, "
                                   f"{steps} steps (t={steps * dt:.2f}), maxdim 256, cutoff 1e-10"},
            "mixed_steps_per_s": rec["mixed"]["steps_per_s"],
            "chi_end": {k: v["chi_end"] for k, v in rec.items()},
            "mixed_vs_fp64_max_abs_dZ": dz, "mixed_vs_fp64_max_abs_dS": ds,
            "fp64_final_S_half": float(rec["fp64"]["s"][-1]), "clocks": clocks,
            "roofline": {"kernel": "whole TEBD step (latency-bound: one grid eigensolver per "
                                   "split)", "bound": "fp64-pipe", "achieved": achieved,
                         "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak if fp64_peak else None,
                         "note": "algorithmic FP64 flops of the FP64 run's steps (two-site "
                                 "tensor, gate leg, Gram matrix, the LAPACK count of the "
                                 "eigensolve, projection, for every gate and every truncating "
                                 "centre move, at the bond dimensions before and after each "
                                 "step) over the step time"},
            "cpu_baseline": cpu,
            "note": "steps/s counts the gate layers and the normalisation (tn_tebd_steps_prec); "
                    "observables are measured between steps, outside the timing"}
    print(json.dumps(line))


def main():
    args = parse()
    if args.workload == "tebd":
        tebd_run(args)
        return
    if args.workload == "tebd-grad":
        tebd_grad_run(args)
        return
    if args.workload == "qjmc":
        qjmc_run(args)
        return
    if args.kernel_sample:
        kernel_sample(args)
        return
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
