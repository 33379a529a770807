// Concurrent quantum-jump trajectories.  Trajectories are independent
// (qjmc.jl:28-166 runs one per call); here a pool of host worker threads,
// each owning a CUDA stream, pulls trajectory indices from
// an atomic counter and runs the single-trajectory driver on its own copy of
// the initial MPS.  Gates and operators are shared read-only device data.
// Per-trajectory kernels are small (chi <= 64 at the QJMC sizes), so
// overlapping many trajectories keeps the GPU busy where one trajectory
// alone is latency bound.
#include <atomic>
#include <mutex>
#include <thread>

#include "mps.cuh"
#include "philox.cuh"

namespace tn {

struct QjmcResult {
    std::vector<int> jumps;
    std::vector<double> times;
    int64_t used = 0;
    int nrows = 0;
};
QjmcResult qjmc_run(tn_mps* psi, const tn_gates* g, int njump, const int* jsites,
                    const double* jops, const double* jcoeffs, int nsteps, double dt,
                    const double* draws, int64_t ndraws, const Trunc& t, int save_every,
                    int nobs, const int* obs_sites, const double* obs_ops, double* obs_out,
                    int max_jumps, bool classical);

// The uniform stream of trajectory `traj` under `seed`: draw k in [0, 1)
// from the 64-bit word (k % 2) of Philox4x32-10(counter = (k / 2 low, traj,
// k / 2 high, 0), key = (seed low, seed high)), its top 53 bits.
void philox_uniforms(uint64_t seed, uint32_t traj, int64_t n, double* out) {
    for (int64_t k = 0; k < n; ++k) out[k] = philox_uniform(seed, traj, (uint64_t)k);
}

void qjmc_batch(const tn_mps* psi0, const tn_gates* g, int njump, const int* jsites,
                const double* jops, const double* jcoeffs, int nsteps, double dt, int ntraj,
                const double* draws, int64_t ndraws_per_traj, uint64_t seed, const Trunc& t,
                int save_every, int nobs, const int* obs_sites, const double* obs_ops,
                double* obs_avg, int* njumps_per_traj, int nworkers) {
    TN_REQUIRE(ndraws_per_traj >= 1, "need at least one draw per trajectory");
    TN_REQUIRE(ntraj >= 1 && nworkers >= 1, "need at least one trajectory and one worker");
    TN_REQUIRE(save_every >= 1, "save_every must be >= 1");
    const int nrows = nsteps / save_every + 1;
    const size_t nout = 2 * (size_t)nrows * std::max(nobs, 1);
    std::atomic<int> next{0};
    std::mutex mu;
    std::string first_err;
    int32_t first_code = TN_OK;
    std::vector<double> total(nout, 0.0);
    nworkers = std::min(nworkers, ntraj);
    const int device = psi0->ctx->device;
    psi0->ctx->sync();  // the initial state is complete before workers read it

    auto worker = [&]() {
        Ctx ctx;
        std::vector<double> local(nout, 0.0), buf(nout, 0.0);
        std::vector<double> own(draws ? 0 : (size_t)ndraws_per_traj);
        try {
            ctx_init(ctx, device);
            for (;;) {
                const int tr = next.fetch_add(1);
                if (tr >= ntraj) break;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (first_code != TN_OK) break;
                }
                tn_mps psi;
                psi.ctx = &ctx;
                psi.N = psi0->N;
                psi.d = psi0->d;
                psi.dims = psi0->dims;
                psi.center = psi0->center;
                psi.A.resize(psi0->N);
                for (int i = 1; i <= psi0->N; ++i) {
                    psi.A[i - 1] = DBuf(&ctx, sizeof(cplx) * psi0->size(i));
                    zcopy(&ctx, psi.A[i - 1].c(), psi0->site(i), psi0->size(i));
                }
                std::fill(buf.begin(), buf.end(), 0.0);
                const double* dr = draws ? draws + (size_t)tr * ndraws_per_traj : own.data();
                if (!draws) philox_uniforms(seed, (uint32_t)tr, ndraws_per_traj, own.data());
                QjmcResult r = qjmc_run(&psi, g, njump, jsites, jops, jcoeffs, nsteps, dt,
                                        dr, ndraws_per_traj, t,
                                        save_every, nobs, obs_sites, obs_ops, buf.data(),
                                        nsteps + 1, true);
                for (size_t k = 0; k < nout; ++k) local[k] += buf[k];
                if (njumps_per_traj) njumps_per_traj[tr] = (int)r.jumps.size();
            }
        } catch (const Error& e) {
            std::lock_guard<std::mutex> lk(mu);
            if (first_code == TN_OK) {
                first_code = e.code;
                first_err = e.what();
            }
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(mu);
            if (first_code == TN_OK) {
                first_code = TN_ERR_INVALID;
                first_err = e.what();
            }
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            for (size_t k = 0; k < nout; ++k) total[k] += local[k];
        }
        ctx_release(ctx);
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < nworkers; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    if (first_code != TN_OK) throw Error(first_code, "trajectory worker: " + first_err);
    for (size_t k = 0; k < 2 * (size_t)nrows * nobs; ++k) obs_avg[k] = total[k] / ntraj;
}

}  // namespace tn
