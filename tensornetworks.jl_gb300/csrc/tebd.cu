// Gate application (structures/mps/gatelist.jl:137-227), the TEBD step loop
// (src/algorithms/mps/tebd.jl:61-84) and one quantum-jump trajectory
// (src/algorithms/mps/qjmc.jl:28-220) on a device-resident MPS.
#include <cmath>

#include "mps.cuh"

namespace tn {

// applygate (gatelist.jl:137-171) without the optional fidelity.
static void applygate(tn_mps* psi, int site, int nsites, const cplx* M, bool direction,
                      const Trunc& t, DBuf& theta, DBuf& theta2) {
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    if (nsites == 1) {
        const int64_t Dl = psi->dl(site), Dr = psi->dr(site);
        DBuf out(ctx, sizeof(cplx) * Dl * d * Dr);
        small_apply(ctx, psi->site(site), out.c(), M, d, d, Dl, Dr, Dl, Dl * d, Dl, Dl * d);
        replacesite1(psi, std::move(out), site, direction, false);
        return;
    }
    two_site(psi, site, theta);
    const int64_t Dl = psi->dl(site), Dr = psi->dr(site + 1);
    const int d2 = d * d;
    const size_t need = sizeof(cplx) * Dl * d2 * Dr;
    if (theta2.bytes < need) theta2 = DBuf(ctx, need);
    small_apply(ctx, theta.c(), theta2.c(), M, d2, d2, Dl, Dr, Dl, Dl * d2, Dl, Dl * d2);
    replacesites2(psi, theta2.c(), site, direction, false, t);
}

void applygates(tn_mps* psi, const tn_gates* g, const Trunc& t) {
    TN_REQUIRE(g->N == psi->N && g->d == psi->d, "GateList and MPS do not match.");
    DBuf theta, theta2;
    for (size_t r = 0; r < g->row_len.size(); ++r) {
        const int s0 = g->row_start[r], len = g->row_len[r];
        if (len == 0) continue;
        const int first = g->sites[s0];
        const int last = g->sites[s0 + len - 1] + g->nsites[s0 + len - 1] - 1;
        const bool direction = !(std::abs(psi->center - first) < std::abs(psi->center - last));
        for (int i = 0; i < len; ++i) {
            const int gi = s0 + (direction ? len - 1 - i : i);
            const int ctr = direction ? g->sites[gi] + g->nsites[gi] - 1 : g->sites[gi];
            movecenter(psi, ctr, t);
            applygate(psi, g->sites[gi], g->nsites[gi], g->M[gi].c(), direction, t, theta, theta2);
        }
    }
}

void tebd_steps(tn_mps* psi, const tn_gates* g, int nsteps, const Trunc& t, double* lognorm) {
    for (int s = 0; s < nsteps; ++s) {
        applygates(psi, g, t);
        const cplx n = mps_norm(psi);
        if (lognorm) *lognorm += std::log(n.x);
        mps_normalize(psi);
    }
}

std::vector<double> qjmc_rates(tn_mps* psi, const std::vector<DBuf>& LdL,
                               const std::vector<int>& sites, const std::vector<cplx>& coeffs) {
    std::vector<Term> terms(sites.size());
    for (size_t j = 0; j < sites.size(); ++j) {
        terms[j].first = sites[j];
        terms[j].len = 1;
        terms[j].dops = {LdL[j].c()};
        terms[j].coeff = cmul(coeffs[j], coeffs[j]);
    }
    std::vector<cplx> v = inner_terms(psi->ctx, psi, psi, terms);
    std::vector<double> r(v.size());
    for (size_t j = 0; j < v.size(); ++j) r[j] = std::hypot(v[j].x, v[j].y);
    return r;
}

// L^dag L as a d x d interleaved matrix
std::vector<double> ldagl(const double* L, int d) {
    std::vector<double> out(2 * (size_t)d * d, 0.0);
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            double re = 0, im = 0;
            for (int k = 0; k < d; ++k) {
                // conj(L[k,i]) * L[k,j]
                const double ar = L[2 * (k + d * i)], ai = -L[2 * (k + d * i) + 1];
                const double br = L[2 * (k + d * j)], bi = L[2 * (k + d * j) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
            }
            out[2 * (i + (size_t)d * j)] = re;
            out[2 * (i + (size_t)d * j) + 1] = im;
        }
    return out;
}

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
                    int max_jumps, bool classical) {
    Ctx* ctx = psi->ctx;
    const int d = psi->d, N = psi->N;
    TN_REQUIRE(save_every >= 1, "save_every must be >= 1");
    std::vector<DBuf> LdL(njump), Lop(njump), Obs(nobs);
    std::vector<int> sites(njump);
    std::vector<cplx> coeffs(njump);
    for (int j = 0; j < njump; ++j) {
        TN_REQUIRE(jsites[j] >= 1 && jsites[j] <= N, "jump site out of range");
        sites[j] = jsites[j];
        coeffs[j] = cmk(jcoeffs[2 * j], jcoeffs[2 * j + 1]);
        std::vector<double> m = ldagl(jops + 2 * (size_t)d * d * j, d);
        upload_op_matrix(ctx, m.data(), d, LdL[j]);
        upload_op_matrix(ctx, jops + 2 * (size_t)d * d * j, d, Lop[j]);
    }
    std::vector<Term> obs(nobs);
    for (int k = 0; k < nobs; ++k) {
        TN_REQUIRE(obs_sites[k] >= 1 && obs_sites[k] <= N, "observable site out of range");
        upload_op_matrix(ctx, obs_ops + 2 * (size_t)d * d * k, d, Obs[k]);
        obs[k].first = obs_sites[k];
        obs[k].len = 1;
        obs[k].dops = {Obs[k].c()};
        obs[k].coeff = cmk(1, 0);
    }
    QjmcResult res;
    auto measure = [&]() {
        if (nobs == 0) return;
        std::vector<cplx> v = inner_terms(ctx, psi, psi, obs);
        for (int k = 0; k < nobs; ++k) {
            obs_out[2 * ((size_t)res.nrows * nobs + k)] = v[k].x;
            obs_out[2 * ((size_t)res.nrows * nobs + k) + 1] = v[k].y;
        }
        ++res.nrows;
    };
    auto draw = [&]() -> double {
        if (res.used >= ndraws) throw Error(TN_ERR_INVALID, "uniform draw stream exhausted");
        return draws[res.used++];
    };
    double time = 0.0;
    measure();
    auto jump = [&](int idx) {
        movecenter(psi, 1, no_trunc());
        apply_site_op(psi, sites[idx], Lop[idx].c());
        movecenter(psi, N, no_trunc());
        movecenter(psi, 1, t);
        mps_normalize(psi);
        TN_REQUIRE((int)res.jumps.size() < max_jumps, "jump record capacity exceeded");
    };
    auto pick = [&](const std::vector<double>& rates, double er, double r) {
        double cum = 0.0;
        for (int j = 0; j < njump; ++j) {
            cum += rates[j];
            if (r < cum / er) return j;
        }
        return -1;
    };
    for (int i = 1; i <= nsteps; ++i) {
        applygates(psi, g, t);
        const double r0 = draw();  // qjmc.jl:64; the decision when not classical
        if (!classical) {
            // qjmc.jl:65-86: the jump probability is the norm lost in the step
            const cplx n = mps_norm(psi);
            const double prob = n.x * n.x;
            mps_normalize(psi);
            if (r0 > prob) {
                std::vector<double> rates = qjmc_rates(psi, LdL, sites, coeffs);
                double er = 0.0;
                for (double r : rates) er += r;
                const int idx = pick(rates, er, draw());
                TN_REQUIRE(idx >= 0, "no jump channel selected (all rates zero)");
                jump(idx);
                res.jumps.push_back(idx + 1);
                res.times.push_back(time + dt);
            }
            time += dt;
            if (i % save_every == 0) measure();
            continue;
        }
        mps_normalize(psi);
        std::vector<double> rates = qjmc_rates(psi, LdL, sites, coeffs);
        double er = 0.0;
        for (double r : rates) er += r;
        const double prob = std::exp(-er * dt);
        if (draw() > prob) {
            const double r = draw();
            int idx = -1;
            double cum = 0.0;
            for (int j = 0; j < njump; ++j) {
                cum += rates[j];
                if (r < cum / er) {
                    idx = j;
                    break;
                }
            }
            TN_REQUIRE(idx >= 0, "no jump channel selected (all rates zero)");
            movecenter(psi, 1, no_trunc());
            apply_site_op(psi, sites[idx], Lop[idx].c());
            movecenter(psi, N, no_trunc());
            movecenter(psi, 1, t);
            mps_normalize(psi);
            TN_REQUIRE((int)res.jumps.size() < max_jumps, "jump record capacity exceeded");
            res.jumps.push_back(idx + 1);
            res.times.push_back(time + dt);
        }
        time += dt;
        if (i % save_every == 0) measure();
    }
    (void)ctx;
    return res;
}

}  // namespace tn
