// Two-site DMRG on the device (src/algorithms/mps/dmrg.jl:1-154) with a
// restarted Lanczos eigensolver equivalent to the reference's call
// eigsolve(Heff, A0, 1, :SR; krylovdim, maxiter=kryloviter, ishermitian=true,
// tol=1e-14) (dmrg.jl:51-53).
//
// Lanczos vectors stay in HBM; dot products are warp-shuffle reductions; the
// projected matrix (krylovdim x krylovdim, real symmetric for a Hermitian
// operator) is diagonalised by cyclic Jacobi on the host in FP64.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>

#include "mixed.cuh"
#include "mps.cuh"
#include "ovl.cuh"

namespace tn {

static const cplx ONE = {1.0, 0.0};

// ---- small dense symmetric eigensolver (cyclic Jacobi) ----------------------
// A is n x n row-major symmetric; on return D ascending, U[i*n + j] = i-th
// component of eigenvector j.
static void jacobi_eig(std::vector<double> A, int n, std::vector<double>& D, std::vector<double>& U) {
    std::vector<double> V((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    double fro = 0;
    for (double x : A) fro += x * x;
    fro = std::sqrt(fro);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a(p, q) * a(p, q);
        if (std::sqrt(off) <= 1e-300 + 1e-17 * fro) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a(p, q);
                if (apq == 0.0) continue;
                const double tau = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < n; ++k) {  // columns
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    D.assign(n, 0.0);
    U.assign((size_t)n * n, 0.0);
    for (int j = 0; j < n; ++j) {
        D[j] = a(idx[j], idx[j]);
        for (int i = 0; i < n; ++i) U[(size_t)i * n + j] = V[(size_t)i * n + idx[j]];
    }
}

// ---- restarted Lanczos -------------------------------------------------------
struct LanczosOut {
    double eig;
    int64_t numops;
    double resid0;  // ||(H - <x0|H|x0>) x0|| of the normalised start vector
};

using MatVec = std::function<void(const cplx*, cplx*)>;

// With `first` given (one cycle, no restart): the start vector's product
// comes from `first` and fixes the whole first row of the projected matrix,
// (theta, rho, 0, ...) with theta the Rayleigh quotient and rho the residual
// norm of that product; the later products come from `mv`, whose error then
// enters only through the coefficients of the correction directions, which
// are O(rho).  With an FP64 `first` and a tensor-core `mv` this is one
// iterative-refinement step of the Ritz vector against its FP64 residual.
static LanczosOut lanczos_lowest(Ctx* ctx, int64_t n, const cplx* x0, const MatVec& mv,
                                 int krylovdim, int maxiter, double tol, DBuf& vec_out,
                                 const MatVec* first = nullptr) {
    TN_REQUIRE(krylovdim >= 1 && krylovdim <= 48, "krylovdim must be in 1..48");
    TN_REQUIRE(maxiter >= 1, "kryloviter must be >= 1");
    TN_REQUIRE(!first || maxiter == 1, "a pinned first product allows one cycle only");
    const int kd = krylovdim;
    std::vector<DBuf> V(kd + 1);
    DBuf W(ctx, sizeof(cplx) * n);
    V[0] = DBuf(ctx, sizeof(cplx) * n);
    zcopy(ctx, V[0].c(), x0, n);
    const double nrm0 = std::sqrt(znorm2(ctx, x0, n));
    zscale(ctx, V[0].c(), n, cmk(1.0 / nrm0, 0.0));

    std::vector<double> H((size_t)(kd + 1) * (kd + 1), 0.0);
    auto h = [&](int i, int j) -> double& { return H[(size_t)i * (kd + 1) + j]; };
    cplx* dcoef = ctx->s_coef.c(ctx, 4 * (kd + 2) + (size_t)(kd + 1) * (kd + 1));
    int K = 0, numiter = 1;
    int64_t numops = 0;
    std::vector<double> D, U;
    double beta = 0, resid0 = 0;
    std::vector<const cplx*> ptr;
    for (;;) {
        if (first && K == 0)
            (*first)(V[0].c(), W.c());
        else
            mv(V[K].c(), W.c());
        ++numops;
        ptr.clear();
        for (int j = 0; j <= K; ++j) ptr.push_back(V[j].c());
        // classical Gram-Schmidt, twice (full reorthogonalisation in FP64)
        multi_dot(ctx, ptr.data(), K + 1, W.c(), n, dcoef);
        multi_axpy(ctx, W.c(), ptr.data(), dcoef, K + 1, n, -1.0);
        multi_dot(ctx, ptr.data(), K + 1, W.c(), n, dcoef + (kd + 2));
        multi_axpy(ctx, W.c(), ptr.data(), dcoef + (kd + 2), K + 1, n, -1.0);
        double* hp = ctx->pinned(4 * (kd + 2));
        TN_CHECK_CUDA(cudaMemcpyAsync(hp, dcoef, sizeof(cplx) * 2 * (kd + 2),
                                      cudaMemcpyDeviceToHost, ctx->stream));
        ctx->sync();
        for (int j = 0; j <= K; ++j) {
            const double v = hp[2 * j] + hp[2 * (kd + 2 + j)];
            h(j, K) = v;
            h(K, j) = v;
        }
        if (first && K >= 1) {  // <x0|H v_K> = <H x0|v_K>: rho for K = 1, else 0
            h(0, K) = K == 1 ? resid0 : 0.0;
            h(K, 0) = h(0, K);
        }
        ++K;
        beta = std::sqrt(znorm2(ctx, W.c(), n));
        if (K == 1) resid0 = beta;
        const bool invariant = beta <= tol || K >= n;
        if (K < kd && !invariant) {
            zscale(ctx, W.c(), n, cmk(1.0 / beta, 0.0));
            V[K] = std::move(W);
            W = DBuf(ctx, sizeof(cplx) * n);
            continue;
        }
        std::vector<double> T((size_t)K * K);
        for (int i = 0; i < K; ++i)
            for (int j = 0; j < K; ++j) T[(size_t)i * K + j] = h(i, j);
        jacobi_eig(T, K, D, U);
        std::vector<double> f(K);
        for (int j = 0; j < K; ++j) f[j] = U[(size_t)(K - 1) * K + j] * beta;
        int conv = 0;
        while (conv < K && std::fabs(f[conv]) <= tol) ++conv;
        if (invariant) conv = std::max(conv, 1);
        if (conv >= 1 || numiter == maxiter) break;
        const int keep = (3 * kd + 2 * conv) / 5;
        // Ritz vectors y_j = sum_i U[i, j] v_i for j < keep
        double* hc = ctx->pinned(2 * (size_t)K * keep + 8);
        for (int j = 0; j < keep; ++j)
            for (int i = 0; i < K; ++i) {
                hc[2 * ((size_t)j * K + i)] = U[(size_t)i * K + j];
                hc[2 * ((size_t)j * K + i) + 1] = 0.0;
            }
        cplx* dU = dcoef + 2 * (kd + 2);
        TN_CHECK_CUDA(cudaMemcpyAsync(dU, hc, sizeof(cplx) * K * keep, cudaMemcpyHostToDevice,
                                      ctx->stream));
        ptr.clear();
        for (int i = 0; i < K; ++i) ptr.push_back(V[i].c());
        std::vector<DBuf> Y(keep);
        for (int j = 0; j < keep; ++j) {
            Y[j] = DBuf(ctx, sizeof(cplx) * n);
            zfill(ctx, Y[j].c(), n, cmk(0, 0));
            multi_axpy(ctx, Y[j].c(), ptr.data(), dU + (size_t)j * K, K, n, 1.0);
        }
        ctx->sync();
        for (int j = 0; j < keep; ++j) V[j] = std::move(Y[j]);
        for (int j = keep; j <= kd; ++j) V[j].reset();
        zscale(ctx, W.c(), n, cmk(1.0 / beta, 0.0));
        V[keep] = std::move(W);
        W = DBuf(ctx, sizeof(cplx) * n);
        std::fill(H.begin(), H.end(), 0.0);
        for (int j = 0; j < keep; ++j) {
            h(j, j) = D[j];
            h(keep, j) = f[j];
            h(j, keep) = f[j];
        }
        K = keep;
        ++numiter;
    }
    // Ritz vector of the lowest value
    double* hc = ctx->pinned(2 * (size_t)K + 8);
    for (int i = 0; i < K; ++i) {
        hc[2 * i] = U[(size_t)i * K + 0];
        hc[2 * i + 1] = 0.0;
    }
    cplx* dU = dcoef + 2 * (kd + 2);
    TN_CHECK_CUDA(cudaMemcpyAsync(dU, hc, sizeof(cplx) * K, cudaMemcpyHostToDevice, ctx->stream));
    ptr.clear();
    for (int i = 0; i < K; ++i) ptr.push_back(V[i].c());
    if (vec_out.bytes < sizeof(cplx) * n) vec_out = DBuf(ctx, sizeof(cplx) * n);
    zfill(ctx, vec_out.c(), n, cmk(0, 0));
    multi_axpy(ctx, vec_out.c(), ptr.data(), dU, K, n, 1.0);
    ctx->sync();
    return LanczosOut{D[0], numops, resid0};
}

// ||H x - <x|H|x> x|| for a unit vector x, with the product from mv
static double residual_norm(Ctx* ctx, int64_t n, const cplx* x, const MatVec& mv, DBuf& y) {
    if (y.bytes < sizeof(cplx) * n) y = DBuf(ctx, sizeof(cplx) * n);
    mv(x, y.c());
    cplx* d = ctx->s_coef.c(ctx, 4);
    multi_dot(ctx, &x, 1, y.c(), n, d);
    multi_axpy(ctx, y.c(), &x, d, 1, n, -1.0);
    return std::sqrt(znorm2(ctx, y.c(), n));
}

// ---- environment cache of <psi|H|psi> (ProjMPS, projmps.jl:16-95) ------------
struct EnvCache {
    Ctx* ctx;
    tn_mps* psi;
    const tn_mpo* H;
    int N;
    std::vector<DBuf> blk;
    std::vector<int64_t> a, w, b;
    DBuf edge;
    int center = 0;
    bool env_mixed = true;  // with ctx->mixed: 3xTF32 environment updates
    EnvCache(tn_mps* p, const tn_mpo* h) : ctx(p->ctx), psi(p), H(h), N(p->N) {
        blk.resize(N + 2);
        a.assign(N + 2, 1);
        w.assign(N + 2, 1);
        b.assign(N + 2, 1);
        edge = DBuf(ctx, sizeof(cplx));
        zfill(ctx, edge.c(), 1, ONE);
    }
    const cplx* block(int i, int64_t& ca, int64_t& cw, int64_t& cb) const {
        if (i < 1 || i > N) {
            ca = cw = cb = 1;
            return edge.c();
        }
        ca = a[i];
        cw = w[i];
        cb = b[i];
        return blk[i].c();
    }
    void buildleft(int i) {
        int64_t la, lw, lb;
        const cplx* L = block(i - 1, la, lw, lb);
        const int64_t na = psi->dr(i), nw = H->w[i], nb = psi->dr(i);
        DBuf out(ctx, sizeof(cplx) * na * nw * nb);
        if (ctx->mixed && env_mixed)
            mixed_env_left(ctx, L, la, lw, lb, psi->site(i), na, H->Ml[i - 1].c(), psi->d, nw,
                           psi->site(i), nb, out.c());
        else
            env_left(ctx, L, la, lw, lb, psi->site(i), na, H, i, psi->site(i), nb, psi->d, out.c());
        blk[i] = std::move(out);
        a[i] = na;
        w[i] = nw;
        b[i] = nb;
    }
    void buildright(int i) {
        int64_t ra, rw, rb;
        const cplx* R = block(i + 1, ra, rw, rb);
        const int64_t na = psi->dl(i), nw = H->w[i - 1], nb = psi->dl(i);
        DBuf out(ctx, sizeof(cplx) * na * nw * nb);
        if (ctx->mixed && env_mixed)
            mixed_env_right(ctx, R, ra, rw, rb, psi->site(i), na, H->Mr[i - 1].c(), psi->d, nw,
                            psi->site(i), nb, out.c());
        else
            env_right(ctx, R, ra, rw, rb, psi->site(i), na, H, i, psi->site(i), nb, psi->d, out.c());
        blk[i] = std::move(out);
        a[i] = na;
        w[i] = nw;
        b[i] = nb;
    }
    void movecenter(int idx) {  // abstractprojmps.jl:60-81
        if (center == 0) {
            for (int i = 1; i <= idx - 1; ++i) buildleft(i);
            for (int i = 1; i <= N - idx; ++i) buildright(N + 1 - i);
        } else if (idx > center) {
            for (int i = 1; i <= idx - center; ++i) buildleft(center - 1 + i);
        } else if (idx < center) {
            for (int i = 1; i <= center - idx; ++i) buildright(center + 1 - i);
        }
        center = idx;
    }
    cplx calculate() {  // projmps.jl:192-216
        const int c = center;
        int64_t la, lw, lb, ra, rw, rb;
        const cplx* L = block(c - 1, la, lw, lb);
        const cplx* R = block(c + 1, ra, rw, rb);
        const int64_t na = psi->dr(c), nw = H->w[c], nb = psi->dr(c);
        DBuf out(ctx, sizeof(cplx) * na * nw * nb);
        env_left(ctx, L, la, lw, lb, psi->site(c), na, H, c, psi->site(c), nb, psi->d, out.c());
        cplx* d = ctx->s_coef.c(ctx, 4);
        bilinear_dot(ctx, out.c(), R, na * nw * nb, d);
        cplx hres;
        TN_CHECK_CUDA(cudaMemcpyAsync(&hres, d, sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
        ctx->sync();
        return hres;
    }
};

void dmrg_run(tn_mps* psi, const DmrgTerms& terms, const tn_dmrg_opts& o, double* energy,
              tn_dmrg_stats* stats) {
    Ctx* ctx = psi->ctx;
    const int N = psi->N, d = psi->d;
    TN_REQUIRE(o.nsites == 2, "only two-site DMRG (nsites=2) is on this path");
    TN_REQUIRE(!terms.H.empty() || !terms.P.empty(),
               "You must provide atleast one MPS/MPO for the Hamiltonian.");
    TN_REQUIRE(terms.hc.size() == terms.H.size() && terms.pc.size() == terms.P.size(),
               "one coefficient per term");
    for (const tn_mpo* H : terms.H)
        TN_REQUIRE(H && H->N == N && H->d == d, "GMPS must share the same properties.");
    for (const tn_mps* P : terms.P)
        TN_REQUIRE(P && P->N == N && P->d == d, "GMPS must share the same properties.");
    const size_t nh = terms.H.size(), np = terms.P.size();
    TN_REQUIRE(N >= 2, "DMRG needs at least two sites");
    TN_REQUIRE(o.precision == TN_PREC_FP64 || o.precision == TN_PREC_MIXED ||
                   o.precision == TN_PREC_MIXED_ENV64,
               "unknown precision");
    const bool mixed_heff = o.precision != TN_PREC_FP64;
    TN_REQUIRE(o.refine >= 0 && o.refine <= 16, "refine must be in 0..16");
    TN_REQUIRE(o.refine == 0 || mixed_heff,
               "refine applies to the mixed precision modes (FP64 runs the reference's Lanczos)");
    auto t0 = std::chrono::steady_clock::now();
    // mixed precision: environment updates and truncation projections run on
    // the tensor cores for the whole call; restored on every exit path
    struct MixedMode {
        Ctx* c;
        bool old;
        ~MixedMode() { c->mixed = old; }
    } mode_guard{ctx, ctx->mixed};
    // ctx->mixed: H_eff products and truncation projections on the tensor
    // cores; the environment updates follow EnvCache::env_mixed (FP64 with
    // TN_PREC_MIXED_ENV64)
    ctx->mixed = mixed_heff;
    movecenter(psi, 1, no_trunc());
    std::vector<std::unique_ptr<EnvCache>> envs;
    std::vector<std::unique_ptr<OvlCache>> ovls;
    for (const tn_mpo* H : terms.H) {
        envs.emplace_back(new EnvCache(psi, H));
        envs.back()->env_mixed = o.precision == TN_PREC_MIXED;
    }
    for (const tn_mps* P : terms.P) ovls.emplace_back(new OvlCache(P, psi));
    // initial cost: the sum of the terms' calculate (projmpssum.jl:101-108);
    // a projector term contributes coeff <phi|psi> as ProjMPS's calculate does
    cplx cost = cmk(0, 0);
    for (size_t t = 0; t < nh; ++t) {
        envs[t]->movecenter(1);
        const cplx v = envs[t]->calculate();
        cost = cadd(cost, cmk(terms.hc[t] * v.x, terms.hc[t] * v.y));
    }
    for (size_t p = 0; p < np; ++p) {
        ovls[p]->movecenter(1);
        const cplx v = ovls[p]->calculate();
        cost = cadd(cost, cmk(terms.pc[p] * v.x, terms.pc[p] * v.y));
    }
    cplx lastcost = cost;
    int D = psi->maxbonddim(), lastD = D;
    double grad = 0.0;
    bool direction = false, converged = false;
    int convsweeps = 0, convgrad = 0, sweeps = 0;
    int64_t matvecs = 0;
    double last_disc = 0.0;
    const Trunc tr{o.cutoff, o.maxdim, o.mindim};
    DBuf theta, vec, out, tmp, tmp2;
    std::vector<MixedWork> mws(nh);
    std::vector<DBuf> kets(np), kets_c(np);
    int bond_updates = 0;
    bool sample_done = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    TN_CHECK_CUDA(cudaEventCreate(&ev0));
    TN_CHECK_CUDA(cudaEventCreate(&ev1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } evg{ev0, ev1};
    while (!converged) {
        if (o.profile_from_sweep >= 0 && sweeps == o.profile_from_sweep) {
            ctx->prof_flush();
            for (auto& c : ctx->prof) c = Ctx::ProfClass{};
            for (double& t : ctx->phase_s) t = 0.0;
            ctx->prof_on = true;
        }
        TN_CHECK_CUDA(cudaEventRecord(ev0, ctx->stream));
        for (int j = 1; j <= N - 1; ++j) {
            if (o.max_bond_updates > 0 && bond_updates >= o.max_bond_updates) {
                sample_done = true;
                break;
            }
            const auto tb0 = std::chrono::steady_clock::now();
            const int site = direction ? N + 1 - j : j;
            const int site1 = direction ? site - 1 : site;
            // phase clock (profiler on only): synchronise, charge the interval
            auto tp = tb0;
            auto phase = [&](int k) {
                if (!ctx->prof_on) return;
                ctx->sync();
                const auto now = std::chrono::steady_clock::now();
                ctx->phase_s[k] += std::chrono::duration<double>(now - tp).count();
                tp = now;
            };
            for (auto& e : envs) e->movecenter(site);
            for (auto& e : ovls) e->movecenter(site);
            phase(0);
            two_site(psi, site1, theta);
            const int64_t cl = psi->dl(site1), cr = psi->dr(site1 + 1);
            const int64_t n = cl * d * d * cr;
            // per MPO term: environment blocks (and mixed-precision operand planes)
            std::vector<const cplx*> Ls(nh), Rs(nh);
            std::vector<int64_t> lws(nh), rws(nh);
            for (size_t t = 0; t < nh; ++t) {
                int64_t la, lb, ra, rb;
                Ls[t] = envs[t]->block(site1 - 1, la, lws[t], lb);
                Rs[t] = envs[t]->block(site1 + 2, ra, rws[t], rb);
                if (mixed_heff)
                    mixed_prepare_env(ctx, mws[t], Ls[t], Rs[t], cl, cr, d, lws[t], rws[t]);
            }
            // per projector term: the local ket K and coeff * K
            for (size_t p = 0; p < np; ++p) {
                ovls[p]->local_ket(site1, kets[p]);
                if (kets_c[p].bytes < sizeof(cplx) * n) kets_c[p] = DBuf(ctx, sizeof(cplx) * n);
                zcopy(ctx, kets_c[p].c(), kets[p].c(), n);
                zscale(ctx, kets_c[p].c(), n, cmk(terms.pc[p], 0.0));
            }
            if (nh > 1 && tmp.bytes < sizeof(cplx) * n) tmp = DBuf(ctx, sizeof(cplx) * n);
            cplx* dproj = ctx->s_mixf.c(ctx, std::max<size_t>(np, 1));
            // y = sum_t c_t H_t x + sum_p c_p K_p <K_p|x>  (product, projmpssum.jl:74-86);
            // tensor cores for the MPO terms when tc (the mixed modes)
            auto product = [&, cl, cr, site1](const cplx* x, cplx* y, bool tc) {
                for (size_t t = 0; t < nh; ++t) {
                    cplx* dst = (t == 0) ? y : tmp.c();
                    const cplx* W12 = terms.H[t]->W12[site1 - 1].c();
                    if (tc)
                        mixed_heff2(ctx, mws[t], W12, cl, cr, d, lws[t], rws[t], x, dst);
                    else
                        heff2_fp64(ctx, Ls[t], W12, Rs[t], cl, cr, d, lws[t], rws[t], x, dst);
                    if (t == 0) {
                        if (terms.hc[0] != 1.0) zscale(ctx, y, n, cmk(terms.hc[0], 0.0));
                    } else {
                        zaxpy(ctx, y, tmp.c(), n, cmk(terms.hc[t], 0.0));
                    }
                }
                if (nh == 0) zfill(ctx, y, n, cmk(0, 0));
                for (size_t p = 0; p < np; ++p) {
                    const cplx* kp = kets[p].c();
                    const cplx* kc = kets_c[p].c();
                    multi_dot(ctx, &kp, 1, x, n, dproj + p);
                    multi_axpy(ctx, y, &kc, dproj + p, 1, n, 1.0);
                }
            };
            MatVec mv = [&](const cplx* x, cplx* y) { product(x, y, mixed_heff); };
            MatVec mv64 = [&](const cplx* x, cplx* y) { product(x, y, false); };
            phase(1);
            LanczosOut lo = lanczos_lowest(ctx, n, theta.c(), mv, o.krylovdim, o.kryloviter, 1e-14, vec);
            matvecs += lo.numops;
            // FP64-residual refinement of the Ritz vector (mixed modes): each
            // step is one Lanczos cycle whose first product is FP64
            const bool rec = stats && bond_updates < stats->bond_cap;
            double rin = -1.0;
            for (int s = 0; s < o.refine; ++s) {
                LanczosOut lr = lanczos_lowest(ctx, n, vec.c(), mv, o.krylovdim, 1, 1e-14, vec, &mv64);
                matvecs += lr.numops;
                if (s == 0) rin = lr.resid0;
                lo.eig = lr.eig;
            }
            if (rec && stats->bond_resid_in) {
                if (rin < 0.0) rin = residual_norm(ctx, n, vec.c(), mv64, tmp2);
                stats->bond_resid_in[bond_updates] = rin;
            }
            if (rec && stats->bond_resid_out)
                stats->bond_resid_out[bond_updates] =
                    (o.refine == 0 && rin >= 0.0) ? rin : residual_norm(ctx, n, vec.c(), mv64, tmp2);
            if (mixed_heff) tc_check_error(ctx);
            phase(2);
            cost = cmk(lo.eig, 0.0);
            SplitResult sr = replacesites2(psi, vec.c(), site1, direction, true, tr);
            last_disc = sr.discarded;
            phase(3);
            if (stats && bond_updates < stats->bond_cap) {
                if (stats->bond_seconds)
                    stats->bond_seconds[bond_updates] =
                        std::chrono::duration<double>(std::chrono::steady_clock::now() - tb0).count();
                if (stats->bond_chi) stats->bond_chi[bond_updates] = (int32_t)std::max(cl, cr);
            }
            ++bond_updates;
        }
        if (sample_done) break;
        for (auto& e : envs) e->movecenter(direction ? 1 : N);
        for (auto& e : ovls) e->movecenter(direction ? 1 : N);
        TN_CHECK_CUDA(cudaEventRecord(ev1, ctx->stream));
        TN_CHECK_CUDA(cudaEventSynchronize(ev1));
        float ms = 0.f;
        TN_CHECK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        if (stats && sweeps < stats->sweep_cap) {
            if (stats->sweep_seconds) stats->sweep_seconds[sweeps] = ms * 1e-3;
            if (stats->sweep_energies) stats->sweep_energies[sweeps] = cost.x;
            if (stats->sweep_maxdim) stats->sweep_maxdim[sweeps] = psi->maxbonddim();
        }
        direction = !direction;
        ++sweeps;
        D = psi->maxbonddim();
        auto diff = [](cplx x, cplx y) {
            const double ax = std::hypot(x.x, x.y);
            const double dd = std::hypot(x.x - y.x, x.y - y.y);
            return ax < 1e-10 ? dd : dd / ax;
        };
        if (sweeps >= o.minsweeps) {
            const double dd = diff(cost, lastcost);
            convsweeps = (dd < o.tol && lastD == D) ? convsweeps + 1 : 0;
            const double g = std::fabs((dd - grad) / (dd + grad));  // NaN compares false
            convgrad = (g < o.tolgrad && lastD == D) ? convgrad + 1 : 0;
            if ((double)std::max(convsweeps, convgrad) >= o.numconverges) converged = true;
            if (sweeps >= o.maxsweeps && o.maxsweeps != 0) converged = true;
        }
        grad = std::fabs(diff(cost, lastcost));
        lastcost = cost;
        lastD = D;
        if (o.verbose) printf("Sweep=%d, energy=%.12f, maxbonddim=%d \n", sweeps, cost.x, D);
    }
    if (o.profile_from_sweep >= 0 && ctx->prof_on) {
        ctx->prof_flush();
        ctx->prof_on = false;
    }
    double e64 = cost.x;
    if (!sample_done) {
        // <psi|H|psi> of the final state: sum_t c_t <psi|H_t|psi> + sum_p c_p
        // |<phi_p|psi>|^2 (the returned cost is the last local Lanczos
        // eigenvalue, as in dmrg.jl:55,98); with 3xTF32 environments it comes
        // from environments rebuilt in FP64
        const bool rebuild = o.precision == TN_PREC_MIXED;
        ctx->mixed = false;
        double acc = 0.0;
        for (size_t t = 0; t < nh; ++t) {
            if (rebuild) {
                EnvCache env64(psi, terms.H[t]);
                env64.movecenter(psi->center);
                acc += terms.hc[t] * env64.calculate().x;
            } else {
                envs[t]->movecenter(psi->center);
                acc += terms.hc[t] * envs[t]->calculate().x;
            }
        }
        for (size_t p = 0; p < np; ++p) {
            ovls[p]->movecenter(psi->center);
            const cplx v = ovls[p]->calculate();
            acc += terms.pc[p] * (v.x * v.x + v.y * v.y);
        }
        e64 = acc;
    }
    // FP64 mode returns the last local eigenvalue as the reference does; mixed
    // mode returns the FP64 <psi|H|psi> (its Lanczos values carry the
    // tensor-core accumulation bias of the environments, ~1e-5 relative)
    *energy = (mixed_heff && !sample_done) ? e64 : cost.x;
    if (stats) {
        stats->sweeps = sweeps;
        stats->maxbonddim = D;
        stats->matvecs = matvecs;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->energy_fp64 = e64;
        stats->last_discarded = last_disc;
        stats->bond_updates = bond_updates;
    }
}

}  // namespace tn
