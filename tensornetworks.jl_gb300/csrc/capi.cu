// extern "C" boundary of libtngpu.so.  Every entry point catches tn::Error and
// CUDA failures, records the message on the context and returns a status.
#include <cmath>
#include <cstring>

#include "mixed.cuh"
#include "mps.cuh"

namespace tn {
void applygates(tn_mps* psi, const tn_gates* g, const Trunc& t);
void tebd_steps(tn_mps* psi, const tn_gates* g, int nsteps, const Trunc& t, double* lognorm);
std::vector<double> qjmc_rates(tn_mps* psi, const std::vector<DBuf>& LdL,
                               const std::vector<int>& sites, const std::vector<cplx>& coeffs);
std::vector<double> ldagl(const double* L, int d);
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
void mixed_unit_heff2(Ctx* ctx, const cplx* L, const cplx* W12, const cplx* R, int64_t cl,
                      int64_t cr, int d, int64_t wl, int64_t wr, const cplx* x, cplx* y);
void mixed_gemm(Ctx* ctx, int64_t m, int64_t n, int64_t k, const cplx* A, bool conj_a,
                const cplx* B, cplx* C);
void heff2_noalloc(Ctx* ctx, int64_t cl, int64_t cr, int d, int64_t wl, int64_t wm, int64_t wr,
                   const cplx* L, const cplx* W1, const cplx* W2, const cplx* R, const cplx* theta,
                   cplx* out);
void qjmc_batch(const tn_mps* psi0, const tn_gates* g, int njump, const int* jsites,
                const double* jops, const double* jcoeffs, int nsteps, double dt, int ntraj,
                const double* draws, int64_t ndraws_per_traj, uint64_t seed, const Trunc& t,
                int save_every, int nobs, const int* obs_sites, const double* obs_ops,
                double* obs_avg, int* njumps_per_traj, int nworkers);
void qjmc_ensemble(const tn_mps* psi0, const tn_gates* g, int njump, const int* jsites,
                   const double* jops, const double* jcoeffs, int nsteps, double dt, int ntraj,
                   const double* draws, int64_t ndraws_per_traj, uint64_t seed, uint32_t first_traj,
                   const Trunc& t, int save_every, int nobs, const int* obs_sites,
                   const double* obs_ops, double* obs_avg, int* njumps_per_traj, int max_jumps,
                   int* jumps, double* jumptimes, int blocks_per_sm, double* stats,
                   bool classical);
void philox_uniforms(uint64_t seed, uint32_t traj, int64_t n, double* out);
struct VmpsResult {
    double cost;
    int sweeps;
};
VmpsResult vmps_run(tn_mps* fit, const std::vector<const tn_mps*>& terms,
                    const std::vector<cplx>& coeffs, const tn_vmps_opts& o);
void mpo_apply(const tn_mpo* O, const tn_mps* psi, const Trunc& t, tn_mps* out);
void mpo_mpo_apply(const tn_mps* A, const tn_mps* B, int d, const Trunc& t, tn_mps* out);
void mps_scale(tn_mps* psi, cplx a);
cplx mps_overlap(const tn_mps* bra, tn_mps* ket);
}  // namespace tn

using namespace tn;

static thread_local std::string g_noctx_err;

#define TN_API_BEGIN(ctxptr)        \
    tn::Ctx* _c = (ctxptr);         \
    try {
#define TN_API_END                                                  \
    return TN_OK;                                                   \
    }                                                               \
    catch (const tn::Error& e) {                                    \
        if (_c) _c->err = e.what(); else g_noctx_err = e.what();    \
        if (_c) { cudaGetLastError(); }                             \
        return e.code;                                              \
    }                                                               \
    catch (const std::bad_alloc&) {                                 \
        if (_c) _c->err = "host allocation failed";                 \
        else g_noctx_err = "host allocation failed";                \
        return TN_ERR_OOM;                                          \
    }                                                               \
    catch (const std::exception& e) {                               \
        if (_c) _c->err = e.what(); else g_noctx_err = e.what();    \
        return TN_ERR_INVALID;                                      \
    }

static Trunc to_trunc(const tn_trunc_opts* t) {
    Trunc r;
    if (t) {
        r.cutoff = t->cutoff;
        r.maxdim = t->maxdim;
        r.mindim = t->mindim;
    }
    TN_REQUIRE(r.cutoff >= 0 && r.maxdim >= 0 && r.mindim >= 0, "negative truncation parameter");
    return r;
}

static void h2d(Ctx* ctx, void* dst, const void* src, size_t bytes) {
    TN_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
}
static void d2h(Ctx* ctx, void* dst, const void* src, size_t bytes) {
    TN_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
}

extern "C" {

int32_t tn_version(void) { return 100; }

int32_t tn_ctx_create(int32_t device, tn_ctx** out) {
    try {
        TN_REQUIRE(out != nullptr, "null output pointer");
        int ndev = 0;
        TN_CHECK_CUDA(cudaGetDeviceCount(&ndev));
        TN_REQUIRE(device >= 0 && device < ndev, "device index out of range");
        tn_ctx* h = new tn_ctx();
        try {
            ctx_init(h->c, device);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return TN_OK;
    } catch (const tn::Error& e) {
        g_noctx_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_noctx_err = "host allocation failed";
        return TN_ERR_OOM;
    } catch (const std::exception& e) {
        g_noctx_err = e.what();
        return TN_ERR_INVALID;
    }
}

int32_t tn_ctx_destroy(tn_ctx* h) {
    if (!h) return TN_OK;
    ctx_release(h->c);
    delete h;
    return TN_OK;
}

const char* tn_last_error(tn_ctx* h) { return h ? h->c.err.c_str() : g_noctx_err.c_str(); }

int64_t tn_kernel_launches(tn_ctx* h) { return h ? h->c.launches : 0; }

int32_t tn_profile_enable(tn_ctx* h, int32_t on) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h, "null argument");
    h->c.prof_on = on != 0;
    TN_API_END
}

int32_t tn_profile_reset(tn_ctx* h) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h, "null argument");
    h->c.prof_flush();
    for (auto& c : h->c.prof) c = Ctx::ProfClass{};
    for (double& t : h->c.phase_s) t = 0.0;
    TN_API_END
}

int32_t tn_profile_phases(tn_ctx* h, double* seconds4) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && seconds4, "null argument");
    for (int i = 0; i < 4; ++i) seconds4[i] = h->c.phase_s[i];
    TN_API_END
}

int32_t tn_profile_read(tn_ctx* h, int64_t* launches, double* ms, double* flops, double* bytes) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && launches && ms && flops && bytes, "null argument");
    h->c.prof_flush();
    for (int i = 0; i < TN_PROF_CLASSES; ++i) {
        launches[i] = h->c.prof[i].launches;
        ms[i] = h->c.prof[i].ms;
        flops[i] = h->c.prof[i].flops;
        bytes[i] = h->c.prof[i].bytes;
    }
    TN_API_END
}

// ---- MPS ----------------------------------------------------------------------
int32_t tn_mps_upload(tn_ctx* h, int32_t N, int32_t d, const int64_t* bonddims,
                      const double* const* site_ptrs, int32_t center, tn_mps** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && out && bonddims && site_ptrs, "null argument");
    TN_REQUIRE(N >= 1 && d >= 1, "N and d must be positive");
    TN_REQUIRE(center >= 0 && center <= N, "center out of range");
    Ctx* ctx = &h->c;
    TN_CHECK_CUDA(cudaSetDevice(ctx->device));
    tn_mps* m = new tn_mps();
    m->ctx = ctx;
    m->N = N;
    m->d = d;
    m->dims.assign(bonddims, bonddims + N + 1);
    m->center = center;
    try {
        for (int i = 0; i <= N; ++i) TN_REQUIRE(m->dims[i] >= 1, "bond dimensions must be positive");
        m->A.resize(N);
        for (int i = 1; i <= N; ++i) {
            const size_t n = m->size(i);
            m->A[i - 1] = DBuf(ctx, sizeof(cplx) * n);
            h2d(ctx, m->A[i - 1].p, site_ptrs[i - 1], sizeof(cplx) * n);
        }
        ctx->sync();
    } catch (...) {
        delete m;
        throw;
    }
    *out = m;
    TN_API_END
}

int32_t tn_mps_download(tn_ctx* h, const tn_mps* m, double* const* site_ptrs) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && m && site_ptrs, "null argument");
    Ctx* ctx = &h->c;
    for (int i = 1; i <= m->N; ++i) d2h(ctx, site_ptrs[i - 1], m->A[i - 1].p, sizeof(cplx) * m->size(i));
    ctx->sync();
    TN_API_END
}

int32_t tn_mps_bonddims(tn_ctx* h, const tn_mps* m, int64_t* bonddims, int32_t* center) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m, "null argument");
    if (bonddims) memcpy(bonddims, m->dims.data(), sizeof(int64_t) * (m->N + 1));
    if (center) *center = m->center;
    TN_API_END
}

int32_t tn_mps_copy(tn_ctx* h, const tn_mps* src, tn_mps** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && src && out, "null argument");
    Ctx* ctx = &h->c;
    tn_mps* m = new tn_mps();
    m->ctx = ctx;
    m->N = src->N;
    m->d = src->d;
    m->dims = src->dims;
    m->center = src->center;
    m->A.resize(src->N);
    for (int i = 1; i <= src->N; ++i) {
        m->A[i - 1] = DBuf(ctx, sizeof(cplx) * src->size(i));
        zcopy(ctx, m->A[i - 1].c(), src->site(i), src->size(i));
    }
    ctx->sync();
    *out = m;
    TN_API_END
}

int32_t tn_mps_destroy(tn_mps* m) {
    if (!m) return TN_OK;
    if (m->ctx) cudaStreamSynchronize(m->ctx->stream);
    delete m;
    return TN_OK;
}

// ---- MPO ----------------------------------------------------------------------
int32_t tn_mpo_upload(tn_ctx* h, int32_t N, int32_t d, const int64_t* wdims,
                      const double* const* site_ptrs, tn_mpo** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && out && wdims && site_ptrs, "null argument");
    TN_REQUIRE(N >= 1 && d >= 1, "N and d must be positive");
    Ctx* ctx = &h->c;
    tn_mpo* o = new tn_mpo();
    o->ctx = ctx;
    o->N = N;
    o->d = d;
    o->w.assign(wdims, wdims + N + 1);
    try {
        TN_REQUIRE(o->w[0] == 1 && o->w[N] == 1, "MPO edge bonds must be 1");
        o->W.resize(N);
        o->Ml.resize(N);
        o->Mr.resize(N);
        o->host.resize(N);
        auto upload = [&](DBuf& dst, const std::vector<double>& v) {
            dst = DBuf(ctx, sizeof(double) * v.size());
            h2d(ctx, dst.p, v.data(), sizeof(double) * v.size());
        };
        for (int i = 1; i <= N; ++i) {
            const int64_t wl = o->w[i - 1], wr = o->w[i];
            TN_REQUIRE(wl >= 1 && wr >= 1, "MPO bond dimensions must be positive");
            const size_t n = (size_t)wl * d * d * wr;
            std::vector<double>& W = o->host[i - 1];
            W.assign(site_ptrs[i - 1], site_ptrs[i - 1] + 2 * n);
            upload(o->W[i - 1], W);
            // W[w, s', s, w'] at w + wl*(s' + d*(s + d*w'))
            std::vector<double> Ml(2 * n), Mr(2 * n);
            const int64_t nIl = wl * d, nIr = d * wr;
            for (int64_t w = 0; w < wl; ++w)
                for (int sp = 0; sp < d; ++sp)
                    for (int s = 0; s < d; ++s)
                        for (int64_t w2 = 0; w2 < wr; ++w2) {
                            const size_t src = w + wl * (sp + d * (s + d * w2));
                            const size_t il = (w + wl * s) + nIl * (sp + d * w2);
                            const size_t ir = (sp + d * w2) + nIr * (w + wl * s);
                            Ml[2 * il] = W[2 * src];
                            Ml[2 * il + 1] = W[2 * src + 1];
                            Mr[2 * ir] = W[2 * src];
                            Mr[2 * ir + 1] = W[2 * src + 1];
                        }
            upload(o->Ml[i - 1], Ml);
            upload(o->Mr[i - 1], Mr);
        }
        // merged two-site operators for H_eff
        o->W12.resize(std::max(N - 1, 0));
        for (int i = 1; i <= N - 1; ++i) {
            const int64_t wl = o->w[i - 1], wm = o->w[i], wr = o->w[i + 1];
            const std::vector<double>& A = o->host[i - 1];
            const std::vector<double>& B = o->host[i];
            const int64_t nI = wl * d * d, nJ = (int64_t)d * d * wr;
            std::vector<double> M(2 * (size_t)nI * nJ, 0.0);
            for (int64_t w = 0; w < wl; ++w)
                for (int s1 = 0; s1 < d; ++s1)
                    for (int s2 = 0; s2 < d; ++s2)
                        for (int p1 = 0; p1 < d; ++p1)
                            for (int p2 = 0; p2 < d; ++p2)
                                for (int64_t w2 = 0; w2 < wr; ++w2) {
                                    double re = 0, im = 0;
                                    for (int64_t v = 0; v < wm; ++v) {
                                        const size_t ia = w + wl * (p1 + d * (s1 + d * v));
                                        const size_t ib = v + wm * (p2 + d * (s2 + d * w2));
                                        const double ar = A[2 * ia], ai = A[2 * ia + 1];
                                        const double br = B[2 * ib], bi = B[2 * ib + 1];
                                        re += ar * br - ai * bi;
                                        im += ar * bi + ai * br;
                                    }
                                    const size_t I = w + wl * (s1 + d * s2);
                                    const size_t J = p1 + d * (p2 + d * w2);
                                    M[2 * (I + nI * J)] = re;
                                    M[2 * (I + nI * J) + 1] = im;
                                }
            upload(o->W12[i - 1], M);
        }
        ctx->sync();
    } catch (...) {
        delete o;
        throw;
    }
    *out = o;
    TN_API_END
}

int32_t tn_mpo_destroy(tn_mpo* o) {
    if (!o) return TN_OK;
    if (o->ctx) cudaStreamSynchronize(o->ctx->stream);
    delete o;
    return TN_OK;
}

// ---- gauge / norm / entropy ------------------------------------------------------
int32_t tn_mps_movecenter(tn_ctx* h, tn_mps* m, int32_t site, const tn_trunc_opts* t) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m, "null argument");
    movecenter(m, site, to_trunc(t));
    m->ctx->sync();
    TN_API_END
}

int32_t tn_mps_norm(tn_ctx* h, tn_mps* m, double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m && out, "null argument");
    cplx n = mps_norm(m);
    out[0] = n.x;
    out[1] = n.y;
    TN_API_END
}

int32_t tn_mps_normalize(tn_ctx* h, tn_mps* m) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m, "null argument");
    mps_normalize(m);
    m->ctx->sync();
    TN_API_END
}

int32_t tn_mps_singular_values(tn_ctx* h, tn_mps* m, int32_t site, double* out, int64_t* n) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m && out && n, "null argument");
    TN_REQUIRE(site >= 1 && site <= m->N, "The index is out of range.");
    std::vector<double> S = singular_values(m, site);
    TN_REQUIRE((int64_t)S.size() <= *n, "output capacity too small");
    memcpy(out, S.data(), sizeof(double) * S.size());
    *n = (int64_t)S.size();
    TN_API_END
}

int32_t tn_mps_entropy(tn_ctx* h, tn_mps* m, int32_t site, double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m && out, "null argument");
    TN_REQUIRE(site >= 1 && site <= m->N, "The index is out of range.");
    std::vector<double> S = singular_values(m, site);
    double e = 0.0;
    for (double s : S) {
        const double s2 = s * s;
        e -= s2 * std::log(s2);  // an exact zero gives NaN, as in gmps.jl:188
    }
    *out = e;
    TN_API_END
}

int32_t tn_mps_applyop(tn_ctx* h, tn_mps* m, int32_t site, const double* op) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(m && op, "null argument");
    TN_REQUIRE(site >= 1 && site <= m->N, "site out of range");
    DBuf M;
    upload_op_matrix(m->ctx, op, m->d, M);
    apply_site_op(m, site, M.c());
    m->ctx->sync();
    TN_API_END
}

int32_t tn_inner_terms(tn_ctx* h, const tn_mps* bra, const tn_mps* ket, int32_t nterms,
                       const int32_t* term_first, const int32_t* term_len, const double* term_ops,
                       const double* coeffs, double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(bra && ket && out, "null argument");
    TN_REQUIRE(nterms >= 0, "negative term count");
    Ctx* ctx = &h->c;
    const int d = ket->d;
    std::vector<Term> terms(nterms);
    std::vector<DBuf> mats;
    size_t off = 0;
    for (int t = 0; t < nterms; ++t) {
        terms[t].first = term_first[t];
        terms[t].len = term_len[t];
        TN_REQUIRE(term_len[t] >= 1, "term length must be positive");
        terms[t].coeff = cmk(coeffs[2 * t], coeffs[2 * t + 1]);
        for (int j = 0; j < term_len[t]; ++j) {
            mats.emplace_back();
            upload_op_matrix(ctx, term_ops + off, d, mats.back());
            off += 2 * (size_t)d * d;
        }
    }
    size_t mi = 0;
    for (int t = 0; t < nterms; ++t)
        for (int j = 0; j < term_len[t]; ++j) terms[t].dops.push_back(mats[mi++].c());
    std::vector<cplx> v = inner_terms(ctx, bra, ket, terms);
    for (int t = 0; t < nterms; ++t) {
        out[2 * t] = v[t].x;
        out[2 * t + 1] = v[t].y;
    }
    TN_API_END
}

// ---- DMRG -----------------------------------------------------------------------
int32_t tn_dmrg(tn_ctx* h, tn_mps* psi, const tn_mpo* H, const tn_dmrg_opts* opts, double* energy,
                tn_dmrg_stats* stats) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && H && opts && energy, "null argument");
    DmrgTerms terms;
    terms.H.push_back(H);
    terms.hc.push_back(1.0);
    dmrg_run(psi, terms, *opts, energy, stats);
    TN_API_END
}

int32_t tn_vmps(tn_ctx* h, int32_t nterms, const tn_mps* const* terms, const double* coeffs,
                const tn_vmps_opts* opts, tn_mps** out, double* cost, int32_t* sweeps) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(terms && opts && out && nterms >= 1, "null argument");
    std::vector<const tn_mps*> ts(terms, terms + nterms);
    std::vector<cplx> cs(nterms, cmk(1, 0));
    if (coeffs)
        for (int k = 0; k < nterms; ++k) cs[k] = cmk(coeffs[2 * k], coeffs[2 * k + 1]);
    for (const tn_mps* t : ts) TN_REQUIRE(t, "null term");
    const tn_mps* src = ts[0];
    tn_mps* fit = new tn_mps();
    try {
        fit->ctx = src->ctx;
        fit->N = src->N;
        fit->d = src->d;
        fit->dims = src->dims;
        fit->center = src->center;
        fit->A.resize(src->N);
        for (int i = 1; i <= src->N; ++i) {
            fit->A[i - 1] = DBuf(src->ctx, sizeof(cplx) * src->size(i));
            zcopy(src->ctx, fit->A[i - 1].c(), src->site(i), src->size(i));
        }
        movecenter(fit, 1, no_trunc());
        VmpsResult r = vmps_run(fit, ts, cs, *opts);
        if (cost) *cost = r.cost;
        if (sweeps) *sweeps = r.sweeps;
        fit->ctx->sync();
    } catch (...) {
        delete fit;
        throw;
    }
    *out = fit;
    TN_API_END
}

int32_t tn_mpo_apply(tn_ctx* h, const tn_mpo* O, const tn_mps* psi, const tn_trunc_opts* t,
                     tn_mps** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(O && psi && out, "null argument");
    tn_mps* r = new tn_mps();
    try {
        mpo_apply(O, psi, t ? to_trunc(t) : no_trunc(), r);
        r->ctx->sync();
    } catch (...) {
        delete r;
        throw;
    }
    *out = r;
    TN_API_END
}

int32_t tn_mpo_mpo_apply(tn_ctx* h, const tn_mps* A, const tn_mps* B, int32_t d,
                         const tn_trunc_opts* t, tn_mps** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(A && B && out, "null argument");
    tn_mps* r = new tn_mps();
    try {
        mpo_mpo_apply(A, B, d, t ? to_trunc(t) : no_trunc(), r);
        r->ctx->sync();
    } catch (...) {
        delete r;
        throw;
    }
    *out = r;
    TN_API_END
}

int32_t tn_mps_scale(tn_ctx* h, tn_mps* psi, const double* a) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && a, "null argument");
    mps_scale(psi, cmk(a[0], a[1]));
    psi->ctx->sync();
    TN_API_END
}

int32_t tn_mps_overlap(tn_ctx* h, const tn_mps* bra, const tn_mps* ket, double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(bra && ket && out, "null argument");
    const cplx v = mps_overlap(bra, const_cast<tn_mps*>(ket));
    out[0] = v.x;
    out[1] = v.y;
    TN_API_END
}

int32_t tn_dmrg_sum(tn_ctx* h, tn_mps* psi, int32_t nmpo, const tn_mpo* const* mpos,
                    const double* mpo_coeffs, int32_t nproj, const tn_mps* const* projs,
                    const double* proj_coeffs, const tn_dmrg_opts* opts, double* energy,
                    tn_dmrg_stats* stats) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && opts && energy && nmpo >= 0 && nproj >= 0, "null argument");
    TN_REQUIRE(nmpo == 0 || mpos, "null MPO list");
    TN_REQUIRE(nproj == 0 || projs, "null projector list");
    DmrgTerms terms;
    for (int t = 0; t < nmpo; ++t) {
        terms.H.push_back(mpos[t]);
        terms.hc.push_back(mpo_coeffs ? mpo_coeffs[t] : 1.0);
    }
    for (int p = 0; p < nproj; ++p) {
        TN_REQUIRE(projs[p] != psi, "a projector term must not be the optimised state");
        terms.P.push_back(projs[p]);
        terms.pc.push_back(proj_coeffs ? proj_coeffs[p] : 1.0);
    }
    dmrg_run(psi, terms, *opts, energy, stats);
    TN_API_END
}

// ---- gates / TEBD / QJMC -----------------------------------------------------------
int32_t tn_gates_upload(tn_ctx* h, int32_t N, int32_t d, int32_t nrows, const int32_t* row_len,
                        const int32_t* sites, const int32_t* gate_nsites,
                        const double* const* gate_ptrs, tn_gates** out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && out && row_len && (nrows == 0 || (sites && gate_nsites && gate_ptrs)), "null argument");
    Ctx* ctx = &h->c;
    tn_gates* g = new tn_gates();
    g->N = N;
    g->d = d;
    try {
        int total = 0;
        for (int r = 0; r < nrows; ++r) {
            TN_REQUIRE(row_len[r] >= 0, "negative row length");
            g->row_start.push_back(total);
            g->row_len.push_back(row_len[r]);
            total += row_len[r];
        }
        g->sites.assign(sites, sites + total);
        g->nsites.assign(gate_nsites, gate_nsites + total);
        g->M.resize(total);
        for (int r = 0; r < nrows; ++r) {
            const int s0 = g->row_start[r];
            for (int i = 0; i < row_len[r]; ++i) {
                const int gi = s0 + i;
                const int ns = g->nsites[gi];
                TN_REQUIRE(ns == 1 || ns == 2, "only one- and two-site gates are on this path");
                TN_REQUIRE(g->sites[gi] >= 1 && g->sites[gi] + ns - 1 <= N,
                           "The bond gates cannot exceed the length of the lattice.");
                if (i > 0)
                    TN_REQUIRE(g->sites[gi - 1] + g->nsites[gi - 1] - 1 < g->sites[gi],
                               "Gates in one sequence cannot be shared by sites.");
                const double* G = gate_ptrs[gi];
                if (ns == 1) {
                    upload_op_matrix(ctx, G, d, g->M[gi]);
                } else {
                    // M[I=(i1,i2), J=(o1,o2)] = G[o1,i1,o2,i2]
                    const int d2 = d * d;
                    std::vector<double> M(2 * (size_t)d2 * d2);
                    for (int o1 = 0; o1 < d; ++o1)
                        for (int i1 = 0; i1 < d; ++i1)
                            for (int o2 = 0; o2 < d; ++o2)
                                for (int i2 = 0; i2 < d; ++i2) {
                                    const size_t src = o1 + d * (i1 + d * (o2 + (size_t)d * i2));
                                    const size_t dst = (i1 + d * i2) + (size_t)d2 * (o1 + d * o2);
                                    M[2 * dst] = G[2 * src];
                                    M[2 * dst + 1] = G[2 * src + 1];
                                }
                    g->M[gi] = DBuf(ctx, sizeof(double) * M.size());
                    h2d(ctx, g->M[gi].p, M.data(), sizeof(double) * M.size());
                    ctx->sync();
                }
            }
        }
    } catch (...) {
        delete g;
        throw;
    }
    *out = g;
    TN_API_END
}

int32_t tn_gates_destroy(tn_gates* g) {
    delete g;
    return TN_OK;
}

int32_t tn_tebd_grad(tn_ctx* h, const tn_mps* psi0, int32_t ngates, const tn_gates* const* gates,
                     int32_t nsteps, const int32_t* step_gate, const tn_trunc_opts* t,
                     int32_t checkpoint_every, int32_t obs_site, const double* obs_op,
                     double broadening, double* f, double* gate_grads) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && psi0 && f && obs_op && (ngates == 0 || gates) && (nsteps == 0 || step_gate),
               "null argument");
    TN_REQUIRE(ngates >= 0 && nsteps >= 0, "negative count");
    TN_REQUIRE(psi0->ctx == &h->c, "MPS belongs to another context");
    std::vector<const tn_gates*> gl(gates, gates + ngates);
    std::vector<int> steps(step_gate, step_gate + nsteps);
    *f = tebd_grad(psi0, gl, steps, to_trunc(t), checkpoint_every, obs_site,
                   obs_op, broadening, gate_grads);
    TN_API_END
}

int32_t tn_applygates(tn_ctx* h, tn_mps* psi, const tn_gates* g, const tn_trunc_opts* t) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && g, "null argument");
    applygates(psi, g, to_trunc(t));
    psi->ctx->sync();
    TN_API_END
}

int32_t tn_tebd_steps(tn_ctx* h, tn_mps* psi, const tn_gates* g, int32_t nsteps,
                      const tn_trunc_opts* t, double* lognorm) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && g, "null argument");
    TN_REQUIRE(nsteps >= 0, "negative step count");
    tebd_steps(psi, g, nsteps, to_trunc(t), lognorm);
    psi->ctx->sync();
    TN_API_END
}

int32_t tn_tebd_steps_prec(tn_ctx* h, tn_mps* psi, const tn_gates* g, int32_t nsteps,
                           const tn_trunc_opts* t, int32_t precision, double* lognorm) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && g, "null argument");
    TN_REQUIRE(nsteps >= 0, "negative step count");
    TN_REQUIRE(precision == TN_PREC_FP64 || precision == TN_PREC_MIXED, "unknown precision");
    Ctx* ctx = psi->ctx;
    // mixed: the two-site contraction and the truncation projections run on
    // the tensor cores; the Gram matrix, eigensolver and norms stay FP64
    struct Guard {
        Ctx* c;
        bool old;
        ~Guard() { c->mixed = old; }
    } guard{ctx, ctx->mixed};
    ctx->mixed = precision == TN_PREC_MIXED;
    tebd_steps(psi, g, nsteps, to_trunc(t), lognorm);
    if (ctx->mixed) tc_check_error(ctx);
    ctx->sync();
    TN_API_END
}

int32_t tn_qjmc_rates(tn_ctx* h, tn_mps* psi, int32_t njump, const int32_t* sites,
                      const double* ops, const double* coeffs, double* rates) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && (njump == 0 || (sites && ops && coeffs && rates)), "null argument");
    Ctx* ctx = &h->c;
    const int d = psi->d;
    std::vector<DBuf> LdL(njump);
    std::vector<int> s(njump);
    std::vector<cplx> c(njump);
    for (int j = 0; j < njump; ++j) {
        TN_REQUIRE(sites[j] >= 1 && sites[j] <= psi->N, "jump site out of range");
        std::vector<double> m = ldagl(ops + 2 * (size_t)d * d * j, d);
        upload_op_matrix(ctx, m.data(), d, LdL[j]);
        s[j] = sites[j];
        c[j] = cmk(coeffs[2 * j], coeffs[2 * j + 1]);
    }
    std::vector<double> r = qjmc_rates(psi, LdL, s, c);
    for (int j = 0; j < njump; ++j) rates[j] = r[j];
    TN_API_END
}

int32_t tn_qjmc_run(tn_ctx* h, tn_mps* psi, const tn_gates* g, int32_t njump,
                    const int32_t* jump_sites, const double* jump_ops, const double* jump_coeffs,
                    int32_t nsteps, double dt, const double* draws, int64_t ndraws,
                    const tn_trunc_opts* t, int32_t save_every, int32_t nobs,
                    const int32_t* obs_sites, const double* obs_ops, double* obs_out,
                    int32_t* jumps, double* jumptimes, int32_t* njumps, int64_t* ndraws_used,
                    int32_t classical) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi && g && njumps && (ndraws == 0 || draws), "null argument");
    TN_REQUIRE(nsteps >= 0 && njump >= 1, "need at least one jump operator");
    QjmcResult r = qjmc_run(psi, g, njump, jump_sites, jump_ops, jump_coeffs, nsteps, dt, draws,
                            ndraws, to_trunc(t), save_every, nobs, obs_sites, obs_ops, obs_out,
                            *njumps, classical != 0);
    for (size_t i = 0; i < r.jumps.size(); ++i) {
        jumps[i] = r.jumps[i];
        jumptimes[i] = r.times[i];
    }
    *njumps = (int32_t)r.jumps.size();
    if (ndraws_used) *ndraws_used = r.used;
    TN_API_END
}

int32_t tn_qjmc_batch(tn_ctx* h, const tn_mps* psi0, const tn_gates* g, int32_t njump,
                      const int32_t* jump_sites, const double* jump_ops, const double* jump_coeffs,
                      int32_t nsteps, double dt, int32_t ntraj, const double* draws,
                      int64_t ndraws_per_traj, uint64_t seed, const tn_trunc_opts* t,
                      int32_t save_every, int32_t nobs, const int32_t* obs_sites,
                      const double* obs_ops, double* obs_avg, int32_t* njumps_per_traj,
                      int32_t nworkers) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi0 && g && obs_avg && jump_sites && jump_ops && jump_coeffs, "null argument");
    TN_REQUIRE(nsteps >= 0 && njump >= 1 && nobs >= 0, "bad counts");
    TN_REQUIRE(nobs == 0 || (obs_sites && obs_ops), "null observables");
    qjmc_batch(psi0, g, njump, jump_sites, jump_ops, jump_coeffs, nsteps, dt, ntraj, draws,
               ndraws_per_traj, seed, to_trunc(t), save_every, nobs, obs_sites, obs_ops, obs_avg,
               njumps_per_traj, nworkers);
    TN_API_END
}

int32_t tn_qjmc_ensemble(tn_ctx* h, const tn_mps* psi0, const tn_gates* g, int32_t njump,
                         const int32_t* jump_sites, const double* jump_ops,
                         const double* jump_coeffs, int32_t nsteps, double dt, int32_t ntraj,
                         const double* draws, int64_t ndraws_per_traj, uint64_t seed,
                         uint32_t first_traj, const tn_trunc_opts* t, int32_t save_every,
                         int32_t nobs, const int32_t* obs_sites, const double* obs_ops,
                         double* obs_avg, int32_t* njumps_per_traj, int32_t max_jumps,
                         int32_t* jumps, double* jumptimes, int32_t blocks_per_sm,
                         double* stats, int32_t classical) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(psi0 && g && obs_avg && jump_sites && jump_ops && jump_coeffs, "null argument");
    TN_REQUIRE(nobs == 0 || (obs_sites && obs_ops), "null observables");
    qjmc_ensemble(psi0, g, njump, jump_sites, jump_ops, jump_coeffs, nsteps, dt, ntraj, draws,
                  ndraws_per_traj, seed, first_traj, to_trunc(t), save_every, nobs, obs_sites,
                  obs_ops, obs_avg, njumps_per_traj, max_jumps, jumps, jumptimes, blocks_per_sm,
                  stats, classical != 0);
    TN_API_END
}

int32_t tn_philox_uniforms(uint64_t seed, uint32_t trajectory, int64_t n, double* out) {
    if (!out || n < 0) return TN_ERR_INVALID;
    philox_uniforms(seed, trajectory, n, out);
    return TN_OK;
}

// ---- unit-level entry points on host buffers ---------------------------------------
int32_t tn_heff2_apply(tn_ctx* h, int64_t cl, int64_t cr, int32_t d, int64_t wl, int64_t wm,
                       int64_t wr, const double* L, const double* W1, const double* W2,
                       const double* R, const double* theta, double* out, int32_t precision) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(L && W1 && W2 && R && theta && out, "null argument");
    TN_REQUIRE(cl >= 1 && cr >= 1 && d >= 1 && wl >= 1 && wm >= 1 && wr >= 1, "bad dimensions");
    Ctx* ctx = &h->c;
    {
        // merged two-site operator W12[(w,s1,s2),(s1',s2',w'')]
        std::vector<double> A(W1, W1 + 2 * (size_t)wl * d * d * wm), B(W2, W2 + 2 * (size_t)wm * d * d * wr);
        const int64_t nI = wl * d * d, nJ = (int64_t)d * d * wr;
        std::vector<double> M(2 * (size_t)nI * nJ, 0.0);
        for (int64_t w = 0; w < wl; ++w)
            for (int s1 = 0; s1 < d; ++s1)
                for (int s2 = 0; s2 < d; ++s2)
                    for (int p1 = 0; p1 < d; ++p1)
                        for (int p2 = 0; p2 < d; ++p2)
                            for (int64_t w2 = 0; w2 < wr; ++w2) {
                                double re = 0, im = 0;
                                for (int64_t v = 0; v < wm; ++v) {
                                    const size_t ia = w + wl * (p1 + d * (s1 + d * v));
                                    const size_t ib = v + wm * (p2 + d * (s2 + d * w2));
                                    re += A[2 * ia] * B[2 * ib] - A[2 * ia + 1] * B[2 * ib + 1];
                                    im += A[2 * ia] * B[2 * ib + 1] + A[2 * ia + 1] * B[2 * ib];
                                }
                                const size_t I = w + wl * (s1 + d * s2), J = p1 + d * (p2 + d * w2);
                                M[2 * (I + nI * J)] = re;
                                M[2 * (I + nI * J) + 1] = im;
                            }
        const size_t nL = (size_t)cl * wl * cl, nR = (size_t)cr * wr * cr, nT = (size_t)cl * d * d * cr;
        DBuf dL(ctx, 16 * nL), dR(ctx, 16 * nR), dT(ctx, 16 * nT), dO(ctx, 16 * nT), dM(ctx, 8 * M.size());
        h2d(ctx, dL.p, L, 16 * nL);
        h2d(ctx, dR.p, R, 16 * nR);
        h2d(ctx, dT.p, theta, 16 * nT);
        h2d(ctx, dM.p, M.data(), 8 * M.size());
        if (precision == TN_PREC_MIXED)
            mixed_unit_heff2(ctx, dL.c(), dM.c(), dR.c(), cl, cr, d, wl, wr, dT.c(), dO.c());
        else
            heff2_fp64(ctx, dL.c(), dM.c(), dR.c(), cl, cr, d, wl, wr, dT.c(), dO.c());
        d2h(ctx, out, dO.p, 16 * nT);
        ctx->sync();
    }
    TN_API_END
}

int32_t tn_heff2_apply_noalloc(tn_ctx* h, int64_t cl, int64_t cr, int32_t d, int64_t wl,
                               int64_t wm, int64_t wr, const double* L, const double* W1,
                               const double* W2, const double* R, const double* theta,
                               double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(h && L && W1 && W2 && R && theta && out, "null argument");
    heff2_noalloc(&h->c, cl, cr, d, wl, wm, wr, reinterpret_cast<const cplx*>(L),
                  reinterpret_cast<const cplx*>(W1), reinterpret_cast<const cplx*>(W2),
                  reinterpret_cast<const cplx*>(R), reinterpret_cast<const cplx*>(theta),
                  reinterpret_cast<cplx*>(out));
    TN_API_END
}

static void host_w_mats(const double* W, int64_t wl, int d, int64_t wr, std::vector<double>& Ml,
                        std::vector<double>& Mr) {
    const size_t n = (size_t)wl * d * d * wr;
    Ml.assign(2 * n, 0.0);
    Mr.assign(2 * n, 0.0);
    const int64_t nIl = wl * d, nIr = d * wr;
    for (int64_t w = 0; w < wl; ++w)
        for (int sp = 0; sp < d; ++sp)
            for (int s = 0; s < d; ++s)
                for (int64_t w2 = 0; w2 < wr; ++w2) {
                    const size_t src = w + wl * (sp + d * (s + d * w2));
                    const size_t il = (w + wl * s) + nIl * (sp + d * w2);
                    const size_t ir = (sp + d * w2) + nIr * (w + wl * s);
                    Ml[2 * il] = W[2 * src];
                    Ml[2 * il + 1] = W[2 * src + 1];
                    Mr[2 * ir] = W[2 * src];
                    Mr[2 * ir + 1] = W[2 * src + 1];
                }
}

int32_t tn_env_left(tn_ctx* h, int64_t cl, int64_t cr, int32_t d, int64_t wl, int64_t wr,
                    const double* L, const double* A, const double* W, double* out, int32_t precision) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(L && A && W && out, "null argument");
    TN_REQUIRE(precision == TN_PREC_FP64 || precision == TN_PREC_MIXED, "unknown precision");
    Ctx* ctx = &h->c;
    tn_mpo H1;
    H1.ctx = ctx;
    H1.N = 1;
    H1.d = d;
    H1.w = {wl, wr};
    std::vector<double> Ml, Mr;
    host_w_mats(W, wl, d, wr, Ml, Mr);
    H1.Ml.resize(1);
    H1.Ml[0] = DBuf(ctx, 8 * Ml.size());
    h2d(ctx, H1.Ml[0].p, Ml.data(), 8 * Ml.size());
    const size_t nL = (size_t)cl * wl * cl, nA = (size_t)cl * d * cr, nO = (size_t)cr * wr * cr;
    DBuf dL(ctx, 16 * nL), dA(ctx, 16 * nA), dO(ctx, 16 * nO);
    h2d(ctx, dL.p, L, 16 * nL);
    h2d(ctx, dA.p, A, 16 * nA);
    if (precision == TN_PREC_MIXED) {
        mixed_env_left(ctx, dL.c(), cl, wl, cl, dA.c(), cr, H1.Ml[0].c(), d, wr, dA.c(), cr, dO.c());
        tc_check_error(ctx);
    } else {
        env_left(ctx, dL.c(), cl, wl, cl, dA.c(), cr, &H1, 1, dA.c(), cr, d, dO.c());
    }
    d2h(ctx, out, dO.p, 16 * nO);
    ctx->sync();
    TN_API_END
}

int32_t tn_env_right(tn_ctx* h, int64_t cl, int64_t cr, int32_t d, int64_t wl, int64_t wr,
                     const double* R, const double* A, const double* W, double* out, int32_t precision) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(R && A && W && out, "null argument");
    TN_REQUIRE(precision == TN_PREC_FP64 || precision == TN_PREC_MIXED, "unknown precision");
    Ctx* ctx = &h->c;
    tn_mpo H1;
    H1.ctx = ctx;
    H1.N = 1;
    H1.d = d;
    H1.w = {wl, wr};
    std::vector<double> Ml, Mr;
    host_w_mats(W, wl, d, wr, Ml, Mr);
    H1.Mr.resize(1);
    H1.Mr[0] = DBuf(ctx, 8 * Mr.size());
    h2d(ctx, H1.Mr[0].p, Mr.data(), 8 * Mr.size());
    const size_t nR = (size_t)cr * wr * cr, nA = (size_t)cl * d * cr, nO = (size_t)cl * wl * cl;
    DBuf dR(ctx, 16 * nR), dA(ctx, 16 * nA), dO(ctx, 16 * nO);
    h2d(ctx, dR.p, R, 16 * nR);
    h2d(ctx, dA.p, A, 16 * nA);
    if (precision == TN_PREC_MIXED) {
        mixed_env_right(ctx, dR.c(), cr, wr, cr, dA.c(), cl, H1.Mr[0].c(), d, wl, dA.c(), cl, dO.c());
        tc_check_error(ctx);
    } else {
        env_right(ctx, dR.c(), cr, wr, cr, dA.c(), cl, &H1, 1, dA.c(), cl, d, dO.c());
    }
    d2h(ctx, out, dO.p, 16 * nO);
    ctx->sync();
    TN_API_END
}

int32_t tn_gate2_apply(tn_ctx* h, int64_t cl, int64_t cm, int64_t cr, int32_t d, const double* A1,
                       const double* A2, const double* G, double* out) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(A1 && A2 && G && out, "null argument");
    Ctx* ctx = &h->c;
    const int d2 = d * d;
    std::vector<double> M(2 * (size_t)d2 * d2);
    for (int o1 = 0; o1 < d; ++o1)
        for (int i1 = 0; i1 < d; ++i1)
            for (int o2 = 0; o2 < d; ++o2)
                for (int i2 = 0; i2 < d; ++i2) {
                    const size_t src = o1 + d * (i1 + d * (o2 + (size_t)d * i2));
                    const size_t dst = (i1 + d * i2) + (size_t)d2 * (o1 + d * o2);
                    M[2 * dst] = G[2 * src];
                    M[2 * dst + 1] = G[2 * src + 1];
                }
    const size_t n1 = (size_t)cl * d * cm, n2 = (size_t)cm * d * cr, nT = (size_t)cl * d2 * cr;
    DBuf d1(ctx, 16 * n1), dd2(ctx, 16 * n2), dT(ctx, 16 * nT), dO(ctx, 16 * nT), dM(ctx, 8 * M.size());
    h2d(ctx, d1.p, A1, 16 * n1);
    h2d(ctx, dd2.p, A2, 16 * n2);
    h2d(ctx, dM.p, M.data(), 8 * M.size());
    const cplx one = cmk(1, 0), zero = cmk(0, 0);
    zgemm(ctx, OP_N, OP_N, cl * d, d * cr, cm, one, d1.c(), cl * d, 0, dd2.c(), cm, 0, zero, dT.c(), cl * d, 0);
    small_apply(ctx, dT.c(), dO.c(), dM.c(), d2, d2, cl, cr, cl, cl * d2, cl, cl * d2);
    d2h(ctx, out, dO.p, 16 * nT);
    ctx->sync();
    TN_API_END
}

int32_t tn_gemm(tn_ctx* h, int64_t m, int64_t n, int64_t k, const double* A, int32_t conj_a,
                const double* B, double* Cout, int32_t precision) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(A && B && Cout, "null argument");
    TN_REQUIRE(m >= 1 && n >= 1 && k >= 1, "bad dimensions");
    Ctx* ctx = &h->c;
    DBuf dA(ctx, 16 * (size_t)m * k), dB(ctx, 16 * (size_t)k * n), dC(ctx, 16 * (size_t)m * n);
    h2d(ctx, dA.p, A, 16 * (size_t)m * k);
    h2d(ctx, dB.p, B, 16 * (size_t)k * n);
    if (precision == TN_PREC_MIXED) {
        mixed_gemm(ctx, m, n, k, dA.c(), conj_a != 0, dB.c(), dC.c());
    } else {
        const cplx one = cmk(1, 0), zero = cmk(0, 0);
        zgemm(ctx, conj_a ? OP_C : OP_N, OP_N, m, n, k, one, dA.c(), conj_a ? k : m, 0, dB.c(), k, 0,
              zero, dC.c(), m, 0);
    }
    d2h(ctx, Cout, dC.p, 16 * (size_t)m * n);
    ctx->sync();
    TN_API_END
}

int32_t tn_truncate(tn_ctx* h, int64_t m, int64_t n, const double* theta, const tn_trunc_opts* t,
                    int32_t direction, double* X, double* Y, double* S, int64_t* k) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(theta && X && Y && S && k, "null argument");
    TN_REQUIRE(m >= 1 && n >= 1, "bad dimensions");
    Ctx* ctx = &h->c;
    Trunc tr = to_trunc(t);
    DBuf dT(ctx, 16 * (size_t)m * n), dX, dY;
    h2d(ctx, dT.p, theta, 16 * (size_t)m * n);
    std::vector<double> Sv;
    SplitResult r = trunc_split(ctx, dT.c(), m, n, tr.cutoff, tr.maxdim, tr.mindim, direction == 0,
                                dX, dY, &Sv);
    TN_REQUIRE(r.k <= *k, "output capacity too small");
    d2h(ctx, X, dX.p, 16 * (size_t)m * r.k);
    d2h(ctx, Y, dY.p, 16 * (size_t)r.k * n);
    ctx->sync();
    memcpy(S, Sv.data(), sizeof(double) * r.k);
    *k = r.k;
    TN_API_END
}

int32_t tn_eigh_top(tn_ctx* h, int64_t n, const double* G, int64_t want, double* lam,
                    double* V) {
    TN_API_BEGIN(h ? &h->c : nullptr)
    TN_REQUIRE(G && lam && V, "null argument");
    TN_REQUIRE(n >= 1 && want >= 1 && want <= n, "bad dimensions");
    Ctx* ctx = &h->c;
    DBuf dG(ctx, 16 * (size_t)n * n), dV(ctx, 16 * (size_t)n * want), dL(ctx, 8 * (size_t)want);
    h2d(ctx, dG.p, G, 16 * (size_t)n * n);
    eig_top(ctx, dG.c(), n, want, dL.d(), dV.c());
    std::vector<double> asc(want);
    d2h(ctx, asc.data(), dL.p, 8 * (size_t)want);
    d2h(ctx, V, dV.p, 16 * (size_t)n * want);
    int herr = 0;
    d2h(ctx, &herr, ctx->d_bar + 2, sizeof(int));
    ctx->sync();
    if (herr) {
        TN_CHECK_CUDA(cudaMemsetAsync(ctx->d_bar + 2, 0, sizeof(unsigned), ctx->stream));
        throw Error(TN_ERR_TIMEOUT, "eigensolver: a bounded grid barrier ran out");
    }
    for (int64_t g = 0; g < want; ++g) lam[g] = asc[want - 1 - g];
    TN_API_END
}

}  // extern "C"
