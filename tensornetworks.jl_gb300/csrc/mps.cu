// Gauge moves, two-site splits, environment blocks, the two-site effective
// Hamiltonian product and expectation values on device-resident MPS.
#include "mps.cuh"
#include "mixed.cuh"

namespace tn {

static const cplx ONE = {1.0, 0.0};
static const cplx ZERO = {0.0, 0.0};

// ---- gauge moves (gmps.jl:60-112) -----------------------------------------
// moveright!: SVD with the right bond as columns, M[(Dl,s),Dr]; the isometry
// stays, S*Vt is absorbed into the next site.
void moveright(tn_mps* psi, int idx, const Trunc& t) {
    if (!(0 < idx && idx < psi->N)) return;
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(idx), Dr = psi->dr(idx), Dr2 = psi->dr(idx + 1);
    DBuf X, Y;
    SplitResult r = trunc_split(ctx, psi->site(idx), Dl * d, Dr, t.cutoff, t.maxdim, t.mindim,
                                true, X, Y, nullptr);
    const int64_t k = r.k;
    DBuf next(ctx, sizeof(cplx) * k * d * Dr2);
    zgemm(ctx, OP_N, OP_N, k, d * Dr2, Dr, ONE, Y.c(), k, 0, psi->site(idx + 1), Dr, 0, ZERO,
          next.c(), k, 0);
    psi->A[idx - 1] = std::move(X);
    psi->A[idx] = std::move(next);
    psi->dims[idx] = k;
}

// moveleft!: SVD with the left bond as columns; the co-isometry stays, U*S is
// absorbed into the previous site.
void moveleft(tn_mps* psi, int idx, const Trunc& t) {
    if (!(1 < idx && idx <= psi->N)) return;
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(idx), Dr = psi->dr(idx), Dl0 = psi->dl(idx - 1);
    DBuf X, Y;
    SplitResult r = trunc_split(ctx, psi->site(idx), Dl, d * Dr, t.cutoff, t.maxdim, t.mindim,
                                false, X, Y, nullptr);
    const int64_t k = r.k;
    DBuf prev(ctx, sizeof(cplx) * Dl0 * d * k);
    zgemm(ctx, OP_N, OP_N, Dl0 * d, k, Dl, ONE, psi->site(idx - 1), Dl0 * d, 0, X.c(), Dl, 0,
          ZERO, prev.c(), Dl0 * d, 0);
    psi->A[idx - 1] = std::move(Y);
    psi->A[idx - 2] = std::move(prev);
    psi->dims[idx - 1] = k;
}

void movecenter(tn_mps* psi, int idx, const Trunc& t) {
    const int N = psi->N;
    TN_REQUIRE(idx >= 1 && idx <= N, "The index is out of range.");
    if (psi->center == 0) {
        for (int i = 1; i <= idx - 1; ++i) moveright(psi, i, t);
        for (int i = 1; i <= N - idx; ++i) moveleft(psi, N + 1 - i, t);
    } else if (idx > psi->center) {
        for (int i = psi->center; i <= idx - 1; ++i) moveright(psi, i, t);
    } else if (idx < psi->center) {
        const int c = psi->center;
        for (int i = 1; i <= c - idx; ++i) moveleft(psi, c + 1 - i, t);
    }
    psi->center = idx;
}

cplx mps_norm(tn_mps* psi) {
    if (psi->center == 0) movecenter(psi, 1, no_trunc());
    const int c = psi->center;
    const double n2 = znorm2(psi->ctx, psi->site(c), psi->size(c));
    return cmk(sqrt(n2), 0.0);
}

void mps_normalize(tn_mps* psi) {
    if (psi->center == 0) movecenter(psi, 1, no_trunc());
    const cplx n = mps_norm(psi);
    const int c = psi->center;
    zscale(psi->ctx, psi->site(c), psi->size(c), cmk(1.0 / n.x, 0.0));
}

void two_site(tn_mps* psi, int site, DBuf& buf) {
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(site), Dm = psi->dr(site), Dr = psi->dr(site + 1);
    const size_t need = sizeof(cplx) * Dl * d * d * Dr;
    if (buf.bytes < need) buf = DBuf(ctx, need);
    if (ctx->mixed && Dm >= 64) {
        // mixed-precision sweep: the two-site tensor only seeds the Lanczos
        // solve, so the 3xTF32 tensor-core product is enough
        mixed_gemm(ctx, Dl * d, d * Dr, Dm, psi->site(site), false, psi->site(site + 1), buf.c());
        return;
    }
    zgemm(ctx, OP_N, OP_N, Dl * d, d * Dr, Dm, ONE, psi->site(site), Dl * d, 0,
          psi->site(site + 1), Dm, 0, ZERO, buf.c(), Dl * d, 0);
}

SplitResult replacesites2(tn_mps* psi, const cplx* theta, int site, bool direction, bool normalize,
                          const Trunc& t, std::vector<double>* S) {
    const int d = psi->d;
    const int64_t Dl = psi->dl(site), Dr = psi->dr(site + 1);
    DBuf X, Y;
    SplitResult r = trunc_split(psi->ctx, theta, Dl * d, d * Dr, t.cutoff, t.maxdim, t.mindim,
                                !direction, X, Y, S);
    psi->A[site - 1] = std::move(X);
    psi->A[site] = std::move(Y);
    psi->dims[site] = r.k;
    psi->center = direction ? site : site + 1;
    if (normalize) mps_normalize(psi);
    return r;
}

void replacesite1(tn_mps* psi, DBuf&& A, int site, bool direction, bool normalize) {
    psi->A[site - 1] = std::move(A);
    const int nxt = site + 1 - 2 * (direction ? 1 : 0);
    if (0 < nxt && nxt <= psi->N) movecenter(psi, nxt, no_trunc());
    if (normalize) mps_normalize(psi);
}

std::vector<double> singular_values(tn_mps* psi, int site) {
    movecenter(psi, site, no_trunc());
    Ctx* ctx = psi->ctx;
    const int64_t m = psi->dl(site) * psi->d, n = psi->dr(site);
    DBuf X, Y;
    std::vector<double> S;
    trunc_split(ctx, psi->site(site), m, n, 0.0, 0, 1, m <= n, X, Y, &S);
    return S;
}

// ---- environment blocks (projmps.jl:50-95) ---------------------------------
void env_left(Ctx* ctx, const cplx* L, int64_t ca, int64_t wl, int64_t cb, const cplx* A,
              int64_t ca2, const tn_mpo* H, int site, const cplx* B, int64_t cb2, int d, cplx* out) {
    if (!H) {
        cplx* X = ctx->s_t1.c(ctx, (size_t)ca * d * cb2);
        zgemm(ctx, OP_N, OP_N, ca, d * cb2, cb, ONE, L, ca, 0, B, cb, 0, ZERO, X, ca, 0);
        zgemm(ctx, OP_C, OP_N, ca2, cb2, ca * d, ONE, A, ca * d, 0, X, ca * d, 0, ZERO, out, ca2, 0);
        return;
    }
    const int64_t wr = H->w[site];
    cplx* X = ctx->s_t1.c(ctx, (size_t)ca * wl * d * cb2);
    cplx* Y = ctx->s_t2.c(ctx, (size_t)ca * d * wr * cb2);
    zgemm(ctx, OP_N, OP_N, ca * wl, d * cb2, cb, ONE, L, ca * wl, 0, B, cb, 0, ZERO, X, ca * wl, 0);
    small_apply(ctx, X, Y, H->Ml[site - 1].c(), (int)(wl * d), (int)(d * wr), ca, cb2, ca,
                ca * wl * d, ca, ca * d * wr);
    zgemm(ctx, OP_C, OP_N, ca2, wr * cb2, ca * d, ONE, A, ca * d, 0, Y, ca * d, 0, ZERO, out, ca2, 0);
}

void env_right(Ctx* ctx, const cplx* R, int64_t ca2, int64_t wr, int64_t cb2, const cplx* A,
               int64_t ca, const tn_mpo* H, int site, const cplx* B, int64_t cb, int d, cplx* out) {
    if (!H) {
        cplx* Z = ctx->s_t1.c(ctx, (size_t)ca * d * cb2);
        zgemm(ctx, OP_R, OP_N, ca * d, cb2, ca2, ONE, A, ca * d, 0, R, ca2, 0, ZERO, Z, ca * d, 0);
        zgemm(ctx, OP_N, OP_T, ca, cb, d * cb2, ONE, Z, ca, 0, B, cb, 0, ZERO, out, ca, 0);
        return;
    }
    const int64_t wl = H->w[site - 1];
    cplx* Z = ctx->s_t1.c(ctx, (size_t)ca * d * wr * cb2);
    cplx* Z2 = ctx->s_t2.c(ctx, (size_t)ca * wl * d * cb2);
    zgemm(ctx, OP_R, OP_N, ca * d, wr * cb2, ca2, ONE, A, ca * d, 0, R, ca2, 0, ZERO, Z, ca * d, 0);
    small_apply(ctx, Z, Z2, H->Mr[site - 1].c(), (int)(d * wr), (int)(wl * d), ca, cb2, ca,
                ca * d * wr, ca, ca * wl * d);
    zgemm(ctx, OP_N, OP_T, ca * wl, cb, d * cb2, ONE, Z2, ca * wl, 0, B, cb, 0, ZERO, out, ca * wl, 0);
}

// out[a,s1',s2',c'] = sum L[a,w,b] W12[(w,s1,s2),(s1',s2',w'')] th[b,s1,s2,c] R[c',w'',c]
// as L*theta (GEMM), the W12 leg (small_apply), then *R^T (GEMM).
void heff2_fp64(Ctx* ctx, const cplx* L, const cplx* W12, const cplx* R, int64_t cl, int64_t cr,
                int d, int64_t wl, int64_t wr, const cplx* theta, cplx* out) {
    const int64_t d2 = (int64_t)d * d;
    cplx* T1 = ctx->s_t1.c(ctx, (size_t)cl * wl * d2 * cr);
    cplx* T2 = ctx->s_t2.c(ctx, (size_t)cl * d2 * wr * cr);
    zgemm(ctx, OP_N, OP_N, cl * wl, d2 * cr, cl, ONE, L, cl * wl, 0, theta, cl, 0, ZERO, T1,
          cl * wl, 0);
    small_apply(ctx, T1, T2, W12, (int)(wl * d2), (int)(d2 * wr), cl, cr, cl, cl * wl * d2, cl,
                cl * d2 * wr);
    zgemm(ctx, OP_N, OP_T, cl * d2, cr, wr * cr, ONE, T2, cl * d2, 0, R, cr, 0, ZERO, out, cl * d2, 0);
}

// ---- operators on the physical leg ------------------------------------------
void upload_op_matrix(Ctx* ctx, const double* op, int d, DBuf& out) {
    // small_apply form M[I=i, J=o] = op[o, i]
    std::vector<cplx> M((size_t)d * d);
    for (int o = 0; o < d; ++o)
        for (int i = 0; i < d; ++i) {
            const double* e = op + 2 * (o + (size_t)d * i);
            M[i + (size_t)d * o] = cmk(e[0], e[1]);
        }
    out = DBuf(ctx, sizeof(cplx) * M.size());
    TN_CHECK_CUDA(cudaMemcpyAsync(out.p, M.data(), sizeof(cplx) * M.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
    ctx->sync();
}

void apply_site_op(tn_mps* psi, int site, const cplx* M) {
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(site), Dr = psi->dr(site);
    DBuf out(ctx, sizeof(cplx) * Dl * d * Dr);
    small_apply(ctx, psi->site(site), out.c(), M, d, d, Dl, Dr, Dl, Dl * d, Dl, Dl * d);
    psi->A[site - 1] = std::move(out);
}

// ---- expectation values (mps.jl:87-134) ------------------------------------
std::vector<cplx> inner_terms(Ctx* ctx, const tn_mps* bra, const tn_mps* ket,
                              const std::vector<Term>& terms) {
    const int N = ket->N, d = ket->d;
    TN_REQUIRE(bra->N == N && bra->d == d, "GMPS must share the same properties.");
    // right overlap blocks: R[i] is the block from site i (i = N+1 is the edge)
    std::vector<DBuf> R(N + 2);
    std::vector<int64_t> ra(N + 2, 1), rb(N + 2, 1);
    R[N + 1] = DBuf(ctx, sizeof(cplx));
    zfill(ctx, R[N + 1].c(), 1, ONE);
    for (int i = N; i >= 2; --i) {
        ra[i] = bra->dl(i);
        rb[i] = ket->dl(i);
        R[i] = DBuf(ctx, sizeof(cplx) * ra[i] * rb[i]);
        env_right(ctx, R[i + 1].c(), ra[i + 1], 1, rb[i + 1], bra->site(i), ra[i], nullptr, i,
                  ket->site(i), rb[i], d, R[i].c());
    }
    DBuf out(ctx, sizeof(cplx) * std::max<size_t>(terms.size(), 1));
    DBuf L(ctx, sizeof(cplx)), Lt1, Lt2, B;
    zfill(ctx, L.c(), 1, ONE);
    int64_t la = 1, lb = 1;
    std::vector<std::vector<size_t>> by_site(N + 1);
    for (size_t t = 0; t < terms.size(); ++t) {
        TN_REQUIRE(terms[t].first >= 1 && terms[t].first + terms[t].len - 1 <= N && terms[t].len >= 1,
                   "term sites out of range");
        by_site[terms[t].first].push_back(t);
    }
    for (int site = 1; site <= N; ++site) {
        for (size_t t : by_site[site]) {
            const Term& T = terms[t];
            int64_t ta = la, tb = lb;
            const cplx* cur = L.c();
            for (int j = 0; j < T.len; ++j) {
                const int s = site + j;
                const int64_t Dl = ket->dl(s), Dr = ket->dr(s);
                const size_t nb = sizeof(cplx) * Dl * d * Dr;
                if (B.bytes < nb) B = DBuf(ctx, nb);
                small_apply(ctx, ket->site(s), B.c(), T.dops[j], d, d, Dl, Dr, Dl, Dl * d, Dl, Dl * d);
                DBuf& dst = (j % 2 == 0) ? Lt1 : Lt2;
                const size_t nl = sizeof(cplx) * bra->dr(s) * Dr;
                if (dst.bytes < nl) dst = DBuf(ctx, nl);
                env_left(ctx, cur, ta, 1, tb, bra->site(s), bra->dr(s), nullptr, s, B.c(), Dr, d,
                         dst.c());
                cur = dst.c();
                ta = bra->dr(s);
                tb = Dr;
            }
            const int rs = site + T.len;
            bilinear_dot(ctx, cur, R[rs].c(), ta * tb, out.c() + t);
        }
        DBuf Ln(ctx, sizeof(cplx) * bra->dr(site) * ket->dr(site));
        env_left(ctx, L.c(), la, 1, lb, bra->site(site), bra->dr(site), nullptr, site,
                 ket->site(site), ket->dr(site), d, Ln.c());
        L = std::move(Ln);
        la = bra->dr(site);
        lb = ket->dr(site);
    }
    std::vector<cplx> res(terms.size());
    if (!terms.empty()) {
        TN_CHECK_CUDA(cudaMemcpyAsync(res.data(), out.p, sizeof(cplx) * res.size(),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    }
    ctx->sync();
    for (size_t t = 0; t < terms.size(); ++t) res[t] = cmul(terms[t].coeff, res[t]);
    return res;
}

}  // namespace tn
