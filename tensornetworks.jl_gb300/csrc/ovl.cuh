// Overlap environments <phi|psi> with a movable centre, shared by the DMRG
// projector terms and the variational MPS fit (projmps.jl:16-95 with the
// objects [phi, psi]).
#pragma once

#include "mps.cuh"

namespace tn {

struct OvlCache {
    Ctx* ctx;
    const tn_mps* phi;
    tn_mps* psi;
    int N;
    std::vector<DBuf> blk;  // blk[i]: left block through i (i < centre) or right block from i
    std::vector<int64_t> a, b;
    DBuf edge;
    int center = 0;
    OvlCache(const tn_mps* f, tn_mps* p) : ctx(p->ctx), phi(f), psi(p), N(p->N) {
        blk.resize(N + 2);
        a.assign(N + 2, 1);
        b.assign(N + 2, 1);
        edge = DBuf(ctx, sizeof(cplx));
        zfill(ctx, edge.c(), 1, cmk(1, 0));
    }
    const cplx* block(int i, int64_t& ca, int64_t& cb) const {
        if (i < 1 || i > N) {
            ca = cb = 1;
            return edge.c();
        }
        ca = a[i];
        cb = b[i];
        return blk[i].c();
    }
    void buildleft(int i) {
        int64_t la, lb;
        const cplx* L = block(i - 1, la, lb);
        const int64_t na = phi->dr(i), nb = psi->dr(i);
        DBuf out(ctx, sizeof(cplx) * na * nb);
        env_left(ctx, L, la, 1, lb, phi->site(i), na, nullptr, i, psi->site(i), nb, psi->d, out.c());
        blk[i] = std::move(out);
        a[i] = na;
        b[i] = nb;
    }
    void buildright(int i) {
        int64_t ra, rb;
        const cplx* R = block(i + 1, ra, rb);
        const int64_t na = phi->dl(i), nb = psi->dl(i);
        DBuf out(ctx, sizeof(cplx) * na * nb);
        env_right(ctx, R, ra, 1, rb, phi->site(i), na, nullptr, i, psi->site(i), nb, psi->d, out.c());
        blk[i] = std::move(out);
        a[i] = na;
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
    // <phi|psi> contracted at the centre (calculate, projmps.jl:192-216)
    cplx calculate() {
        const int c = center;
        int64_t la, lb, ra, rb;
        const cplx* L = block(c - 1, la, lb);
        const cplx* R = block(c + 1, ra, rb);
        const int64_t na = phi->dr(c), nb = psi->dr(c);
        DBuf out(ctx, sizeof(cplx) * na * nb);
        env_left(ctx, L, la, 1, lb, phi->site(c), na, nullptr, c, psi->site(c), nb, psi->d, out.c());
        cplx* d = ctx->s_coef.c(ctx, 4);
        bilinear_dot(ctx, out.c(), R, na * nb, d);
        cplx hres;
        TN_CHECK_CUDA(cudaMemcpyAsync(&hres, d, sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
        ctx->sync();
        return hres;
    }
    // The projected two-site ket of phi in psi's local basis at bond
    // (site1, site1+1): K[b, s1, s2, c] = sum conj(L[x, b]) phi1[x, s1, y]
    // phi2[y, s2, z] conj(R[z, c]), i.e. conj of project() (projmps.jl:156-189).
    void local_ket(int site1, DBuf& K) {
        const int d = psi->d;
        int64_t la, lb, ra, rb;
        const cplx* L = block(site1 - 1, la, lb);
        const cplx* R = block(site1 + 2, ra, rb);
        const int64_t x = phi->dl(site1), y = phi->dr(site1), z = phi->dr(site1 + 1);
        DBuf Phi(ctx, sizeof(cplx) * x * d * d * z), T(ctx, sizeof(cplx) * lb * d * d * z);
        zgemm(ctx, OP_N, OP_N, x * d, d * z, y, cmk(1, 0), phi->site(site1), x * d, 0, phi->site(site1 + 1),
              y, 0, cmk(0, 0), Phi.c(), x * d, 0);
        zgemm(ctx, OP_C, OP_N, lb, d * d * z, la, cmk(1, 0), L, la, 0, Phi.c(), x, 0, cmk(0, 0), T.c(), lb, 0);
        const size_t nk = sizeof(cplx) * lb * d * d * rb;
        if (K.bytes < nk) K = DBuf(ctx, nk);
        zgemm(ctx, OP_N, OP_R, lb * d * d, rb, z, cmk(1, 0), T.c(), lb * d * d, 0, R, ra, 0, cmk(0, 0), K.c(),
              lb * d * d, 0);
    }
};

}  // namespace tn
