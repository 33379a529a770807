// Variational MPS fitting and MPO-MPS products on the device
// (src/algorithms/mps/vmps.jl:1-105, src/structures/mps/mpo.jl:105-146,
// src/structures/mps/abstractmps.jl:100-107).
//
// vmps fits an MPS to a weighted sum of MPSs by two-site sweeps: at each
// bond the target's local two-site tensor is the sum over the terms of the
// term's two sites contracted with the overlap environments <term|fit>
// (OvlCache::local_ket), which replaces the fit's two sites through the
// truncated split.  The MPO-MPS product contracts each site with its MPO
// tensor (bond dimensions multiply), left-canonicalises without truncation
// and then moves the centre to site 1 with the caller's truncation.
#include <cmath>
#include <cstdio>
#include <memory>

#include "ovl.cuh"

namespace tn {

namespace {

// phi[(w + wl*a), o, (w2 + wr*b)] = sum_s M[w, o, s, w2] A[a, s, b]
// (the index grouping of MPOMPSProduct, mpo.jl:130-136)
__global__ void mpo_mps_site_kernel(const cplx* __restrict__ M, const cplx* __restrict__ A,
                                    int64_t wl, int64_t wr, int64_t al, int64_t ar, int d,
                                    cplx* __restrict__ out) {
    const int64_t L = wl * al, R = wr * ar, total = L * d * R;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = e % L, o = (e / L) % d, r = e / (L * d);
        const int64_t w = l % wl, a = l / wl, w2 = r % wr, b = r / wr;
        cplx acc = cmk(0, 0);
        for (int s = 0; s < d; ++s)
            acc = cfma(M[w + wl * (o + d * (s + d * w2))], A[a + al * (s + (int64_t)d * b)], acc);
        out[e] = acc;
    }
}

// Fused MPO sites (physical index p = o + d i, the column-major grouping of
// [Dl, o, i, Dr]): out[(a + Da b), (o + d i), (a2 + Da2 b2)] =
// sum_k A[a, (o + d k), a2] B[b, (k + d i), b2] (MPOMPOProduct, mpo.jl:151-158)
__global__ void mpo_mpo_site_kernel(const cplx* __restrict__ A, const cplx* __restrict__ B,
                                    int64_t da, int64_t da2, int64_t db, int64_t db2, int d,
                                    cplx* __restrict__ out) {
    const int64_t d2 = (int64_t)d * d, L = da * db, R = da2 * db2, total = L * d2 * R;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = e % L, p = (e / L) % d2, r = e / (L * d2);
        const int64_t a = l % da, b = l / da, a2 = r % da2, b2 = r / da2;
        const int64_t o = p % d, i = p / d;
        cplx acc = cmk(0, 0);
        for (int k = 0; k < d; ++k)
            acc = cfma(A[a + da * ((o + d * k) + d2 * a2)], B[b + db * ((k + d * i) + d2 * b2)], acc);
        out[e] = acc;
    }
}

}  // namespace

// MPOMPOProduct(O1, O2; trunc) (mpo.jl:147-167) on fused MPOs: MPSs of
// physical dimension d^2 whose index is (o + d i).  The product's sites are
// built, left-canonicalised without truncation, then the centre moves to
// site 1 with the caller's truncation, as for the MPO-MPS product.
void mpo_mpo_apply(const tn_mps* A, const tn_mps* B, int d, const Trunc& t, tn_mps* out) {
    TN_REQUIRE(A->N == B->N && A->d == B->d, "GMPS must share the same physical dims.");
    TN_REQUIRE(d >= 1 && (int64_t)d * d == A->d, "fused MPOs have physical dimension d^2");
    Ctx* ctx = A->ctx;
    const int N = A->N, d2 = d * d;
    out->ctx = ctx;
    out->N = N;
    out->d = d2;
    out->dims.assign(N + 1, 1);
    out->A.clear();
    out->A.resize(N);
    for (int i = 0; i <= N; ++i) out->dims[i] = A->dims[i] * B->dims[i];
    for (int i = 1; i <= N; ++i) {
        const int64_t da = A->dl(i), da2 = A->dr(i), db = B->dl(i), db2 = B->dr(i);
        const int64_t total = da * db * d2 * da2 * db2;
        out->A[i - 1] = DBuf(ctx, sizeof(cplx) * total);
        const int64_t g = std::min<int64_t>((total + 255) / 256, (int64_t)ctx->sm_count * 8);
        mpo_mpo_site_kernel<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, ctx->stream>>>(
            A->site(i), B->site(i), da, da2, db, db2, d, out->A[i - 1].c());
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    }
    out->center = 0;
    movecenter(out, N, no_trunc());
    movecenter(out, 1, t);
}

// psi <- a psi: the centre tensor (site 1 without a centre) is scaled
// (*(psi, a), abstractmps.jl:100-107).
void mps_scale(tn_mps* psi, cplx a) {
    const int site = psi->center != 0 ? psi->center : 1;
    zscale(psi->ctx, psi->site(site), psi->size(site), a);
}

// <bra|ket> by one left-to-right sweep of overlap blocks.
cplx mps_overlap(const tn_mps* bra, tn_mps* ket) {
    TN_REQUIRE(bra->N == ket->N && bra->d == ket->d, "GMPS must share the same properties.");
    OvlCache oc(bra, ket);
    oc.movecenter(ket->N);
    return oc.calculate();
}

// MPOMPSProduct(O, psi; trunc) (mpo.jl:125-146): a new MPS.
void mpo_apply(const tn_mpo* O, const tn_mps* psi, const Trunc& t, tn_mps* out) {
    TN_REQUIRE(O->N == psi->N && O->d == psi->d, "GMPS must share the same physical dims.");
    Ctx* ctx = psi->ctx;
    const int N = psi->N, d = psi->d;
    out->ctx = ctx;
    out->N = N;
    out->d = d;
    out->dims.assign(N + 1, 1);
    out->A.clear();
    out->A.resize(N);
    for (int i = 0; i <= N; ++i) out->dims[i] = O->w[i] * psi->dims[i];
    for (int i = 1; i <= N; ++i) {
        const int64_t wl = O->w[i - 1], wr = O->w[i], al = psi->dl(i), ar = psi->dr(i);
        const int64_t total = wl * al * d * wr * ar;
        out->A[i - 1] = DBuf(ctx, sizeof(cplx) * total);
        const int64_t g = std::min<int64_t>((total + 255) / 256, (int64_t)ctx->sm_count * 8);
        mpo_mps_site_kernel<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, ctx->stream>>>(
            O->W[i - 1].c(), psi->site(i), wl, wr, al, ar, d, out->A[i - 1].c());
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    }
    // left-canonical without truncation, then the centre to site 1 with it
    // (the product's centre is unset, so movecenter!(phi, 1) sweeps from N)
    out->center = 0;
    movecenter(out, N, no_trunc());
    movecenter(out, 1, t);
}

// vmps(psis...; kwargs) (vmps.jl:1-105) with complex weights: fit = the
// first term's state, centred at 1, fitted to sum_k c_k |term_k>.
struct VmpsResult {
    double cost;
    int sweeps;
};
VmpsResult vmps_run(tn_mps* fit, const std::vector<const tn_mps*>& terms,
                    const std::vector<cplx>& coeffs, const tn_vmps_opts& o) {
    TN_REQUIRE(!terms.empty() && coeffs.size() == terms.size(), "vmps needs at least one term");
    TN_REQUIRE(o.nsites == 2, "only two-site fitting (nsites=2) is on this path");
    Ctx* ctx = fit->ctx;
    const int N = fit->N, d = fit->d;
    for (const tn_mps* t : terms)
        TN_REQUIRE(t->N == N && t->d == d, "GMPS must share the same properties.");
    TN_REQUIRE(N >= 2, "vmps needs at least two sites");
    std::vector<std::unique_ptr<OvlCache>> ovl;
    for (const tn_mps* t : terms) {
        ovl.emplace_back(new OvlCache(t, fit));
        ovl.back()->movecenter(1);
    }
    const Trunc tr{o.cutoff, o.maxdim, o.mindim};
    // cost = |fit|^2 - 2 |sum_k <c_k term_k|fit>| (calculatecost, vmps.jl:18-25)
    auto cost_of = [&]() {
        const cplx nrm = mps_norm(fit);
        cplx c = cmk(0, 0);
        for (size_t k = 0; k < ovl.size(); ++k) {
            const cplx v = ovl[k]->calculate();
            c = cadd(c, cmul(cconj(coeffs[k]), v));
        }
        const double n2 = nrm.x * nrm.x + nrm.y * nrm.y;
        return n2 - 2.0 * std::hypot(c.x, c.y);
    };
    auto diff = [](double x, double y) {
        return std::fabs(x) < 1e-10 ? std::fabs(x - y) : std::fabs((x - y) / x);
    };
    double lastcost = cost_of();
    int D = fit->maxbonddim(), lastD = D;
    bool direction = false, converged = false;
    int convsweeps = 0, sweeps = 0;
    double cost = lastcost;
    DBuf vec, K;
    while (!converged) {
        for (int j = 1; j <= N - 1; ++j) {
            const int site = direction ? N + 1 - j : j;
            const int site1 = direction ? site - 1 : site;
            for (auto& e : ovl) e->movecenter(site);
            const int64_t n = fit->dl(site1) * d * d * fit->dr(site1 + 1);
            if (vec.bytes < sizeof(cplx) * n) vec = DBuf(ctx, sizeof(cplx) * n);
            zfill(ctx, vec.c(), n, cmk(0, 0));
            for (size_t k = 0; k < ovl.size(); ++k) {
                ovl[k]->local_ket(site1, K);
                zaxpy(ctx, vec.c(), K.c(), n, coeffs[k]);
            }
            replacesites2(fit, vec.c(), site1, direction, false, tr);
        }
        for (auto& e : ovl) e->movecenter(direction ? 1 : N);
        direction = !direction;
        ++sweeps;
        D = fit->maxbonddim();
        cost = cost_of();
        if (sweeps >= o.minsweeps) {
            // the reference's reset `convergedsweeps == 0` (vmps.jl:67) is a
            // comparison, so converged sweeps accumulate; mirrored here
            if (diff(cost, lastcost) < o.tol && lastD == D) ++convsweeps;
            if ((double)convsweeps >= o.numconverges) converged = true;
            if (sweeps >= o.maxsweeps && o.maxsweeps != 0) converged = true;
        }
        lastcost = cost;
        lastD = D;
        if (o.verbose) printf("Sweep=%d, energy=%.12f, maxbonddim=%d \n", sweeps, cost, D);
    }
    return VmpsResult{cost, sweeps};
}

}  // namespace tn
