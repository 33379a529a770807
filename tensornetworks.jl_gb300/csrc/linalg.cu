// Context, stream-ordered memory, and the truncated two-factor split that
// replaces LAPACK gesdd in svd(x, idx; cutoff, maxdim, mindim)
// (src/tensors.jl:168-227).
//
// The split forms the Gram matrix on the side of the isometric factor, so the
// isometry is an eigenvector matrix (orthonormal to working precision) and
// the other factor is a projection; no division by small singular values is
// needed.  The Gram product runs on our GEMM, the Hermitian eigenproblem on
// this library's FP64 eigensolver (eig.cu), and the keep rule on the
// warp-shuffle kernel.
#include "common.cuh"
#include "mixed.cuh"

#include <cstring>

namespace tn {

// ---- memory ----------------------------------------------------------------
DBuf::DBuf(Ctx* c, size_t b) : ctx(c), bytes(b) {
    if (b == 0) return;
    cudaError_t e = cudaMallocAsync(&p, b, c->stream);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        (void)cudaGetLastError();
        throw Error(TN_ERR_OOM, "device allocation of " + std::to_string(b) + " bytes failed");
    }
}
DBuf::~DBuf() { reset(); }
DBuf& DBuf::operator=(DBuf&& o) noexcept {
    if (this != &o) {
        reset();
        p = o.p;
        bytes = o.bytes;
        ctx = o.ctx;
        o.p = nullptr;
        o.bytes = 0;
    }
    return *this;
}
void DBuf::reset() {
    if (p && ctx) cudaFreeAsync(p, ctx->stream);
    p = nullptr;
    bytes = 0;
}

void* Scratch::get(Ctx* ctx, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (buf.bytes < bytes) {
        buf.reset();
        buf = DBuf(ctx, bytes + bytes / 4);
    }
    return buf.p;
}

double* Ctx::pinned(size_t n) {
    if (h_pinned_n < n) {
        if (h_pinned) cudaFreeHost(h_pinned);
        h_pinned = nullptr;
        TN_CHECK_CUDA(cudaMallocHost(&h_pinned, n * sizeof(double)));
        h_pinned_n = n;
    }
    return h_pinned;
}

void ctx_init(Ctx& c, int device) {
    TN_CHECK_CUDA(cudaSetDevice(device));
    c.device = device;
    TN_CHECK_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    TN_CHECK_CUDA(cudaDeviceGetDefaultMemPool(&c.pool, device));
    uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
    TN_CHECK_CUDA(cudaMemPoolSetAttribute(c.pool, cudaMemPoolAttrReleaseThreshold, &thr));
    TN_CHECK_CUDA(cudaMalloc(&c.d_info, sizeof(int)));
    TN_CHECK_CUDA(cudaMalloc(&c.d_bar, 4 * sizeof(unsigned)));
    TN_CHECK_CUDA(cudaMemset(c.d_bar, 0, 4 * sizeof(unsigned)));
    TN_CHECK_CUDA(cudaMalloc(&c.d_err, sizeof(int)));
    TN_CHECK_CUDA(cudaMemset(c.d_err, 0, sizeof(int)));
    TN_CHECK_CUDA(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device));
}

void ctx_release(Ctx& c) {
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    // scratch buffers release through the stream before it goes away
    Scratch* all[] = {&c.s_gram, &c.s_eigval, &c.s_work, &c.s_x, &c.s_y, &c.s_t1, &c.s_t2,
                      &c.s_dot, &c.s_coef, &c.s_mixa, &c.s_mixb, &c.s_mixc, &c.s_mixd, &c.s_mixe,
                      &c.s_mixf, &c.s_eig, &c.s_splitk};
    for (Scratch* s : all) s->buf.reset();
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.d_info) cudaFree(c.d_info);
    if (c.d_bar) cudaFree(c.d_bar);
    if (c.d_err) cudaFree(c.d_err);
    if (c.h_pinned) cudaFreeHost(c.h_pinned);
    for (auto& r : c.prof_pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : c.ev_pool) cudaEventDestroy(e);
    if (c.stream) cudaStreamDestroy(c.stream);
    c = Ctx{};
}

cudaEvent_t Ctx::ev_get() {
    if (!ev_pool.empty()) {
        cudaEvent_t e = ev_pool.back();
        ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    TN_CHECK_CUDA(cudaEventCreate(&e));
    return e;
}

void Ctx::prof_flush() {
    if (prof_pending.empty()) return;
    TN_CHECK_CUDA(cudaEventSynchronize(prof_pending.back().b));
    for (ProfRec& r : prof_pending) {
        float ms = 0.f;
        TN_CHECK_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        ProfClass& c = prof[r.cls];
        c.launches += 1;
        c.ms += ms;
        c.flops += r.flops;
        c.bytes += r.bytes;
        ev_pool.push_back(r.a);
        ev_pool.push_back(r.b);
    }
    prof_pending.clear();
}

// ---- eigen-decomposition ---------------------------------------------------
void heev_full(Ctx* ctx, cplx* G, int64_t n, double* dlam) {
    DBuf V(ctx, sizeof(cplx) * n * n);
    eig_top(ctx, G, n, n, dlam, V.c());
    take_top_eigvecs(ctx, V.c(), n, n, G);  // descending -> ascending columns
    int h = 0;
    TN_CHECK_CUDA(cudaMemcpyAsync(&h, ctx->d_bar + 2, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    ctx->sync();
    if (h) {
        TN_CHECK_CUDA(cudaMemsetAsync(ctx->d_bar + 2, 0, sizeof(unsigned), ctx->stream));
        throw Error(TN_ERR_TIMEOUT, "eigensolver: a bounded grid barrier ran out");
    }
}

// ---- truncated split -------------------------------------------------------
SplitResult trunc_split(Ctx* ctx, const cplx* theta, int64_t m, int64_t n, double cutoff,
                        int64_t maxdim, int64_t mindim, bool left_iso, DBuf& X, DBuf& Y,
                        std::vector<double>* S) {
    TN_REQUIRE(m > 0 && n > 0, "trunc_split: empty matrix");
    const int64_t sz = std::min(m, n);
    const int64_t g = left_iso ? m : n;
    TN_REQUIRE(g <= 4096, "trunc_split: Gram matrix order above 4096 (bond dimension x d)");
    cplx* G = ctx->s_gram.c(ctx, (size_t)g * g);
    const cplx one = cmk(1, 0), zero = cmk(0, 0);
    if (left_iso)  // G = theta theta^H
        zgemm(ctx, OP_N, OP_C, m, m, n, one, theta, m, 0, theta, m, 0, zero, G, m, 0, 1, true);
    else  // G = theta^H theta
        zgemm(ctx, OP_C, OP_N, n, n, m, one, theta, m, 0, theta, m, 0, zero, G, n, 0, 1, true);
    // eigenpairs the keep rule can select: max(maxdim, mindim), at most sz
    const int64_t maxd = (maxdim <= 0 || maxdim > sz) ? sz : maxdim;
    const int64_t want = std::min(sz, std::max(maxd, mindim));
    double* lam = ctx->s_eigval.d(ctx, (size_t)want + sz + 2);
    double* dS = lam + want;
    double* dtotal = lam + want + sz;  // the trace gives the weight below the computed values
    gram_trace(ctx, G, g, dtotal);
    cplx* V = ctx->s_x.c(ctx, (size_t)g * want);  // top eigenvectors, descending
    eig_top(ctx, G, g, want, lam, V);
    // the eigensolver's barrier status is read back with the keep-rule result
    KeepResult kr = keep_rule(ctx, lam, want, want, cutoff, maxdim, mindim, dS, dtotal,
                              reinterpret_cast<const int*>(ctx->d_bar + 2));
    const int64_t k = kr.k;
    TN_REQUIRE(k <= want, "trunc_split: keep rule selected more vectors than computed");
    // tensor-core projection in mixed mode, for products large enough to pay
    // for the operand conversion
    const bool use_tc = ctx->mixed && (double)m * n * k >= (double)(1 << 21);
    if (left_iso) {
        X = DBuf(ctx, sizeof(cplx) * m * k);
        Y = DBuf(ctx, sizeof(cplx) * k * n);
        zcopy(ctx, X.c(), V, m * k);
        if (use_tc)  // the isometry stays exact; the projection on the tensor cores
            mixed_gemm(ctx, k, n, m, X.c(), true, theta, Y.c());
        else
            zgemm(ctx, OP_C, OP_N, k, n, m, one, X.c(), m, 0, theta, m, 0, zero, Y.c(), k, 0);
    } else {
        X = DBuf(ctx, sizeof(cplx) * m * k);
        Y = DBuf(ctx, sizeof(cplx) * k * n);
        if (use_tc)
            mixed_gemm(ctx, m, k, n, theta, false, V, X.c());
        else
            zgemm(ctx, OP_N, OP_N, m, k, n, one, theta, m, 0, V, n, 0, zero, X.c(), m, 0);
        conj_transpose(ctx, V, n, k, Y.c());  // Y = V^H (k x n)
    }
    if (S) {
        // Singular values as norms of the projected factor (U^H theta rows or
        // theta V columns): accurate to eps * sigma_max even where the Gram
        // eigenvalue sits at the sqrt(eps) noise floor.
        if (left_iso)
            row_norms(ctx, Y.c(), k, n, dS);
        else
            col_norms(ctx, X.c(), m, k, dS);
        S->resize(k);
        TN_CHECK_CUDA(cudaMemcpyAsync(S->data(), dS, sizeof(double) * k, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        ctx->sync();
    }
    return SplitResult{k, kr.discarded, kr.total};
}

}  // namespace tn
