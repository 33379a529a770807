// Context, stream-ordered memory, and the truncated two-factor split that
// replaces LAPACK gesdd in svd(x, idx; cutoff, maxdim, mindim)
// (src/tensors.jl:168-227).
//
// The split forms the Gram matrix on the side of the isometric factor, so the
// isometry is an eigenvector matrix (orthonormal to working precision) and
// the other factor is a projection; no division by small singular values is
// needed.  The Gram product runs on our GEMM, the Hermitian eigenproblem on
// cuSOLVER's zheevd (FP64), and the keep rule on the warp-shuffle kernel.
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
    TN_CHECK_SOLVER(cusolverDnCreate(&c.solver));
    TN_CHECK_SOLVER(cusolverDnSetStream(c.solver, c.stream));
    TN_CHECK_CUDA(cudaMalloc(&c.d_info, sizeof(int)));
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
                      &c.s_mixf};
    for (Scratch* s : all) s->buf.reset();
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.solver) cusolverDnDestroy(c.solver);
    if (c.d_info) cudaFree(c.d_info);
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
int64_t heevd(Ctx* ctx, cplx* G, int64_t n, double* dlam, int64_t top, bool check) {
    auto* A = reinterpret_cast<cuDoubleComplex*>(G);
    const bool partial = top > 0 && top < n;
    int lwork = 0, meig = (int)n;
    // top eigenpairs only: the tridiagonal reduction is shared, the
    // back-transformation covers top columns instead of n
    const int il = (int)(n - top + 1), iu = (int)n;
    if (partial)
        TN_CHECK_SOLVER(cusolverDnZheevdx_bufferSize(
            ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER,
            (int)n, A, (int)n, 0.0, 0.0, il, iu, &meig, dlam, &lwork));
    else
        TN_CHECK_SOLVER(cusolverDnZheevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR,
                                                    CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n,
                                                    dlam, &lwork));
    cuDoubleComplex* work = static_cast<cuDoubleComplex*>(
        ctx->s_work.get(ctx, sizeof(cuDoubleComplex) * (size_t)std::max(lwork, 1)));
    ProfScope ps(ctx, 2, 0.0, 16.0 * n * n);
    if (partial)
        TN_CHECK_SOLVER(cusolverDnZheevdx(ctx->solver, CUSOLVER_EIG_MODE_VECTOR,
                                          CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER, (int)n, A,
                                          (int)n, 0.0, 0.0, il, iu, &meig, dlam, work, lwork,
                                          ctx->d_info));
    else
        TN_CHECK_SOLVER(cusolverDnZheevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR,
                                         CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, dlam, work,
                                         lwork, ctx->d_info));
    if (check) {
        int info = 0;
        TN_CHECK_CUDA(cudaMemcpyAsync(&info, ctx->d_info, sizeof(int), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        ctx->sync();
        if (info != 0)
            throw Error(TN_ERR_NUMERIC, std::string(partial ? "zheevdx" : "zheevd") +
                                            " failed, info = " + std::to_string(info));
    }
    if (partial && meig != (int)top)
        throw Error(TN_ERR_NUMERIC, "zheevdx returned " + std::to_string(meig) + " of " +
                                        std::to_string(top) + " eigenpairs");
    return partial ? top : n;
}

// ---- truncated split -------------------------------------------------------
SplitResult trunc_split(Ctx* ctx, const cplx* theta, int64_t m, int64_t n, double cutoff,
                        int64_t maxdim, int64_t mindim, bool left_iso, DBuf& X, DBuf& Y,
                        std::vector<double>* S) {
    TN_REQUIRE(m > 0 && n > 0, "trunc_split: empty matrix");
    const int64_t sz = std::min(m, n);
    const int64_t g = left_iso ? m : n;
    TN_REQUIRE(g <= 46340, "trunc_split: Gram matrix too large for 32-bit solver indexing");
    cplx* G = ctx->s_gram.c(ctx, (size_t)g * g);
    double* lam = ctx->s_eigval.d(ctx, (size_t)g + sz + 1);
    double* dS = lam + g;
    const cplx one = cmk(1, 0), zero = cmk(0, 0);
    if (left_iso)  // G = theta theta^H
        zgemm(ctx, OP_N, OP_C, m, m, n, one, theta, m, 0, theta, m, 0, zero, G, m, 0, 1, true);
    else  // G = theta^H theta
        zgemm(ctx, OP_C, OP_N, n, n, m, one, theta, m, 0, theta, m, 0, zero, G, n, 0, 1, true);
    // eigenpairs the keep rule can select: max(maxdim, mindim), at most sz
    const int64_t maxd = (maxdim <= 0 || maxdim > sz) ? sz : maxdim;
    const int64_t want = std::min(sz, std::max(maxd, mindim));
    const bool partial = g >= 32 && want < g;
    double* dtotal = nullptr;
    if (partial) {  // the trace gives the weight below the computed eigenvalues
        dtotal = lam + g + sz;
        gram_trace(ctx, G, g, dtotal);
    }
    // the solver status is read back with the keep-rule result (one synchronisation)
    const int64_t ne = heevd(ctx, G, g, lam, partial ? want : 0, false);
    KeepResult kr = keep_rule(ctx, lam, ne, std::min(sz, ne), cutoff, maxdim, mindim, dS, dtotal,
                              ctx->d_info);
    const int64_t k = kr.k;
    TN_REQUIRE(k <= ne, "trunc_split: keep rule selected more vectors than computed");
    // tensor-core projection in mixed mode, for products large enough to pay
    // for the operand conversion
    const bool use_tc = ctx->mixed && (double)m * n * k >= (double)(1 << 21);
    if (left_iso) {
        X = DBuf(ctx, sizeof(cplx) * m * k);
        Y = DBuf(ctx, sizeof(cplx) * k * n);
        take_top_eigvecs(ctx, G, m, k, X.c(), ne);
        if (use_tc)  // the isometry stays exact; the projection on the tensor cores
            mixed_gemm(ctx, k, n, m, X.c(), true, theta, Y.c());
        else
            zgemm(ctx, OP_C, OP_N, k, n, m, one, X.c(), m, 0, theta, m, 0, zero, Y.c(), k, 0);
    } else {
        DBuf V(ctx, sizeof(cplx) * n * k);
        take_top_eigvecs(ctx, G, n, k, V.c(), ne);
        X = DBuf(ctx, sizeof(cplx) * m * k);
        Y = DBuf(ctx, sizeof(cplx) * k * n);
        if (use_tc)
            mixed_gemm(ctx, m, k, n, theta, false, V.c(), X.c());
        else
            zgemm(ctx, OP_N, OP_N, m, k, n, one, theta, m, 0, V.c(), n, 0, zero, X.c(), m, 0);
        conj_transpose(ctx, V.c(), n, k, Y.c());  // Y = V^H (k x n)
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
