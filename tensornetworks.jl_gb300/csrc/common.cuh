// Internal declarations shared by the libtngpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tngpu.h"

typedef double2 cplx;

namespace tn {

// Error carrying a TN_ERR_* status; caught at the C ABI boundary.
struct Error : public std::runtime_error {
    int32_t code;
    Error(int32_t c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define TN_CHECK_CUDA(expr)                                                          \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess)                                                       \
            throw ::tn::Error(_e == cudaErrorMemoryAllocation ? TN_ERR_OOM : TN_ERR_CUDA, \
                              std::string(#expr) + ": " + cudaGetErrorString(_e));   \
    } while (0)

#define TN_REQUIRE(cond, msg)                                                        \
    do {                                                                             \
        if (!(cond)) throw ::tn::Error(TN_ERR_INVALID, msg);                         \
    } while (0)

// Stream-ordered device buffer drawn from the context's memory pool.
struct Ctx;
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    Ctx* ctx = nullptr;
    DBuf() = default;
    DBuf(Ctx* c, size_t b);
    ~DBuf();
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept { *this = std::move(o); }
    DBuf& operator=(DBuf&& o) noexcept;
    void reset();
    template <class T> T* as() const { return static_cast<T*>(p); }
    cplx* c() const { return static_cast<cplx*>(p); }
    double* d() const { return static_cast<double*>(p); }
};

// Growable scratch buffer (keeps its allocation between uses).
struct Scratch {
    DBuf buf;
    void* get(Ctx* ctx, size_t bytes);
    cplx* c(Ctx* ctx, size_t n) { return static_cast<cplx*>(get(ctx, n * sizeof(cplx))); }
    double* d(Ctx* ctx, size_t n) { return static_cast<double*>(get(ctx, n * sizeof(double))); }
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    std::string err;
    int64_t launches = 0;
    int sm_count = 0;
    // reusable scratch for the hot path
    Scratch s_gram, s_eigval, s_work, s_x, s_y, s_t1, s_t2, s_dot, s_coef, s_mixa, s_mixb, s_mixc,
        s_mixd, s_mixe, s_mixf, s_eig, s_splitk;
    int* d_info = nullptr;
    // grid-barrier words of the eigensolver's cooperative kernels: arrival
    // count, generation, and an error word set when a bounded wait ran out
    unsigned* d_bar = nullptr;
    int* d_err = nullptr;  // set by device code when a bounded wait runs out
    // mixed precision on: environment updates and truncation projections run
    // on the tensor cores (set for the duration of a mixed-precision sweep)
    bool mixed = false;
    // split-K FP64 GEMMs draw partial buffers from the pool; callers that must
    // not allocate turn them off
    bool splitk = true;
    double* h_pinned = nullptr;  // small pinned staging area
    size_t h_pinned_n = 0;
    // kernel profiler: CUDA events around launches, per class
    struct ProfClass {
        int64_t launches = 0;
        double ms = 0, flops = 0, bytes = 0;
    };
    struct ProfRec {
        int cls;
        cudaEvent_t a, b;
        double flops, bytes;
    };
    bool prof_on = false;
    ProfClass prof[TN_PROF_CLASSES];
    // host wall seconds per DMRG phase while profiling (synchronised at each
    // phase end): 0 environment update, 1 two-site tensor and operand
    // preparation, 2 Lanczos, 3 truncation and normalisation
    double phase_s[4] = {0, 0, 0, 0};
    std::vector<ProfRec> prof_pending;
    std::vector<cudaEvent_t> ev_pool;
    cudaEvent_t ev_get();
    void prof_flush();  // resolves pending event pairs (synchronises)
    void sync() { TN_CHECK_CUDA(cudaStreamSynchronize(stream)); }
    void count() {
        ++launches;
        if (prof_on) ++prof[TN_PROF_CLASSES - 1].launches;  // class 7 counts every launch
    }
    double* pinned(size_t n);
};

// Records a CUDA event pair around the launches in its scope when the
// context's profiler is on.
struct ProfScope {
    Ctx* ctx;
    int cls;
    double flops, bytes;
    cudaEvent_t a = nullptr;
    ProfScope(Ctx* c, int k, double f, double b) : ctx(c), cls(k), flops(f), bytes(b) {
        if (ctx->prof_on) {
            a = ctx->ev_get();
            cudaEventRecord(a, ctx->stream);
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = ctx->ev_get();
            cudaEventRecord(b, ctx->stream);
            ctx->prof_pending.push_back({cls, a, b, flops, bytes});
            if (ctx->prof_pending.size() > 4096) ctx->prof_flush();
        }
    }
};

// stream, pool settings and device flags of a context
void ctx_init(Ctx& c, int device);
void ctx_release(Ctx& c);

// ---- small complex helpers ----------------------------------------------
__host__ __device__ inline cplx cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline cplx cadd(cplx a, cplx b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ inline cplx csub(cplx a, cplx b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ inline cplx cmul(cplx a, cplx b) {
    return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline cplx cconj(cplx a) { return cmk(a.x, -a.y); }
__host__ __device__ inline cplx cfma(cplx a, cplx b, cplx c) {  // a*b + c
    return cmk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}

// hi + lo += v in float-float arithmetic: hi takes the rounded sum, lo the
// exact rounding error (Knuth's TwoSum; additions only, so no contraction).
// Summing FP32 partials this way keeps ~46 bits without FP64 instructions,
// which GB300 issues at a small fraction of the FP32 rate.
__host__ __device__ inline void ff_add(float& hi, float& lo, float v) {
    const float t = hi + v;
    const float bp = t - hi;
    const float e = (hi - (t - bp)) + (v - bp);
    hi = t;
    lo += e;
}

// ---- kernels (kernels_fp64.cu) -----------------------------------------
enum Op { OP_N = 0, OP_T = 1, OP_C = 2, OP_R = 3 };  // R: conjugate without transpose

// C[m x n] = alpha * op(A) * op(B) + beta * C, column-major, batched by count.
void zgemm(Ctx* ctx, Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplx alpha, const cplx* A,
           int64_t lda, int64_t strideA, const cplx* B, int64_t ldb, int64_t strideB, cplx beta,
           cplx* C, int64_t ldc, int64_t strideC, int64_t batch = 1, bool lower_only = false);

// out[a + lda_o*J + ldc_o*c] (=|+=) sum_I in[a + lda_i*I + ldc_i*c] * M[I + nI*J]
void small_apply(Ctx* ctx, const cplx* in, cplx* out, const cplx* M, int nI, int nJ, int64_t na,
                 int64_t nc, int64_t lda_i, int64_t ldc_i, int64_t lda_o, int64_t ldc_o,
                 bool accumulate = false);

// out[j] = <v_j, w> for K vectors; result left in device memory dout (K cplx).
void multi_dot(Ctx* ctx, const cplx* const* dV, int K, const cplx* w, int64_t n, cplx* dout);
// w += sum_j coef[j] * v_j, coef on the device (K cplx); sign applied to coefs.
void multi_axpy(Ctx* ctx, cplx* w, const cplx* const* dV, const cplx* dcoef, int K, int64_t n,
                double sign);
void zscale(Ctx* ctx, cplx* x, int64_t n, cplx a);
void zaxpy(Ctx* ctx, cplx* y, const cplx* x, int64_t n, cplx a);  // y += a x
void zscale_dev(Ctx* ctx, cplx* x, int64_t n, const double* dnorm, int invert);  // x *= 1/norm
void zcopy(Ctx* ctx, cplx* dst, const cplx* src, int64_t n);
void zfill(Ctx* ctx, cplx* dst, int64_t n, cplx v);
void bilinear_dot(Ctx* ctx, const cplx* x, const cplx* y, int64_t n, cplx* dout);  // sum x*y
double znorm2(Ctx* ctx, const cplx* x, int64_t n);  // ||x||^2, synchronous
// take k eigenvectors, largest first: dst[:, j] = G[:, ncols-1-j] (ncols < 0:
// ncols = n, a full ascending eigenvector matrix)
void take_top_eigvecs(Ctx* ctx, const cplx* G, int64_t n, int64_t k, cplx* dst,
                      int64_t ncols = -1);
// *dout = sum of the real diagonal of the n x n matrix G (device)
void gram_trace(Ctx* ctx, const cplx* G, int64_t n, double* dout);
// scale columns: X[:, j] *= s[j] (s real, device)
// dst (c x r) = src(r x c)^H, tiled through shared memory for coalescing
void conj_transpose(Ctx* ctx, const cplx* src, int64_t r, int64_t c, cplx* dst);
void scale_cols(Ctx* ctx, cplx* X, int64_t m, int64_t k, const double* s, int invert);
// column norms of X (m x k) / row norms of Y (k x n), warp-shuffle reductions
void col_norms(Ctx* ctx, const cplx* X, int64_t m, int64_t k, double* out);
void row_norms(Ctx* ctx, const cplx* Y, int64_t k, int64_t n, double* out);
void scale_rows(Ctx* ctx, cplx* X, int64_t k, int64_t n, const double* s, int invert);

// Keep rule of tensors.jl:200-215 on ascending eigenvalues lam[0..n) of a Gram
// matrix whose top sz values are the squared singular values.  Writes
// (k, total, discarded) to host.  Also writes kept singular values (descending)
// into dS when non-null.  With dtotal (device, the Gram trace) the n values
// are only the top of the spectrum: the weight below them is the trace minus
// their sum.
struct KeepResult { int64_t k; double total; double discarded; };
// dinfo (device, optional): an eigensolver status read back in the same
// synchronisation; nonzero raises TN_ERR_NUMERIC.
KeepResult keep_rule(Ctx* ctx, const double* dlam, int64_t n, int64_t sz, double cutoff,
                     int64_t maxdim, int64_t mindim, double* dS, const double* dtotal = nullptr,
                     const int* dinfo = nullptr);

// ---- linear algebra (linalg.cu) ----------------------------------------
// Truncated split theta (m x n) ~= X (m x k) Y (k x n).  left_iso: X is an
// isometry (sweeping right); else Y is a co-isometry (sweeping left).  X, Y
// are allocated into the given DBufs.  Singular values (descending) go to S
// (host vector) when non-null.
struct SplitResult { int64_t k; double discarded; double total; };
SplitResult trunc_split(Ctx* ctx, const cplx* theta, int64_t m, int64_t n, double cutoff,
                        int64_t maxdim, int64_t mindim, bool left_iso, DBuf& X, DBuf& Y,
                        std::vector<double>* S);
// Top `want` eigenpairs of the Hermitian n x n matrix G (lower triangle read,
// G destroyed), hand-written FP64 kernels (eig.cu): lam_asc[want-1-g] is the
// g-th largest eigenvalue and X[:, g] (n x want) its eigenvector.  No host
// synchronisation; a timed-out grid barrier leaves ctx->d_bar[2] nonzero.
void eig_top(Ctx* ctx, cplx* G, int64_t n, int64_t want, double* lam_asc, cplx* X);
// Full eigen-decomposition, ascending: eigenvalues in dlam[0..n), eigenvectors
// overwrite G (column j belongs to dlam[j]); synchronises and checks.
void heev_full(Ctx* ctx, cplx* G, int64_t n, double* dlam);


}  // namespace tn
