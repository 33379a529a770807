// FP64 kernels of the plain (parity) path: complex GEMM, the small-operator
// contraction used for MPO/gate legs, Lanczos vector reductions (warp
// shuffles) and the truncation keep rule.
//
// GB300 executes FP64 on the SIMT pipes at a small fraction of its tensor
// rate, so these kernels are compute-bound at modest tile sizes: a 64x64
// complex tile per 256-thread block with a 4x4 complex register tile per
// thread keeps the DFMA pipe busy while shared-memory traffic stays far below
// its bandwidth.
#include "common.cuh"

namespace tn {

namespace {

constexpr int GB_M = 64, GB_N = 64, GB_K = 16;

template <int OPA, int OPB>
__global__ void __launch_bounds__(256) zgemm_kernel(int64_t M, int64_t N, int64_t K, cplx alpha,
                                                    const cplx* __restrict__ A, int64_t lda,
                                                    int64_t sA, const cplx* __restrict__ B,
                                                    int64_t ldb, int64_t sB, cplx beta,
                                                    cplx* __restrict__ C, int64_t ldc, int64_t sC,
                                                    int lower, int64_t kc) {
    __shared__ cplx As[GB_K][GB_M + 1];
    __shared__ cplx Bs[GB_K][GB_N + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    // kc > 0: split K; blockIdx.z is the chunk and C the chunk's partial
    // (M x N, ld M); otherwise blockIdx.z is the batch index
    const int64_t bz = kc > 0 ? 0 : blockIdx.z;
    const int64_t k_lo = kc > 0 ? (int64_t)blockIdx.z * kc : 0;
    const int64_t k_hi = kc > 0 ? min(K, k_lo + kc) : K;
    A += bz * sA;
    B += bz * sB;
    C += kc > 0 ? (int64_t)blockIdx.z * M * N : bz * sC;
    const int64_t m0 = (int64_t)blockIdx.x * GB_M, n0 = (int64_t)blockIdx.y * GB_N;
    // lower: only the lower triangle is wanted (a Hermitian Gram matrix read
    // by the eigensolver, which reads the lower triangle); tiles strictly
    // above the diagonal skip
    if (lower && n0 >= m0 + GB_M) return;
    cplx acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cmk(0.0, 0.0);

    for (int64_t k0 = k_lo; k0 < k_hi; k0 += GB_K) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int mm, kk;
            if (OPA == OP_N || OPA == OP_R) {
                mm = tid & 63;
                kk = (tid >> 6) + 4 * i;
            } else {
                kk = tid & 15;
                mm = (tid >> 4) + 16 * i;
            }
            const int64_t gm = m0 + mm, gk = k0 + kk;
            cplx v = cmk(0.0, 0.0);
            if (gm < M && gk < k_hi) {
                v = (OPA == OP_N || OPA == OP_R) ? A[gm + gk * lda] : A[gk + gm * lda];
                if (OPA == OP_C || OPA == OP_R) v.y = -v.y;
            }
            As[kk][mm] = v;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int kk, nn;
            if (OPB == OP_N || OPB == OP_R) {
                kk = tid & 15;
                nn = (tid >> 4) + 16 * i;
            } else {
                nn = tid & 63;
                kk = (tid >> 6) + 4 * i;
            }
            const int64_t gn = n0 + nn, gk = k0 + kk;
            cplx v = cmk(0.0, 0.0);
            if (gn < N && gk < k_hi) {
                v = (OPB == OP_N || OPB == OP_R) ? B[gk + gn * ldb] : B[gn + gk * ldb];
                if (OPB == OP_C || OPB == OP_R) v.y = -v.y;
            }
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            cplx a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t gn = n0 + ty + 16 * j;
        if (gn >= N) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t gm = m0 + tx + 16 * i;
            if (gm >= M) continue;
            cplx v = cmul(alpha, acc[i][j]);
            if (use_beta) v = cfma(beta, C[gm + gn * ldc], v);
            C[gm + gn * ldc] = v;
        }
    }
}

// Thin or small products (min(m, n) < 48): one thread per output element, a
// plain dot product over k.  The 64x64 tile kernel would spend GB300's scarce
// FP64 issue slots on zero padding there (a 10 x 10 product costs a full tile).
template <int OPA, int OPB>
__global__ void __launch_bounds__(64) zgemm_small_kernel(int64_t M, int64_t N, int64_t K, cplx alpha,
                                                         const cplx* __restrict__ A, int64_t lda,
                                                         int64_t sA, const cplx* __restrict__ B,
                                                         int64_t ldb, int64_t sB, cplx beta,
                                                         cplx* __restrict__ C, int64_t ldc,
                                                         int64_t sC, int64_t batch, int lower) {
    const int64_t total = M * N * batch;
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % M, j = (idx / M) % N, b = idx / (M * N);
        if (lower && i < j) continue;  // only the lower triangle is wanted
        const cplx* a = A + b * sA;
        const cplx* bb = B + b * sB;
        cplx acc = cmk(0.0, 0.0);
        for (int64_t l = 0; l < K; ++l) {
            cplx x = (OPA == OP_N || OPA == OP_R) ? a[i + l * lda] : a[l + i * lda];
            if (OPA == OP_C || OPA == OP_R) x.y = -x.y;
            cplx y = (OPB == OP_N || OPB == OP_R) ? bb[l + j * ldb] : bb[j + l * ldb];
            if (OPB == OP_C || OPB == OP_R) y.y = -y.y;
            acc = cfma(x, y, acc);
        }
        cplx* c = C + b * sC + i + j * ldc;
        cplx v = cmul(alpha, acc);
        if (use_beta) v = cfma(beta, *c, v);
        *c = v;
    }
}

// C = alpha sum_z P[z] + beta C over the split-K partials in chunk order
// (deterministic); lower: entries above the diagonal are left alone.
__global__ void splitk_reduce_kernel(const cplx* __restrict__ P, int64_t M, int64_t N, int S,
                                     cplx alpha, cplx beta, cplx* __restrict__ C, int64_t ldc,
                                     int lower) {
    const int64_t total = M * N;
    const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % M, j = e / M;
        if (lower && i < j) continue;
        cplx acc = cmk(0, 0);
        for (int z = 0; z < S; ++z) acc = cadd(acc, P[e + (int64_t)z * total]);
        cplx v = cmul(alpha, acc);
        if (use_beta) v = cfma(beta, C[i + j * ldc], v);
        C[i + j * ldc] = v;
    }
}

template <int OPA>
void zgemm_small_dispatch_b(Ctx* ctx, Op opb, int64_t m, int64_t n, int64_t k, cplx alpha,
                            const cplx* A, int64_t lda, int64_t sA, const cplx* B, int64_t ldb,
                            int64_t sB, cplx beta, cplx* C, int64_t ldc, int64_t sC, int64_t batch,
                            int lower) {
    int64_t blocks = (m * n * batch + 63) / 64;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (blocks > cap) blocks = cap;
    const unsigned g = (unsigned)(blocks < 1 ? 1 : blocks);
    switch (opb) {
#define TN_ZS(OB) case OB: zgemm_small_kernel<OPA, OB><<<g, 64, 0, ctx->stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, lower); break;
        TN_ZS(OP_N) TN_ZS(OP_T) TN_ZS(OP_C) TN_ZS(OP_R)
#undef TN_ZS
    }
}

template <int OPA>
void zgemm_dispatch_b(Ctx* ctx, Op opb, dim3 grid, int64_t m, int64_t n, int64_t k, cplx alpha,
                      const cplx* A, int64_t lda, int64_t sA, const cplx* B, int64_t ldb,
                      int64_t sB, cplx beta, cplx* C, int64_t ldc, int64_t sC, int lower,
                      int64_t kc) {
    switch (opb) {
        case OP_N:
            zgemm_kernel<OPA, OP_N><<<grid, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, kc);
            break;
        case OP_T:
            zgemm_kernel<OPA, OP_T><<<grid, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, kc);
            break;
        case OP_C:
            zgemm_kernel<OPA, OP_C><<<grid, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, kc);
            break;
        case OP_R:
            zgemm_kernel<OPA, OP_R><<<grid, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, kc);
            break;
    }
}

// -------------------------------------------------------------------------
__global__ void small_apply_kernel(const cplx* __restrict__ in, cplx* __restrict__ out,
                                   const cplx* __restrict__ M, int nI, int nJ, int64_t na,
                                   int64_t nc, int64_t lda_i, int64_t ldc_i, int64_t lda_o,
                                   int64_t ldc_o, int accumulate) {
    extern __shared__ cplx sM[];
    for (int t = threadIdx.x; t < nI * nJ; t += blockDim.x) sM[t] = M[t];
    __syncthreads();
    const int64_t total = na * nc;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = idx % na, c = idx / na;
        const cplx* x = in + a + ldc_i * c;
        cplx* y = out + a + ldc_o * c;
        for (int J0 = 0; J0 < nJ; J0 += 4) {
            cplx s[4] = {cmk(0, 0), cmk(0, 0), cmk(0, 0), cmk(0, 0)};
            for (int I = 0; I < nI; ++I) {
                const cplx v = x[lda_i * I];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (J0 + j < nJ) s[j] = cfma(v, sM[I + nI * (J0 + j)], s[j]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (J0 + j >= nJ) break;
                cplx* dst = y + lda_o * (J0 + j);
                *dst = accumulate ? cadd(*dst, s[j]) : s[j];
            }
        }
    }
}

// -------------------------------------------------------------------------
constexpr int MAXV = 8;
struct PtrPack {
    const cplx* p[MAXV];
};

__device__ inline cplx warp_sum(cplx v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// partial[blk*K + j] = sum over this block's slice of conj(v_j[i]) * w[i]
template <int K>
__global__ void __launch_bounds__(256) multi_dot_kernel(PtrPack V, const cplx* __restrict__ w,
                                                        int64_t n, cplx* __restrict__ partial) {
    cplx acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = cmk(0, 0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const cplx wi = w[i];
#pragma unroll
        for (int j = 0; j < K; ++j) acc[j] = cfma(cconj(V.p[j][i]), wi, acc[j]);
    }
    __shared__ cplx red[8][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        cplx s = warp_sum(acc[j]);
        if (lane == 0) red[warp][j] = s;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        cplx s = cmk(0, 0);
        for (int wp = 0; wp < (int)(blockDim.x >> 5); ++wp) s = cadd(s, red[wp][threadIdx.x]);
        partial[blockIdx.x * K + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) bilinear_dot_kernel(const cplx* __restrict__ x,
                                                           const cplx* __restrict__ y, int64_t n,
                                                           cplx* __restrict__ partial) {
    cplx acc = cmk(0, 0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        acc = cfma(x[i], y[i], acc);
    __shared__ cplx red[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    acc = warp_sum(acc);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        cplx s = cmk(0, 0);
        for (int wp = 0; wp < (int)(blockDim.x >> 5); ++wp) s = cadd(s, red[wp]);
        partial[blockIdx.x] = s;
    }
}

__global__ void reduce_partials_kernel(const cplx* __restrict__ partial, int nblk, int K,
                                       cplx* __restrict__ out) {
    // one warp per output, fixed order -> deterministic
    const int j = blockIdx.x;
    cplx s = cmk(0, 0);
    for (int b = threadIdx.x; b < nblk; b += 32) s = cadd(s, partial[b * K + j]);
    s = warp_sum(s);
    if (threadIdx.x == 0) out[j] = s;
}

template <int K>
__global__ void multi_axpy_kernel(cplx* __restrict__ w, PtrPack V, const cplx* __restrict__ coef,
                                  int64_t n, double sign) {
    cplx c[K];
#pragma unroll
    for (int j = 0; j < K; ++j) c[j] = cmk(sign * coef[j].x, sign * coef[j].y);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        cplx acc = w[i];
#pragma unroll
        for (int j = 0; j < K; ++j) acc = cfma(c[j], V.p[j][i], acc);
        w[i] = acc;
    }
}

__global__ void zaxpy_kernel(cplx* __restrict__ y, const cplx* __restrict__ x, int64_t n, cplx a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = cfma(a, x[i], y[i]);
}

__global__ void zscale_kernel(cplx* x, int64_t n, cplx a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = cmul(a, x[i]);
}

__global__ void zscale_dev_kernel(cplx* x, int64_t n, const double* dnorm2, int invert_sqrt) {
    const double s = invert_sqrt ? 1.0 / sqrt(*dnorm2) : *dnorm2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = cmk(x[i].x * s, x[i].y * s);
}

__global__ void zfill_kernel(cplx* x, int64_t n, cplx v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}

__global__ void top_eigvecs_kernel(const cplx* __restrict__ G, int64_t n, int64_t k,
                                   int64_t ncols, cplx* __restrict__ dst) {
    const int64_t total = n * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        dst[i + n * j] = G[i + n * (ncols - 1 - j)];
    }
}

// *out = sum_i Re G[i, i] (one block)
__global__ void __launch_bounds__(1024) gram_trace_kernel(const cplx* __restrict__ G, int64_t n,
                                                          double* __restrict__ out) {
    __shared__ double ws[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += G[i + n * i].x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        *out = t;
    }
}

__global__ void scale_cols_kernel(cplx* X, int64_t m, int64_t k, const double* s, int invert) {
    const int64_t total = m * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = idx / m;
        const double f = invert ? (s[j] > 0 ? 1.0 / s[j] : 0.0) : s[j];
        X[idx] = cmk(X[idx].x * f, X[idx].y * f);
    }
}

__global__ void scale_rows_kernel(cplx* X, int64_t k, int64_t n, const double* s, int invert) {
    const int64_t total = k * n;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = idx % k;
        const double f = invert ? (s[j] > 0 ? 1.0 / s[j] : 0.0) : s[j];
        X[idx] = cmk(X[idx].x * f, X[idx].y * f);
    }
}

__global__ void conj_transpose_kernel(const cplx* __restrict__ src, int64_t r, int64_t c,
                                      cplx* __restrict__ dst) {
    __shared__ cplx tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t gr = r0 + threadIdx.x, gc = c0 + j;
        if (gr < r && gc < c) tile[j][threadIdx.x] = src[gr + r * gc];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t gc = c0 + threadIdx.x, gr = r0 + j;
        if (gr < r && gc < c) dst[gc + c * gr] = cconj(tile[threadIdx.x][j]);
    }
}

// out[j] = ||X[:, j]||, one warp per column
__global__ void col_norms_kernel(const cplx* __restrict__ X, int64_t m, int64_t k,
                                 double* __restrict__ out) {
    const int64_t j = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (j >= k) return;
    double s = 0.0;
    for (int64_t i = lane; i < m; i += 32) {
        const cplx v = X[i + m * j];
        s = fma(v.x, v.x, fma(v.y, v.y, s));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[j] = sqrt(s);
}

// out[i] = ||Y[i, :]|| for a column-major k x n matrix, one thread per row
__global__ void row_norms_kernel(const cplx* __restrict__ Y, int64_t k, int64_t n,
                                 double* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= k) return;
    double s = 0.0;
    for (int64_t j = 0; j < n; ++j) {
        const cplx v = Y[i + k * j];
        s = fma(v.x, v.x, fma(v.y, v.y, s));
    }
    out[i] = sqrt(s);
}

// -------------------------------------------------------------------------
// Keep rule (src/tensors.jl:200-215) on ascending Gram eigenvalues.  One
// block; thread t owns a contiguous chunk of the descending squared singular
// values; suffix sums come from a warp-shuffle scan over chunk totals.
struct KeepDev {
    int64_t k;
    double total, discarded;
};

__device__ inline double s2_at(const double* lam, int64_t n, int64_t i) {
    const double v = lam[n - 1 - i];
    return v > 0.0 ? v : 0.0;
}

__global__ void __launch_bounds__(1024) keep_rule_kernel(const double* __restrict__ lam, int64_t n,
                                                         int64_t sz, double cutoff, int64_t maxdim,
                                                         int64_t mindim, double* __restrict__ S_out,
                                                         const double* __restrict__ dtotal,
                                                         KeepDev* __restrict__ res) {
    __shared__ double wsum[32];
    __shared__ long long wcnt[32];
    __shared__ double s_total, s_rest;
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int nw = T >> 5;
    const int64_t per = (sz + T - 1) / T;
    const int64_t lo = min((int64_t)t * per, sz), hi = min(lo + per, sz);
    double local = 0.0;
    for (int64_t i = hi - 1; i >= lo; --i) local += s2_at(lam, n, i);
    // inclusive suffix scan over threads: incl(t) = sum_{t' >= t} local(t')
    double v = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v += u;
    }
    if (lane == 0) wsum[warp] = v;  // warp total
    __syncthreads();
    if (t == 0) {
        double acc = 0.0;
        for (int w = nw - 1; w >= 0; --w) {
            const double tw = wsum[w];
            wsum[w] = acc;  // sum of warps after w
            acc += tw;
        }
        // partial spectrum: the weight below the available values is the
        // trace minus their sum
        const double rest = dtotal ? fmax(*dtotal - acc, 0.0) : 0.0;
        s_rest = rest;
        s_total = acc + rest;
    }
    __syncthreads();
    const double rest = s_rest;
    const double after = v - local + wsum[warp] + rest;  // weight after chunk t
    const double total = s_total;
    long long cnt = 0;
    double tail = after;
    for (int64_t i = hi - 1; i >= lo; --i) {
        tail += s2_at(lam, n, i);
        if (tail / total > cutoff) ++cnt;  // NaN (total 0) compares false
        if (S_out) S_out[i] = sqrt(s2_at(lam, n, i));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0) wcnt[warp] = cnt;
    __syncthreads();
    if (t == 0) {
        long long c = 0;
        for (int w = 0; w < nw; ++w) c += wcnt[w];
        int64_t mind = min(mindim, sz);
        int64_t maxd = (maxdim == 0 || maxdim > sz) ? sz : maxdim;
        if (maxd == 0) maxd = 1;
        if (cutoff != 0.0) {
            const int64_t idxs = c > 0 ? (int64_t)c : 1;
            maxd = min(maxd, idxs);
        }
        const int64_t k = max(maxd, mind);
        res->k = k;
        res->total = total;
        res->discarded = 0.0;
    }
    __syncthreads();
    // discarded weight = sum_{i >= k} s2 / total
    const int64_t k = res->k;
    double disc = 0.0;
    for (int64_t i = max(lo, k); i < hi; ++i) disc += s2_at(lam, n, i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) disc += __shfl_down_sync(0xffffffffu, disc, o);
    __syncthreads();
    if (lane == 0) wsum[warp] = disc;
    __syncthreads();
    if (t == 0) {
        double d = rest;
        for (int w = 0; w < nw; ++w) d += wsum[w];
        res->discarded = total > 0 ? d / total : 0.0;
    }
}

inline int grid_for(Ctx* ctx, int64_t n, int threads = 256) {
    int64_t g = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)ctx->sm_count * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// -------------------------------------------------------------------------
void zgemm(Ctx* ctx, Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplx alpha, const cplx* A,
           int64_t lda, int64_t sA, const cplx* B, int64_t ldb, int64_t sB, cplx beta, cplx* C,
           int64_t ldc, int64_t sC, int64_t batch, bool lower_only) {
    if (m <= 0 || n <= 0 || batch <= 0) return;
    const int lower = lower_only ? 1 : 0;
    TN_REQUIRE((n + GB_N - 1) / GB_N <= 65535 && batch <= 65535, "zgemm: grid too large");
    dim3 grid((unsigned)((m + GB_M - 1) / GB_M), (unsigned)((n + GB_N - 1) / GB_N), (unsigned)batch);
    if (k <= 0) {  // C = beta * C
        alpha = cmk(0, 0);
    }
    ProfScope ps(ctx, 1, (lower ? 0.5 : 1.0) * 8.0 * m * n * (double)std::max<int64_t>(k, 0) * batch,
                 16.0 * (double)(m * k + k * n + m * n) * batch);
    if (std::min(m, n) < 48) {
        switch (opa) {
            case OP_N: zgemm_small_dispatch_b<OP_N>(ctx, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, lower); break;
            case OP_T: zgemm_small_dispatch_b<OP_T>(ctx, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, lower); break;
            case OP_C: zgemm_small_dispatch_b<OP_C>(ctx, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, lower); break;
            case OP_R: zgemm_small_dispatch_b<OP_R>(ctx, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, lower); break;
        }
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
        return;
    }
    // Split K when the tiles cannot fill the SMs (the Gram and projection
    // products of bond dimensions 128-512): S chunks of at least 128, each
    // into its own partial, summed in chunk order by a second kernel.
    const int64_t tiles = (int64_t)grid.x * grid.y;
    int64_t S = 1;
    if (ctx->splitk && batch == 1 && k >= 512 && tiles < ctx->sm_count)
        S = std::min<int64_t>((2 * ctx->sm_count + tiles - 1) / tiles, k / 128);
    if (S > 1) {
        const int64_t kc = ((k + S - 1) / S + GB_K - 1) / GB_K * GB_K;
        S = (k + kc - 1) / kc;
        cplx* P = ctx->s_splitk.c(ctx, (size_t)(S * m * n));
        dim3 g2(grid.x, grid.y, (unsigned)S);
        const cplx one = cmk(1, 0), zero = cmk(0, 0);
        switch (opa) {
            case OP_N: zgemm_dispatch_b<OP_N>(ctx, opb, g2, m, n, k, one, A, lda, 0, B, ldb, 0, zero, P, m, 0, lower, kc); break;
            case OP_T: zgemm_dispatch_b<OP_T>(ctx, opb, g2, m, n, k, one, A, lda, 0, B, ldb, 0, zero, P, m, 0, lower, kc); break;
            case OP_C: zgemm_dispatch_b<OP_C>(ctx, opb, g2, m, n, k, one, A, lda, 0, B, ldb, 0, zero, P, m, 0, lower, kc); break;
            case OP_R: zgemm_dispatch_b<OP_R>(ctx, opb, g2, m, n, k, one, A, lda, 0, B, ldb, 0, zero, P, m, 0, lower, kc); break;
        }
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
        const int64_t blocks = std::min<int64_t>((m * n + 255) / 256, (int64_t)ctx->sm_count * 8);
        splitk_reduce_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(P, m, n, (int)S, alpha, beta,
                                                                        C, ldc, lower);
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
        return;
    }
    switch (opa) {
        case OP_N: zgemm_dispatch_b<OP_N>(ctx, opb, grid, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, 0); break;
        case OP_T: zgemm_dispatch_b<OP_T>(ctx, opb, grid, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, 0); break;
        case OP_C: zgemm_dispatch_b<OP_C>(ctx, opb, grid, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, 0); break;
        case OP_R: zgemm_dispatch_b<OP_R>(ctx, opb, grid, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, lower, 0); break;
    }
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void small_apply(Ctx* ctx, const cplx* in, cplx* out, const cplx* M, int nI, int nJ, int64_t na,
                 int64_t nc, int64_t lda_i, int64_t ldc_i, int64_t lda_o, int64_t ldc_o,
                 bool accumulate) {
    if (na <= 0 || nc <= 0) return;
    TN_REQUIRE(nI * nJ <= 4096, "small_apply: operator too large");
    const size_t smem = sizeof(cplx) * nI * nJ;
    // the whole operator is staged in shared memory: up to 64 KiB, above the
    // 48 KiB a launch gets without opting in
    if (smem > 48 * 1024)
        TN_CHECK_CUDA(cudaFuncSetAttribute(small_apply_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(cplx) * 4096)));
    ProfScope ps(ctx, 3, 8.0 * na * nc * nI * nJ, 16.0 * na * nc * (nI + nJ));
    small_apply_kernel<<<grid_for(ctx, na * nc), 256, smem, ctx->stream>>>(
        in, out, M, nI, nJ, na, nc, lda_i, ldc_i, lda_o, ldc_o, accumulate ? 1 : 0);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void multi_dot(Ctx* ctx, const cplx* const* hV, int K, const cplx* w, int64_t n, cplx* dout) {
    ProfScope ps(ctx, 6, 8.0 * n * K, 16.0 * n * (K + 1));
    const int nblk = grid_for(ctx, n);
    cplx* partial = ctx->s_dot.c(ctx, (size_t)nblk * MAXV);
    for (int j0 = 0; j0 < K; j0 += MAXV) {
        const int kk = std::min(MAXV, K - j0);
        PtrPack P{};
        for (int j = 0; j < kk; ++j) P.p[j] = hV[j0 + j];
        switch (kk) {
#define TN_MD(KK) case KK: multi_dot_kernel<KK><<<nblk, 256, 0, ctx->stream>>>(P, w, n, partial); break;
            TN_MD(1) TN_MD(2) TN_MD(3) TN_MD(4) TN_MD(5) TN_MD(6) TN_MD(7) TN_MD(8)
#undef TN_MD
        }
        ctx->count();
        reduce_partials_kernel<<<kk, 32, 0, ctx->stream>>>(partial, nblk, kk, dout + j0);
        ctx->count();
    }
    TN_CHECK_CUDA(cudaGetLastError());
}

void bilinear_dot(Ctx* ctx, const cplx* x, const cplx* y, int64_t n, cplx* dout) {
    const int nblk = grid_for(ctx, n);
    cplx* partial = ctx->s_dot.c(ctx, (size_t)nblk * MAXV);
    bilinear_dot_kernel<<<nblk, 256, 0, ctx->stream>>>(x, y, n, partial);
    ctx->count();
    reduce_partials_kernel<<<1, 32, 0, ctx->stream>>>(partial, nblk, 1, dout);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void multi_axpy(Ctx* ctx, cplx* w, const cplx* const* hV, const cplx* dcoef, int K, int64_t n,
                double sign) {
    ProfScope ps(ctx, 6, 8.0 * n * K, 16.0 * n * (K + 2));
    const int nblk = grid_for(ctx, n);
    for (int j0 = 0; j0 < K; j0 += MAXV) {
        const int kk = std::min(MAXV, K - j0);
        PtrPack P{};
        for (int j = 0; j < kk; ++j) P.p[j] = hV[j0 + j];
        switch (kk) {
#define TN_MA(KK) case KK: multi_axpy_kernel<KK><<<nblk, 256, 0, ctx->stream>>>(w, P, dcoef + j0, n, sign); break;
            TN_MA(1) TN_MA(2) TN_MA(3) TN_MA(4) TN_MA(5) TN_MA(6) TN_MA(7) TN_MA(8)
#undef TN_MA
        }
        ctx->count();
    }
    TN_CHECK_CUDA(cudaGetLastError());
}

void zaxpy(Ctx* ctx, cplx* y, const cplx* x, int64_t n, cplx a) {
    if (n <= 0) return;
    ProfScope ps(ctx, 6, 8.0 * n, 48.0 * n);
    zaxpy_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(y, x, n, a);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void zscale(Ctx* ctx, cplx* x, int64_t n, cplx a) {
    if (n <= 0) return;
    zscale_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(x, n, a);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void zscale_dev(Ctx* ctx, cplx* x, int64_t n, const double* dnorm2, int invert) {
    if (n <= 0) return;
    zscale_dev_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(x, n, dnorm2, invert);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void zcopy(Ctx* ctx, cplx* dst, const cplx* src, int64_t n) {
    if (n <= 0) return;
    TN_CHECK_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(cplx), cudaMemcpyDeviceToDevice, ctx->stream));
}

void zfill(Ctx* ctx, cplx* dst, int64_t n, cplx v) {
    if (n <= 0) return;
    zfill_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(dst, n, v);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

double znorm2(Ctx* ctx, const cplx* x, int64_t n) {
    cplx* d = ctx->s_coef.c(ctx, 16);
    const cplx* V[1] = {x};
    multi_dot(ctx, V, 1, x, n, d);
    double* h = ctx->pinned(2);
    TN_CHECK_CUDA(cudaMemcpyAsync(h, d, sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    return h[0];
}

void take_top_eigvecs(Ctx* ctx, const cplx* G, int64_t n, int64_t k, cplx* dst, int64_t ncols) {
    if (n <= 0 || k <= 0) return;
    if (ncols < 0) ncols = n;
    TN_REQUIRE(k <= ncols, "take_top_eigvecs: k exceeds the available eigenvectors");
    top_eigvecs_kernel<<<grid_for(ctx, n * k), 256, 0, ctx->stream>>>(G, n, k, ncols, dst);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void gram_trace(Ctx* ctx, const cplx* G, int64_t n, double* dout) {
    gram_trace_kernel<<<1, 1024, 0, ctx->stream>>>(G, n, dout);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void conj_transpose(Ctx* ctx, const cplx* src, int64_t r, int64_t c, cplx* dst) {
    if (r <= 0 || c <= 0) return;
    TN_REQUIRE((c + 31) / 32 <= 65535, "conj_transpose: too many columns");
    dim3 grid((unsigned)((r + 31) / 32), (unsigned)((c + 31) / 32));
    conj_transpose_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>(src, r, c, dst);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void col_norms(Ctx* ctx, const cplx* X, int64_t m, int64_t k, double* out) {
    if (m <= 0 || k <= 0) return;
    col_norms_kernel<<<(unsigned)((k + 7) / 8), 256, 0, ctx->stream>>>(X, m, k, out);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void row_norms(Ctx* ctx, const cplx* Y, int64_t k, int64_t n, double* out) {
    if (n <= 0 || k <= 0) return;
    row_norms_kernel<<<(unsigned)((k + 127) / 128), 128, 0, ctx->stream>>>(Y, k, n, out);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void scale_cols(Ctx* ctx, cplx* X, int64_t m, int64_t k, const double* s, int invert) {
    if (m <= 0 || k <= 0) return;
    scale_cols_kernel<<<grid_for(ctx, m * k), 256, 0, ctx->stream>>>(X, m, k, s, invert);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void scale_rows(Ctx* ctx, cplx* X, int64_t k, int64_t n, const double* s, int invert) {
    if (n <= 0 || k <= 0) return;
    scale_rows_kernel<<<grid_for(ctx, n * k), 256, 0, ctx->stream>>>(X, k, n, s, invert);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

KeepResult keep_rule(Ctx* ctx, const double* dlam, int64_t n, int64_t sz, double cutoff,
                     int64_t maxdim, int64_t mindim, double* dS, const double* dtotal,
                     const int* dinfo) {
    TN_REQUIRE(sz <= n, "keep_rule: more singular values than eigenvalues");
    KeepDev* dres = static_cast<KeepDev*>(ctx->s_coef.get(ctx, 256));
    keep_rule_kernel<<<1, 1024, 0, ctx->stream>>>(dlam, n, sz, cutoff, maxdim, mindim, dS, dtotal,
                                                  dres);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    double* h = ctx->pinned(4);
    TN_CHECK_CUDA(cudaMemcpyAsync(h, dres, sizeof(KeepDev), cudaMemcpyDeviceToHost, ctx->stream));
    if (dinfo)
        TN_CHECK_CUDA(cudaMemcpyAsync(reinterpret_cast<int*>(h + 3), dinfo, sizeof(int),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (dinfo && *reinterpret_cast<int*>(h + 3) != 0) {
        // the eigensolver's error word: a bounded grid barrier ran out
        TN_CHECK_CUDA(cudaMemsetAsync(const_cast<int*>(dinfo), 0, sizeof(int), ctx->stream));
        throw Error(TN_ERR_TIMEOUT, "eigensolver: a bounded grid barrier ran out");
    }
    KeepDev r;
    memcpy(&r, h, sizeof(KeepDev));
    return KeepResult{r.k, r.total, r.discarded};
}

}  // namespace tn
