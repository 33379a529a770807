// Mixed-precision two-site H_eff product (projmps.jl:103-145 in the optimal
// contraction order) on the tcgen05 GEMM:
//
//   T1[(a w), (s1 s2 c)] = L[(a w), b] theta[b, (s1 s2 c)]       tensor cores
//   T2[(a s1' s2'), (w'' c)] = sum W12 T1                         FP32 SIMT
//   out[(a s1' s2'), c']   = T2 R[c', (w'' c)]^T                  tensor cores
//
// Inputs and outputs are FP64 complex.  Operands enter the tensor cores as
// split TF32 planes (hi = tf32(x), lo = tf32(x - hi)), laid out K-major by
// coalesced shared-memory transposes; T1 stays FP32.
#include "mixed.cuh"
#include "tc_gemm.cuh"

namespace tn {

namespace {

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void split_store(float* planes, size_t plane, size_t off, double re,
                                            double im) {
    const float rh = to_tf32((float)re), ih = to_tf32((float)im);
    const float rl = to_tf32((float)(re - (double)rh)), il = to_tf32((float)(im - (double)ih));
    planes[off] = rh;
    planes[plane + off] = ih;
    planes[2 * plane + off] = rl;
    planes[3 * plane + off] = il;
}

// planes[z][r][k] <- src[k + K*r]: a column-major K x rows matrix whose
// columns become operand rows (already K-major).
__global__ void split_natural_kernel(const cplx* __restrict__ src, int64_t rows, int64_t K,
                                     float* __restrict__ planes, int64_t ld) {
    const size_t plane = (size_t)rows * ld;
    const int64_t total = rows * ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ld, k = i - r * ld;
        double re = 0.0, im = 0.0;
        if (k < K) {
            const cplx v = src[k + K * r];
            re = v.x;
            im = v.y;
        }
        split_store(planes, plane, (size_t)i, re, im);
    }
}

// planes[z][r][k] <- src[r + lds*k]: a column-major rows x K matrix
// transposed to K-major through a 32 x 32 shared-memory tile.
__global__ void split_transpose_kernel(const cplx* __restrict__ src, int64_t rows, int64_t K,
                                       int64_t lds, float* __restrict__ planes, int64_t ld) {
    __shared__ cplx tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 32;
    const size_t plane = (size_t)rows * ld;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t r = r0 + threadIdx.x, k = k0 + j;
        tile[j][threadIdx.x] = (r < rows && k < K) ? src[r + lds * k] : cmk(0, 0);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t r = r0 + j, k = k0 + threadIdx.x;
        if (r < rows && k < ld) {
            const cplx v = tile[threadIdx.x][j];
            split_store(planes, plane, (size_t)r * ld + k, v.x, v.y);
        }
    }
}

// The W12 leg.  Block = 32 values of a x 8 values of c.  Reads T1 (FP32
// planar, column-major [(a w), (s1 s2 c)]) coalesced along a, applies the
// nI x nJ operator from shared memory, stages the nJ results per (a, c) in
// shared memory and writes K-major split planes T2[(a s1' s2')][(w'' c)]
// coalesced along (w'' c).
constexpr int MID_A = 32, MID_C = 8, MID_MAXJ = 32;

__global__ void __launch_bounds__(256) heff_mid_kernel(
    const float* __restrict__ t1r, const float* __restrict__ t1i, int S1, int64_t chunk1,
    int64_t ldt1, int64_t cl,
    int64_t cr, int d, int wl, int wr, const cplx* __restrict__ W12, float* __restrict__ planes,
    int64_t ld2, int64_t rows2) {
    const int d2 = d * d, nI = wl * d2, nJ = d2 * wr;
    extern __shared__ float sm[];
    float2* sW = reinterpret_cast<float2*>(sm);                 // nI * nJ
    float2* sY = sW + nI * nJ;                                   // [MID_C][MID_A][nJ]
    for (int t = threadIdx.x; t < nI * nJ; t += blockDim.x)
        sW[t] = make_float2((float)W12[t].x, (float)W12[t].y);
    __syncthreads();
    const int ta = threadIdx.x & 31, tc = threadIdx.x >> 5;
    const int64_t a = (int64_t)blockIdx.x * MID_A + ta;
    const int64_t c = (int64_t)blockIdx.y * MID_C + tc;
    float2 y[MID_MAXJ];
#pragma unroll
    for (int J = 0; J < MID_MAXJ; ++J) y[J] = make_float2(0.f, 0.f);
    if (a < cl && c < cr) {
        for (int I = 0; I < nI; ++I) {
            // I = w + wl*(s1 + d*s2); T1 row (a + cl*w), column (s1 + d*s2 + d2*c)
            const int w = I % wl, s12 = I / wl;
            const int64_t off = (a + cl * w) + ldt1 * (s12 + (int64_t)d2 * c);
            // sum the K-chunk partials of GEMM1 in float-float, then round
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int z = 0; z < S1; ++z) {
                ff_add(rh, rl, t1r[(size_t)z * chunk1 + off]);
                ff_add(ih, il, t1i[(size_t)z * chunk1 + off]);
            }
            const float xr = rh + rl, xi = ih + il;
#pragma unroll
            for (int J = 0; J < MID_MAXJ; ++J) {
                if (J < nJ) {
                    const float2 m = sW[I + nI * J];
                    y[J].x = fmaf(xr, m.x, fmaf(-xi, m.y, y[J].x));
                    y[J].y = fmaf(xr, m.y, fmaf(xi, m.x, y[J].y));
                }
            }
        }
    }
#pragma unroll
    for (int J = 0; J < MID_MAXJ; ++J)
        if (J < nJ) sY[(tc * MID_A + ta) * nJ + J] = y[J];
    __syncthreads();
    // rows (a, s1', s2') x columns (w'' + wr*c) for this block's c range
    const size_t plane = (size_t)rows2 * ld2;
    // each thread keeps one column (w'', c) and walks rows: the divisions by
    // wr happen once per thread, the row split is by the power-of-two MID_A
    const int ncol = wr * MID_C;  // <= 64: d2 * wr <= MID_MAXJ
    const int nrow = MID_A * d2;
    const int rpp = blockDim.x / ncol;  // rows per pass
    const int tcol = threadIdx.x % ncol, trow = threadIdx.x / ncol;
    if (trow >= rpp) return;
    const int w2 = tcol % wr, cloc = tcol / wr;
    const int64_t cg = (int64_t)blockIdx.y * MID_C + cloc;
    if (cg >= cr) return;
    const int64_t Kc = w2 + (int64_t)wr * cg;
    for (int row = trow; row < nrow; row += rpp) {
        const int al = row % MID_A, s12 = row / MID_A;
        const int64_t ag = (int64_t)blockIdx.x * MID_A + al;
        if (ag >= cl) continue;
        const float2 v = sY[(cloc * MID_A + al) * nJ + (s12 + d2 * w2)];
        const int64_t R = ag + cl * s12;
        const size_t off = (size_t)R * ld2 + Kc;
        const float rh = to_tf32(v.x), ih = to_tf32(v.y);
        planes[off] = rh;
        planes[plane + off] = ih;
        planes[2 * plane + off] = to_tf32(v.x - rh);
        planes[3 * plane + off] = to_tf32(v.y - ih);
    }
}

// ---- environment legs ------------------------------------------------------
constexpr int ENV_MAX = 16;  // w * d on either side of an MPO leg

__device__ __forceinline__ void store_split(float* planes, size_t plane, size_t off, float re,
                                            float im) {
    const float rh = to_tf32(re), ih = to_tf32(im);
    planes[off] = rh;
    planes[plane + off] = ih;
    planes[2 * plane + off] = to_tf32(re - rh);
    planes[3 * plane + off] = to_tf32(im - ih);
}

// Left environment leg: X[(a w),(s b')] (K-chunk partials, FP32 planar,
// column-major) -> Y[(a s'),(w' b')] = sum_{w,s} X Ml[(w,s),(s',w')], written
// as split planes with rows (w' b') and K = (a s') (coalesced along a).
__global__ void __launch_bounds__(128) env_left_leg_kernel(
    const float* __restrict__ P, int S, int64_t chunk, int64_t M, int64_t plane_in, int64_t ca,
    int wl, int d, int wr, const cplx* __restrict__ Ml, float* __restrict__ planes, int64_t ld,
    int64_t rows) {
    const int nI = wl * d, nJ = d * wr;
    __shared__ float2 sM[ENV_MAX * ENV_MAX];
    for (int t = threadIdx.x; t < nI * nJ; t += blockDim.x)
        sM[t] = make_float2((float)Ml[t].x, (float)Ml[t].y);
    __syncthreads();
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, bp = blockIdx.y;
    if (a >= ca) return;
    float2 x[ENV_MAX];
#pragma unroll
    for (int I = 0; I < ENV_MAX; ++I) {
        x[I] = make_float2(0.f, 0.f);
        if (I < nI) {
            const int w = I % wl, s = I / wl;
            const int64_t off = (a + ca * w) + M * (s + (int64_t)d * bp);
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int z = 0; z < S; ++z) {
                ff_add(rh, rl, P[(size_t)z * chunk + off]);
                ff_add(ih, il, P[(size_t)z * chunk + plane_in + off]);
            }
            x[I] = make_float2(rh + rl, ih + il);
        }
    }
    const size_t plane = (size_t)rows * ld;
    for (int J = 0; J < nJ; ++J) {
        float yr = 0.f, yi = 0.f;
#pragma unroll
        for (int I = 0; I < ENV_MAX; ++I) {
            if (I < nI) {
                const float2 m = sM[I + nI * J];
                yr = fmaf(x[I].x, m.x, fmaf(-x[I].y, m.y, yr));
                yi = fmaf(x[I].x, m.y, fmaf(x[I].y, m.x, yi));
            }
        }
        const int sp = J % d, wp = J / d;
        const int64_t n = wp + (int64_t)wr * bp, k = a + ca * sp;
        store_split(planes, plane, (size_t)n * ld + k, yr, yi);
    }
}

// Right environment leg: Z[(a s'),(w' b')] partials -> Z2[(a w),(s b')] =
// sum_{s',w'} Z Mr[(s',w'),(w,s)], written as split planes with rows (a w)
// and K = (s b'), staged through shared memory (32 a x 8 b' per block).
constexpr int ENVR_A = 32, ENVR_B = 8;
__global__ void __launch_bounds__(256) env_right_leg_kernel(
    const float* __restrict__ P, int S, int64_t chunk, int64_t M, int64_t plane_in, int64_t ca,
    int64_t cb2, int wl, int d, int wr, const cplx* __restrict__ Mr, float* __restrict__ planes,
    int64_t ld, int64_t rows) {
    const int nI = d * wr, nJ = wl * d;
    __shared__ float2 sM[ENV_MAX * ENV_MAX];
    __shared__ float2 sY[ENVR_B][ENVR_A][ENV_MAX];
    for (int t = threadIdx.x; t < nI * nJ; t += blockDim.x)
        sM[t] = make_float2((float)Mr[t].x, (float)Mr[t].y);
    __syncthreads();
    const int ta = threadIdx.x & 31, tb = threadIdx.x >> 5;
    const int64_t a = (int64_t)blockIdx.x * ENVR_A + ta, bp = (int64_t)blockIdx.y * ENVR_B + tb;
    float2 x[ENV_MAX];
#pragma unroll
    for (int I = 0; I < ENV_MAX; ++I) {
        x[I] = make_float2(0.f, 0.f);
        if (I < nI && a < ca && bp < cb2) {
            const int sp = I % d, wp = I / d;
            const int64_t off = (a + ca * sp) + M * (wp + (int64_t)wr * bp);
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int z = 0; z < S; ++z) {
                ff_add(rh, rl, P[(size_t)z * chunk + off]);
                ff_add(ih, il, P[(size_t)z * chunk + plane_in + off]);
            }
            x[I] = make_float2(rh + rl, ih + il);
        }
    }
    for (int J = 0; J < nJ; ++J) {
        float yr = 0.f, yi = 0.f;
#pragma unroll
        for (int I = 0; I < ENV_MAX; ++I) {
            if (I < nI) {
                const float2 m = sM[I + nI * J];
                yr = fmaf(x[I].x, m.x, fmaf(-x[I].y, m.y, yr));
                yi = fmaf(x[I].x, m.y, fmaf(x[I].y, m.x, yi));
            }
        }
        sY[tb][ta][J] = make_float2(yr, yi);
    }
    __syncthreads();
    // rows (a + ca*w) of this block's a range; columns k = s + d*b' of its b' range
    const size_t plane = (size_t)rows * ld;
    const int ncol = d * ENVR_B, nrow = ENVR_A * wl;
    for (int e = threadIdx.x; e < nrow * ncol; e += blockDim.x) {
        const int col = e % ncol, row = e / ncol;
        const int al = row % ENVR_A, w = row / ENVR_A;
        const int s = col % d, bl = col / d;
        const int64_t ag = (int64_t)blockIdx.x * ENVR_A + al;
        const int64_t bg = (int64_t)blockIdx.y * ENVR_B + bl;
        if (ag >= ca || bg >= cb2) continue;
        const float2 v = sY[bl][al][w + wl * s];
        store_split(planes, plane, (size_t)(ag + ca * w) * ld + (s + (int64_t)d * bg), v.x, v.y);
    }
}

// zero the K padding columns [K, ld) of T2 planes (only when ld > K)
__global__ void zero_pad_kernel(float* planes, int64_t rows, int64_t K, int64_t ld) {
    const int64_t pad = ld - K;
    const int64_t total = 4 * rows * pad;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t z = i / (rows * pad), rem = i % (rows * pad);
        const int64_t r = rem / pad, k = K + rem % pad;
        planes[(size_t)z * rows * ld + (size_t)r * ld + k] = 0.f;
    }
}

inline int grid_n(Ctx* ctx, int64_t n) {
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

void split_natural(Ctx* ctx, const cplx* src, int64_t rows, int64_t K, TcPlanes& t, Scratch& s) {
    t.rows = rows;
    t.K = K;
    t.ld = tc_ld(K);
    t.p = static_cast<float*>(s.get(ctx, sizeof(float) * t.floats()));
    ProfScope ps(ctx, 5, 0.0, 16.0 * rows * K + 16.0 * rows * t.ld);
    split_natural_kernel<<<grid_n(ctx, rows * t.ld), 256, 0, ctx->stream>>>(src, rows, K, t.p, t.ld);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void split_transpose(Ctx* ctx, const cplx* src, int64_t rows, int64_t K, int64_t lds, TcPlanes& t,
                     Scratch& s) {
    t.rows = rows;
    t.K = K;
    t.ld = tc_ld(K);
    t.p = static_cast<float*>(s.get(ctx, sizeof(float) * t.floats()));
    TN_REQUIRE((t.ld + 31) / 32 <= 65535, "split_transpose: K too large");
    dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((t.ld + 31) / 32));
    ProfScope ps(ctx, 5, 0.0, 16.0 * rows * K + 16.0 * rows * t.ld);
    split_transpose_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>(src, rows, K, lds, t.p, t.ld);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

void heff2_planes(Ctx* ctx, MixedWork& B, const cplx* W12, int64_t cl, int64_t cr, int d,
                  int64_t wl, int64_t wr, const cplx* x, cplx* y) {
    const int64_t d2 = (int64_t)d * d;
    TN_REQUIRE(d2 * wr <= MID_MAXJ && wl * d2 <= 64, "mixed H_eff: MPO bond too large");
    // theta as GEMM1's B operand: rows (s1 s2 c), K = b
    TcPlanes th;
    split_natural(ctx, x, d2 * cr, cl, th, B.th);
    // T1 = L * theta, FP32 planar column-major [(a w), (s1 s2 c)]
    const int64_t M1 = cl * wl, N1 = d2 * cr;
    const int S1 = tc_chunks(cl);
    const int64_t chunk1 = 2 * M1 * N1;
    float* t1 = static_cast<float*>(B.t1.get(ctx, sizeof(float) * (size_t)S1 * chunk1));
    tc_cgemm_partials(ctx, B.Lp, th, M1, N1, cl, false, TC_KCHUNK, t1, M1, M1 * N1, chunk1);
    // T2 planes, K-major rows (a s1' s2'), K = (w'' c)
    TcPlanes t2;
    t2.rows = cl * d2;
    t2.K = wr * cr;
    t2.ld = tc_ld(t2.K);
    t2.p = static_cast<float*>(B.t2.get(ctx, sizeof(float) * t2.floats()));
    if (t2.ld > t2.K) {
        zero_pad_kernel<<<grid_n(ctx, 4 * t2.rows * (t2.ld - t2.K)), 256, 0, ctx->stream>>>(
            t2.p, t2.rows, t2.K, t2.ld);
        ctx->count();
    }
    const int nI = (int)(wl * d2), nJ = (int)(d2 * wr);
    const size_t smem = sizeof(float2) * ((size_t)nI * nJ + (size_t)MID_C * MID_A * nJ);
    dim3 grid((unsigned)((cl + MID_A - 1) / MID_A), (unsigned)((cr + MID_C - 1) / MID_C));
    TN_REQUIRE(grid.y <= 65535, "mixed H_eff: chi too large");
    ProfScope ps(ctx, 4, 8.0 * cl * cr * nI * nJ,
                 8.0 * (double)S1 * M1 * N1 + 16.0 * (double)t2.rows * t2.K);
    heff_mid_kernel<<<grid, 256, smem, ctx->stream>>>(t1, t1 + (size_t)M1 * N1, S1, chunk1, M1,
                                                      cl, cr, d, (int)wl, (int)wr, W12, t2.p,
                                                      t2.ld, t2.rows);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    // out = T2 * R^T, partials summed in float-float into FP64 [(a s1' s2'), c']
    const int64_t M3 = cl * d2, N3 = cr;
    const int S3 = tc_chunks(wr * cr);
    const int64_t chunk3 = 2 * M3 * N3;
    float* p3 = static_cast<float*>(B.p3.get(ctx, sizeof(float) * (size_t)S3 * chunk3));
    tc_cgemm_partials(ctx, t2, B.Rp, M3, N3, wr * cr, false, TC_KCHUNK, p3, M3, M3 * N3, chunk3);
    tc_reduce_fp64(ctx, p3, S3, M3, N3, M3, M3 * N3, chunk3, y, M3, false);
}

}  // namespace

void mixed_prepare_env(Ctx* ctx, MixedWork& mw, const cplx* L, const cplx* R, int64_t cl,
                       int64_t cr, int d, int64_t wl, int64_t wr) {
    MixedWork& B = mw;
    // L as GEMM1's A operand: rows (a w), K = b; R as GEMM3's B: rows c', K = (w'' c)
    split_transpose(ctx, L, cl * wl, cl, cl * wl, B.Lp, B.L);
    split_transpose(ctx, R, cr, wr * cr, cr, B.Rp, B.R);
    mw.cl = cl;
    mw.cr = cr;
    mw.wl = wl;
    mw.wr = wr;
    mw.d = d;
}

void mixed_heff2(Ctx* ctx, MixedWork& mw, const cplx* W12, int64_t cl, int64_t cr, int d,
                 int64_t wl, int64_t wr, const cplx* x, cplx* y) {
    TN_REQUIRE(mw.cl == cl && mw.cr == cr && mw.wl == wl && mw.wr == wr && mw.d == d,
               "mixed H_eff: environment not prepared for this bond");
    heff2_planes(ctx, mw, W12, cl, cr, d, wl, wr, x, y);
}

// L'[a',w',b'] = sum L[a,w,b] conj(A[a,s',a']) W[w,s',s,w'] B[b,s,b']
// (projmps.jl:50-66) with both GEMMs on the tensor cores.
void mixed_env_left(Ctx* ctx, const cplx* L, int64_t ca, int64_t wl, int64_t cb, const cplx* A,
                    int64_t ca2, const cplx* Ml, int d, int64_t wr, const cplx* B, int64_t cb2,
                    cplx* out) {
    TN_REQUIRE(wl * d <= ENV_MAX && wr * d <= ENV_MAX, "mixed environment: MPO bond too large");
    TcPlanes pL, pB, pY, pA;
    // X[(a w), (s b')] = L[(a w), b] B[b, (s b')]
    split_transpose(ctx, L, ca * wl, cb, ca * wl, pL, ctx->s_mixa);
    split_natural(ctx, B, d * cb2, cb, pB, ctx->s_mixb);
    const int64_t M1 = ca * wl, N1 = d * cb2;
    const int S1 = tc_chunks(cb);
    const int64_t ch1 = 2 * M1 * N1;
    float* P1 = static_cast<float*>(ctx->s_mixc.get(ctx, sizeof(float) * (size_t)S1 * ch1));
    tc_cgemm_partials(ctx, pL, pB, M1, N1, cb, false, TC_KCHUNK, P1, M1, M1 * N1, ch1);
    // Y as split planes, rows (w' b'), K = (a s')
    pY.rows = wr * cb2;
    pY.K = ca * d;
    pY.ld = tc_ld(pY.K);
    pY.p = static_cast<float*>(ctx->s_mixd.get(ctx, sizeof(float) * pY.floats()));
    {
        ProfScope ps(ctx, 4, 8.0 * ca * cb2 * (wl * d) * (d * wr),
                     8.0 * (double)S1 * M1 * N1 + 16.0 * (double)pY.rows * pY.K);
        dim3 grid((unsigned)((ca + 127) / 128), (unsigned)cb2);
        env_left_leg_kernel<<<grid, 128, 0, ctx->stream>>>(P1, S1, ch1, M1, M1 * N1, ca, (int)wl, d,
                                                           (int)wr, Ml, pY.p, pY.ld, pY.rows);
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    }
    // out[a', (w' b')] = conj(A)[(a s'), a']^T Y
    split_natural(ctx, A, ca2, ca * d, pA, ctx->s_mixa);
    const int64_t M3 = ca2, N3 = wr * cb2;
    const int S3 = tc_chunks(ca * d);
    const int64_t ch3 = 2 * M3 * N3;
    float* P3 = static_cast<float*>(ctx->s_mixe.get(ctx, sizeof(float) * (size_t)S3 * ch3));
    tc_cgemm_partials(ctx, pA, pY, M3, N3, ca * d, true, TC_KCHUNK, P3, M3, M3 * N3, ch3);
    tc_reduce_fp64(ctx, P3, S3, M3, N3, M3, M3 * N3, ch3, out, M3, false);
}

// R[a,w,b] = sum B[b,s,b'] R'[a',w',b'] W[w,s',s,w'] conj(A[a,s',a'])
// (projmps.jl:74-95) with both GEMMs on the tensor cores.
void mixed_env_right(Ctx* ctx, const cplx* R, int64_t ca2, int64_t wr, int64_t cb2, const cplx* A,
                     int64_t ca, const cplx* Mr, int d, int64_t wl, const cplx* B, int64_t cb,
                     cplx* out) {
    TN_REQUIRE(wl * d <= ENV_MAX && wr * d <= ENV_MAX, "mixed environment: MPO bond too large");
    TcPlanes pA, pR, pZ, pB;
    // Z[(a s'), (w' b')] = conj(A)[(a s'), a'] R[a', (w' b')]
    split_transpose(ctx, A, ca * d, ca2, ca * d, pA, ctx->s_mixa);
    split_natural(ctx, R, wr * cb2, ca2, pR, ctx->s_mixb);
    const int64_t M1 = ca * d, N1 = wr * cb2;
    const int S1 = tc_chunks(ca2);
    const int64_t ch1 = 2 * M1 * N1;
    float* P1 = static_cast<float*>(ctx->s_mixc.get(ctx, sizeof(float) * (size_t)S1 * ch1));
    tc_cgemm_partials(ctx, pA, pR, M1, N1, ca2, true, TC_KCHUNK, P1, M1, M1 * N1, ch1);
    // Z2 as split planes, rows (a w), K = (s b')
    pZ.rows = ca * wl;
    pZ.K = d * cb2;
    pZ.ld = tc_ld(pZ.K);
    pZ.p = static_cast<float*>(ctx->s_mixd.get(ctx, sizeof(float) * pZ.floats()));
    {
        ProfScope ps(ctx, 4, 8.0 * ca * cb2 * (wl * d) * (d * wr),
                     8.0 * (double)S1 * M1 * N1 + 16.0 * (double)pZ.rows * pZ.K);
        dim3 grid((unsigned)((ca + ENVR_A - 1) / ENVR_A), (unsigned)((cb2 + ENVR_B - 1) / ENVR_B));
        TN_REQUIRE(grid.y <= 65535, "mixed environment: chi too large");
        env_right_leg_kernel<<<grid, 256, 0, ctx->stream>>>(P1, S1, ch1, M1, M1 * N1, ca, cb2,
                                                            (int)wl, d, (int)wr, Mr, pZ.p, pZ.ld,
                                                            pZ.rows);
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    }
    // out[(a w), b] = Z2[(a w), (s b')] B[b, (s b')]^T
    split_transpose(ctx, B, cb, d * cb2, cb, pB, ctx->s_mixa);
    const int64_t M3 = ca * wl, N3 = cb;
    const int S3 = tc_chunks(d * cb2);
    const int64_t ch3 = 2 * M3 * N3;
    float* P3 = static_cast<float*>(ctx->s_mixe.get(ctx, sizeof(float) * (size_t)S3 * ch3));
    tc_cgemm_partials(ctx, pZ, pB, M3, N3, d * cb2, false, TC_KCHUNK, P3, M3, M3 * N3, ch3);
    tc_reduce_fp64(ctx, P3, S3, M3, N3, M3, M3 * N3, ch3, out, M3, false);
}

// C (m x n, FP64 column-major) = op(A) B on the tensor cores.  A is m x k
// column-major, or k x m when conj_a (op(A) = A^H); B is k x n.
void mixed_gemm(Ctx* ctx, int64_t m, int64_t n, int64_t k, const cplx* A, bool conj_a,
                const cplx* B, cplx* C) {
    Scratch sa, sb;
    TcPlanes pa, pb;
    if (conj_a)  // A^H rows m are columns of A: already K-major
        split_natural(ctx, A, m, k, pa, sa);
    else
        split_transpose(ctx, A, m, k, m, pa, sa);
    split_natural(ctx, B, n, k, pb, sb);
    const int S = tc_chunks(k);
    const int64_t chunk = 2 * m * n;
    Scratch sp;
    float* P = static_cast<float*>(sp.get(ctx, sizeof(float) * (size_t)S * chunk));
    tc_cgemm_partials(ctx, pa, pb, m, n, k, conj_a, TC_KCHUNK, P, m, m * n, chunk);
    tc_reduce_fp64(ctx, P, S, m, n, m, m * n, chunk, C, m, false);
    tc_check_error(ctx);
}

void mixed_unit_heff2(Ctx* ctx, const cplx* L, const cplx* W12, const cplx* R, int64_t cl,
                      int64_t cr, int d, int64_t wl, int64_t wr, const cplx* x, cplx* y) {
    MixedWork mw;
    mixed_prepare_env(ctx, mw, L, R, cl, cr, d, wl, wr);
    mixed_heff2(ctx, mw, W12, cl, cr, d, wl, wr, x, y);
    tc_check_error(ctx);
}

}  // namespace tn
