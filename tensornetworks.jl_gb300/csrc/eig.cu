// Hermitian eigensolver of the truncated split, FP64, on the device.
//
// The reference's svd(x, idx; cutoff, maxdim, mindim) (src/tensors.jl:168-227)
// calls LAPACK gesdd on the grouped tensor.  This library forms the Gram
// matrix of the isometric side instead and needs its top eigenpairs; this
// file computes them with five hand-written steps:
//
//   1. Householder reduction G = Q T Q^H to a real symmetric tridiagonal T.
//      One persistent cooperative kernel, one block per SM.  At step j the
//      rows of the unreduced block are re-partitioned over the blocks; each
//      block applies the previous step's rank-2 update to its rows and, in the
//      same pass, accumulates its rows of the Hermitian matvec of this step,
//      so every unreduced element is read and written once per step.  Every
//      block recomputes the Householder vector of column j itself; one grid
//      barrier per step (a bounded spin on the global timer) publishes the
//      matvec.
//   2. Bisection with Sturm counts (LDL^T pivots) for the wanted eigenvalues,
//      one thread per eigenvalue.
//   3. Inverse iteration with a partially pivoted tridiagonal LU, one thread
//      per eigenvector, shifts of a cluster pulled apart by a few ulps of |T|.
//   4. Householder QR of those vectors in descending-eigenvalue order: every
//      vector is orthogonalised against all vectors of larger eigenvalue,
//      which makes degenerate multiplets and clusters orthonormal, and the
//      explicit orthonormal factor replaces the vectors.
//   5. Back-transformation X = Q Z by the reflectors of step 1, one warp per
//      column of X.
//
// GB300 issues FP64 at two FMAs per clock per SM, so steps 1 and 5 (O(n^3)
// and O(n^2 k)) bound the time; the rest is latency.
#include <cmath>

#include "common.cuh"
#include "eig_dev.cuh"

namespace tn {

namespace {

using namespace eigdev;

constexpr uint64_t EIG_WAIT_NS = 2000000000ull;  // 2 s bound on a barrier wait
constexpr int EIG_T = 256;                      // threads per block
constexpr int64_t EIG_MAXN = 4096;              // vectors of step 1 live in shared memory

__device__ __forceinline__ uint64_t gclock() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Barrier {
    unsigned* count;
    unsigned* gen;
    int* err;
};

// Grid-wide barrier of a cooperative launch.  `passed` (thread 0's copy) is
// the number of barriers this block has completed.  A wait is bounded by the
// global timer; when it runs out, or another block reported that, the error
// flag is set and every thread gets false: the kernel then returns.
__device__ bool grid_barrier(const Barrier& b, unsigned& passed) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned g = passed;
        if (atomicAdd(b.count, 1u) == gridDim.x - 1) {
            atomicExch(b.count, 0u);
            __threadfence();
            atomicExch(b.gen, g + 1u);
        } else {
            const uint64_t t0 = gclock();
            while (*(volatile unsigned*)b.gen == g) {
                if (*(volatile int*)b.err) {
                    ok = 0;
                    break;
                }
                if (gclock() - t0 > EIG_WAIT_NS) {
                    atomicExch(b.err, 1);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        passed = g + 1u;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---- 1. tridiagonal reduction ------------------------------------------------
struct TrdArgs {
    cplx* A;      // n x n Hermitian, both triangles; reflector j in A[j+2:, j] on exit
    int64_t n;
    double* d;    // n diagonal of T
    double* e;    // n-1 off-diagonal of T
    cplx* tau;    // n-1 reflector scalars (H_j = I - tau_j v_j v_j^H, v_j[j+1] = 1)
    cplx* y;      // n matvec of the current step
    cplx* dpart;  // gridDim.x partial dot products
    Barrier bar;
};

constexpr int TRD_PER = (int)(EIG_MAXN / EIG_T);  // column entries per thread

__global__ void __launch_bounds__(EIG_T) hetrd_kernel(TrdArgs p) {
    extern __shared__ cplx sv[];
    const int64_t n = p.n;
    cplx* vp = sv;           // v of the previous step (its update is pending)
    cplx* wp = sv + n;       // w of the previous step
    cplx* vc = sv + 2 * n;   // v of this step
    cplx* red = sv + 3 * n;  // per-thread partial row sums
    __shared__ double ws[32];
    __shared__ cplx s_c[3];
    const int T = blockDim.x, tid = threadIdx.x;
    const int B = gridDim.x, b = blockIdx.x;
    unsigned passed = 0;
    bool pend = false;
    // column 0 and the norm of x[1:]
    double nrm2 = 0.0;
    for (int64_t i = tid; i < n; i += T) {
        const cplx a = __ldcg(p.A + i);
        vc[i] = a;
        if (i >= 2) nrm2 += a.x * a.x + a.y * a.y;
    }
    nrm2 = block_sum(nrm2, ws);  // synchronises: vc visible
    for (int64_t j = 0; j + 1 < n; ++j) {
        // vc[j] = diagonal, vc[j+1:] = x (pending update applied); nrm2 = |x[1:]|^2
        if (tid == 0) {
            // reflector with H^H x = beta e_1, beta real (LAPACK zlarfg's convention)
            const cplx al = vc[j + 1];
            cplx tau = cmk(0, 0), scale = cmk(0, 0);
            double beta = al.x;
            if (nrm2 != 0.0 || al.y != 0.0) {
                beta = -copysign(sqrt(al.x * al.x + al.y * al.y + nrm2), al.x);
                const double rb = 1.0 / beta;
                tau = cmk((beta - al.x) * rb, -al.y * rb);
                // 1 / (alpha - beta); |alpha - beta| >= |beta| > 0 by the sign choice
                const double ur = al.x - beta, ui = al.y, rd = 1.0 / (ur * ur + ui * ui);
                scale = cmk(ur * rd, -ui * rd);
            }
            s_c[0] = tau;
            s_c[1] = scale;
            if (b == 0) {
                p.d[j] = vc[j].x;
                p.e[j] = beta;
                p.tau[j] = tau;
            }
        }
        __syncthreads();
        const cplx tau = s_c[0], scale = s_c[1];
        for (int64_t i = j + 2 + tid; i < n; i += T) vc[i] = cmul(vc[i], scale);
        if (tid == 0) vc[j + 1] = cmk(1, 0);
        __syncthreads();
        // fused pass over this block's rows of the unreduced block (rows and
        // columns j+1..n-1): pending rank-2 update, then y = tau * A v
        const int64_t m = n - j - 1;
        const int64_t c = (m + B - 1) / B;
        const int64_t r0 = j + 1 + (int64_t)b * c, r1 = min(r0 + c, n);
        double dre = 0.0, dim = 0.0;
        if (r0 < r1) {
            const int cr = (int)(r1 - r0);
            const int cs = T / cr;  // threads per row (cr <= T since n <= EIG_MAXN)
            double ar = 0.0, ai = 0.0;
            if (tid < cs * cr) {
                const int64_t i = r0 + tid % cr;
                const cplx vpi = pend ? vp[i] : cmk(0, 0), wpi = pend ? wp[i] : cmk(0, 0);
                int64_t l = j + 1 + tid / cr;
                // four columns per round: the loads are issued before the math
                for (; l + 3 * cs < n; l += 4 * cs) {
                    cplx a4[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) a4[u] = __ldcg(p.A + i + n * (l + u * cs));
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int64_t lu = l + u * cs;
                        cplx a = a4[u];
                        if (pend) {
                            // a -= w_i conj(v_l) + v_i conj(w_l)
                            const cplx vl = vp[lu], wl = wp[lu];
                            a.x = fma(-wpi.x, vl.x, fma(-wpi.y, vl.y, fma(-vpi.x, wl.x, fma(-vpi.y, wl.y, a.x))));
                            a.y = fma(-wpi.y, vl.x, fma(wpi.x, vl.y, fma(-vpi.y, wl.x, fma(vpi.x, wl.y, a.y))));
                            p.A[i + n * lu] = a;
                        }
                        const cplx x = vc[lu];
                        ar = fma(a.x, x.x, fma(-a.y, x.y, ar));
                        ai = fma(a.x, x.y, fma(a.y, x.x, ai));
                    }
                }
                for (; l < n; l += cs) {
                    cplx a = __ldcg(p.A + i + n * l);
                    if (pend) {
                        const cplx vl = vp[l], wl = wp[l];
                        a.x = fma(-wpi.x, vl.x, fma(-wpi.y, vl.y, fma(-vpi.x, wl.x, fma(-vpi.y, wl.y, a.x))));
                        a.y = fma(-wpi.y, vl.x, fma(wpi.x, vl.y, fma(-vpi.y, wl.x, fma(vpi.x, wl.y, a.y))));
                        p.A[i + n * l] = a;
                    }
                    const cplx x = vc[l];
                    ar = fma(a.x, x.x, fma(-a.y, x.y, ar));
                    ai = fma(a.x, x.y, fma(a.y, x.x, ai));
                }
            }
            red[tid] = cmk(ar, ai);
            __syncthreads();
            // row sums over the cs column groups (red[row + q*cr]) as a tree
            int span = 1;
            while (span < cs) span <<= 1;
            for (int h = span >> 1; h > 0; h >>= 1) {
                if (tid < h * cr && tid + h * cr < cs * cr) red[tid] = cadd(red[tid], red[tid + h * cr]);
                __syncthreads();
            }
            if (tid < cr) {
                const cplx yi = cmul(tau, red[tid]);
                p.y[r0 + tid] = yi;
                const cplx t = cmul(cconj(yi), vc[r0 + tid]);  // y^H v
                dre = t.x;
                dim = t.y;
            }
        }
        dre = block_sum(dre, ws);
        dim = block_sum(dim, ws);
        if (tid == 0) p.dpart[b] = cmk(dre, dim);
        if (!grid_barrier(p.bar, passed)) return;
        // One round of loads after the barrier: the partial dots, y and the
        // next column as the fused pass left it (its pending update is this
        // step's, applied below from registers).
        const cplx q = tid < B ? __ldcg(p.dpart + tid) : cmk(0, 0);
        cplx yv[TRD_PER], cv[TRD_PER];
#pragma unroll
        for (int u = 0; u < TRD_PER; ++u) {
            const int64_t i = j + 1 + tid + (int64_t)u * T;
            if (i < n) {
                yv[u] = __ldcg(p.y + i);
                cv[u] = __ldcg(p.A + i + n * (j + 1));
            }
        }
        // w = y - (tau/2) (y^H v) v, the same in every block (fixed order)
        const double sre = block_sum(q.x, ws), sim = block_sum(q.y, ws);
        const cplx al2 = cmul(cmk(-0.5 * tau.x, -0.5 * tau.y), cmk(sre, sim));
#pragma unroll
        for (int u = 0; u < TRD_PER; ++u) {
            const int64_t i = j + 1 + tid + (int64_t)u * T;
            if (i < n) {
                yv[u] = cfma(al2, vc[i], yv[u]);  // w_i
                wp[i] = yv[u];
            }
        }
        // block 0 keeps the reflector below the subdiagonal of column j
        if (b == 0)
            for (int64_t i = j + 2 + tid; i < n; i += T) p.A[i + n * j] = vc[i];
        cplx* t = vp;  // v_j becomes the pending vector; its buffer is free
        vp = vc;
        vc = t;
        pend = true;
        __syncthreads();  // w_j complete
        // column j+1 with this step's update: a_i - (w_i conj(v_{j+1}) + v_i conj(w_{j+1})),
        // v_{j+1} = 1 (the first reflector entry)
        const cplx wj1 = wp[j + 1];
        nrm2 = 0.0;
#pragma unroll
        for (int u = 0; u < TRD_PER; ++u) {
            const int64_t i = j + 1 + tid + (int64_t)u * T;
            if (i < n) {
                const cplx vi = vp[i];
                cplx a = cv[u];
                a.x -= yv[u].x + (vi.x * wj1.x + vi.y * wj1.y);
                a.y -= yv[u].y + (vi.y * wj1.x - vi.x * wj1.y);
                vc[i] = a;
                if (i >= j + 3) nrm2 += a.x * a.x + a.y * a.y;
            }
        }
        nrm2 = block_sum(nrm2, ws);  // synchronises: vc visible
    }
    if (b == 0 && tid == 0) p.d[n - 1] = vc[n - 1].x;
}

// ---- 2. bisection ------------------------------------------------------------
// (Sturm counts: eig_dev.cuh)

// The g-th largest eigenvalue (number t-1-g ascending) to eps * |T|:
// lam_desc[g], and lam_asc[want-1-g].  bounds = (low, high, pivmin, |T|,
// FP32 pivmin).  Four lanes share one eigenvalue: each round they count at
// the four inner points of a five-way split of the interval, so a round cuts
// it 5x (the eigenvalues' serial Sturm loops are latency bound, and four
// lanes per eigenvalue keep four times as many warps busy).  FP32 counts
// first narrow the interval to 64 FP32 ulps of |T|; it is widened by that
// much again, both ends are checked with FP64 counts (the full interval is
// restored if a check fails), and FP64 rounds finish.
__global__ void bisect_kernel(const double* __restrict__ d, const double* __restrict__ e2,
                              const float* __restrict__ d32, const float* __restrict__ e2f, int t,
                              int want, const double* __restrict__ bounds,
                              double* __restrict__ lam_desc, double* __restrict__ lam_asc) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = gt / BIS_W, m = gt % BIS_W;
    const unsigned grp = 0xFu << ((threadIdx.x & 31) & ~(BIS_W - 1));
    if (g >= want) return;  // whole groups leave together (want is per group)
    bisect_group(g, m, grp, d, e2, d32, e2f, t, want, bounds, lam_desc, lam_asc);
}

// ---- 3. inverse iteration ----------------------------------------------------
// Vector g solves (T - shift_g) z = b three times from a pseudo-random b.
// The factors and the working vector are stored [k][want] so that the
// threads of a warp touch adjacent words; the normalised vector is written
// column-major into Z (t x want).
__global__ void stein_kernel(const double* __restrict__ d, const double* __restrict__ e, int t,
                             int want, const double* __restrict__ shift,
                             const double* __restrict__ bounds, double* __restrict__ fu1,
                             double* __restrict__ fu2, double* __restrict__ fu3,
                             double* __restrict__ fl, unsigned char* __restrict__ piv,
                             double* __restrict__ zw, double* __restrict__ Z) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= want) return;
    stein_vector(g, d, e, t, want, shift, bounds, fu1, fu2, fu3, fl, piv, zw, Z);
}

// ---- 4. Householder QR of the eigenvector block --------------------------------
// Z is t x k column-major (descending eigenvalues).  Column c is owned by
// block c % gridDim.x.  At step j every block rebuilds reflector j from
// column j (finished by its owner at step j-1) and applies it to its columns
// past j.  On exit column j holds the reflector (v_j[j] = 1 implicit) and
// rdiag[j] the diagonal of R.
__global__ void __launch_bounds__(EIG_T) qr_kernel(double* __restrict__ Z, int64_t t, int64_t k,
                                                  double* __restrict__ qtau,
                                                  double* __restrict__ rdiag, Barrier bar) {
    extern __shared__ double sq[];  // reflector, t entries
    __shared__ double ws[32];
    __shared__ double s_tau, s_scale;
    const int T = blockDim.x, tid = threadIdx.x, B = gridDim.x, b = blockIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    unsigned passed = 0;
    for (int64_t j = 0; j < k; ++j) {
        if (j > 0 && !grid_barrier(bar, passed)) return;
        const double* zj = Z + j * t;
        double nrm2 = 0.0;
#pragma unroll 4
        for (int64_t i = j + tid; i < t; i += T) {
            const double v = __ldcg(zj + i);
            sq[i] = v;
            if (i > j) nrm2 += v * v;
        }
        nrm2 = block_sum(nrm2, ws);
        if (tid == 0) {
            const double al = sq[j];
            double tau = 0.0, beta = al, scale = 0.0;
            if (nrm2 != 0.0) {
                beta = -copysign(sqrt(al * al + nrm2), al);
                tau = (beta - al) / beta;
                scale = 1.0 / (al - beta);
            }
            s_tau = tau;
            s_scale = scale;
            sq[j] = 1.0;
            if (j % B == b) {
                qtau[j] = tau;
                rdiag[j] = beta;
            }
        }
        __syncthreads();
        const double scale = s_scale, tau = s_tau;
        for (int64_t i = j + 1 + tid; i < t; i += T) sq[i] *= scale;
        __syncthreads();
        if (j % B == b)  // the owner stores the reflector in place of column j
            for (int64_t i = j + 1 + tid; i < t; i += T) Z[i + j * t] = sq[i];
        if (tau == 0.0) continue;
        // apply H_j = I - tau v v^T to this block's columns c > j, one warp per column
        for (int64_t c = j + 1 + ((b - (j + 1) % B) + B) % B + (int64_t)warp * B; c < k;
             c += (int64_t)nw * B) {
            double* zc = Z + c * t;
            // four accumulators: the dot product is not one dependent FP64 chain
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int64_t i = j + lane;
            for (; i + 96 < t; i += 128) {
                s0 = fma(sq[i], zc[i], s0);
                s1 = fma(sq[i + 32], zc[i + 32], s1);
                s2 = fma(sq[i + 64], zc[i + 64], s2);
                s3 = fma(sq[i + 96], zc[i + 96], s3);
            }
            for (; i < t; i += 32) s0 = fma(sq[i], zc[i], s0);
            double s = warp_sum((s0 + s1) + (s2 + s3));
            s = __shfl_sync(0xffffffffu, s, 0) * tau;
#pragma unroll 4
            for (int64_t i = j + lane; i < t; i += 32) zc[i] -= s * sq[i];
        }
    }
}

// Q's first k columns from the reflectors of qr_kernel: column c is
// H_0 H_1 ... H_c e_c, signed so that it follows the input vector
// (sign of rdiag[c]); one warp per column, written to Q (t x k, column-major).
__global__ void qr_form_kernel(const double* __restrict__ Zr, int64_t t, int64_t k,
                               const double* __restrict__ qtau, const double* __restrict__ rdiag,
                               double* __restrict__ Q) {
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= k) return;
    qr_form_column(w, lane, Zr, t, k, qtau, rdiag, Q);
}

// ---- 5. back-transformation ----------------------------------------------------

// Group q covers reflectors a = q*BT_G .. a+BT_G-1 (those < n-1):
// H_a H_{a+1} ... = I - V T V^H with T upper triangular (LAPACK zlarft,
// forward, columnwise): T[r][r] = tau_r, T[0:r, r] = -tau_r T[0:r, 0:r] V^H v_r.
// One warp per group; T is stored column-major, 16 entries per group.
__global__ void wy_factor_kernel(const cplx* __restrict__ A, int64_t n, const cplx* __restrict__ tau,
                                 int64_t ngroups, cplx* __restrict__ Tg) {
    const int lane = threadIdx.x & 31;
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= ngroups) return;
    wy_group(q, lane, A, n, tau, Tg);
}

// X[:, c] = H_0 ... H_{n-2} [z_c] with z_c real (n rows), one warp per column,
// the reflectors applied a group at a time from the last group to the first:
// x <- x - V (T (V^H x)), the four dot products in one pass over x.
__global__ void backtransform_kernel(const cplx* __restrict__ A, int64_t n,
                                     const cplx* __restrict__ Tg, int64_t ngroups,
                                     const double* __restrict__ Z, int64_t k,
                                     cplx* __restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= k) return;
    bt_column(c, lane, A, n, Tg, ngroups, Z, X);
}

// Upper triangle from the lower one, and a real diagonal.
__global__ void hermitian_fill_kernel(cplx* __restrict__ A, int64_t n) {
    const int64_t total = n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % n, l = e / n;
        if (i < l) A[i + n * l] = cconj(A[l + n * i]);
        else if (i == l) A[i + n * l].y = 0.0;
    }
}

// Shifts for inverse iteration: descending eigenvalues pulled apart so that
// consecutive shifts differ by at least sep (LAPACK dstein's perturbation).
__global__ void separate_shifts_kernel(const double* __restrict__ lam, int want,
                                       const double* __restrict__ bounds,
                                       double* __restrict__ shift) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    separate_shifts_serial(lam, want, bounds, shift);
}

// Gershgorin interval, pivot guards and |T| (bounds[0..4]), and FP32 copies
// of d and e^2 for the bisection's first phase; one block.
__global__ void tri_bounds_kernel(const double* __restrict__ d, const double* __restrict__ e,
                                  int t, double* __restrict__ out, float* __restrict__ d32,
                                  float* __restrict__ e2f, double* __restrict__ e2) {
    __shared__ double slo[EIG_T], shi[EIG_T], sm[EIG_T];
    tri_bounds_block(d, e, t, out, d32, e2f, e2, slo, shi, sm);
}

inline unsigned nblk(int64_t n, int threads) { return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads); }

}  // namespace

// Top `want` eigenpairs of the Hermitian n x n matrix G (lower triangle
// read; G is destroyed).  lam_asc[want-1-g] and X[:, g] (n x want,
// column-major) hold the g-th largest eigenvalue and its eigenvector.
// Everything runs on the context's stream without host synchronisation; a
// grid barrier that timed out leaves a nonzero word at ctx->eig_err(),
// which the caller reads with its next synchronisation (keep_rule's dinfo).
void eig_top(Ctx* ctx, cplx* G, int64_t n, int64_t want, double* lam_asc, cplx* X) {
    TN_REQUIRE(n >= 1 && want >= 1 && want <= n, "eig_top: bad sizes");
    TN_REQUIRE(n <= EIG_MAXN, "eig_top: matrix order above 4096");
    // blocks of step 1: about one per 8 rows below n = 256 (cheaper barriers),
    // every SM above (the FP64 issue rate of all SMs)
    const unsigned B1 = (unsigned)std::min<int64_t>(
        ctx->sm_count, std::max<int64_t>(1, n >= 256 ? ctx->sm_count : n / 8));
    TN_REQUIRE((n - 1 + B1 - 1) / B1 <= EIG_T, "eig_top: too few blocks for the row partition");
    ProfScope ps(ctx, 2, 16.0 / 3.0 * n * n * n + 8.0 * n * n * want, 16.0 * n * n);
    const size_t nd = (size_t)n, nw = nd * (size_t)want;
    // scratch layout, 256-byte aligned pieces
    const size_t sizes[] = {sizeof(double) * nd,     sizeof(double) * nd,    sizeof(cplx) * nd,
                            sizeof(cplx) * nd,       sizeof(cplx) * B1,      sizeof(double) * 8,
                            sizeof(double) * want,   sizeof(double) * want,  sizeof(double) * want,
                            sizeof(double) * want,   sizeof(double) * nw,    sizeof(double) * nw,
                            sizeof(double) * nw,     sizeof(double) * nw,    sizeof(double) * nw,
                            sizeof(double) * nw,     sizeof(double) * nw,    nw,
                            sizeof(float) * nd,      sizeof(float) * nd,
                            sizeof(cplx) * (nd / BT_G + 1) * BT_G * BT_G,
                            sizeof(double) * nd};
    constexpr int NP = sizeof(sizes) / sizeof(sizes[0]);
    size_t total = 0;
    for (size_t b : sizes) total += (b + 255) / 256 * 256;
    char* base = static_cast<char*>(ctx->s_eig.get(ctx, total));
    void* piece[NP];
    for (int i = 0; i < NP; ++i) {
        piece[i] = base;
        base += (sizes[i] + 255) / 256 * 256;
    }
    double* d = static_cast<double*>(piece[0]);
    double* e = static_cast<double*>(piece[1]);
    cplx* tau = static_cast<cplx*>(piece[2]);
    cplx* y = static_cast<cplx*>(piece[3]);
    cplx* dpart = static_cast<cplx*>(piece[4]);
    double* bounds = static_cast<double*>(piece[5]);
    double* shift = static_cast<double*>(piece[6]);
    double* qtau = static_cast<double*>(piece[7]);
    double* rdiag = static_cast<double*>(piece[8]);
    double* lam_desc = static_cast<double*>(piece[9]);
    double* Z = static_cast<double*>(piece[10]);
    double* Q = static_cast<double*>(piece[11]);
    double* f1 = static_cast<double*>(piece[12]);
    double* f2 = static_cast<double*>(piece[13]);
    double* f3 = static_cast<double*>(piece[14]);
    double* fl = static_cast<double*>(piece[15]);
    double* zw = static_cast<double*>(piece[16]);
    unsigned char* pv = static_cast<unsigned char*>(piece[17]);
    float* d32 = static_cast<float*>(piece[18]);
    float* e2f = static_cast<float*>(piece[19]);
    cplx* Tw = static_cast<cplx*>(piece[20]);
    double* e2 = static_cast<double*>(piece[21]);
    unsigned* bw = ctx->d_bar;
    Barrier bar{bw, bw + 1, reinterpret_cast<int*>(bw + 2)};
    TN_CHECK_CUDA(cudaMemsetAsync(bw, 0, 3 * sizeof(unsigned), ctx->stream));

    hermitian_fill_kernel<<<std::min<unsigned>(nblk(n * n, 256), (unsigned)ctx->sm_count * 8), 256,
                            0, ctx->stream>>>(G, n);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    if (n >= 2) {
        const size_t smem = sizeof(cplx) * (3 * nd + EIG_T);
        // the limit for the largest order, the same from every thread: host
        // threads that solve concurrently (QJMC workers) never lower it
        TN_CHECK_CUDA(cudaFuncSetAttribute(hetrd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(cplx) * (3 * EIG_MAXN + EIG_T))));
        int occ = 0;
        TN_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, hetrd_kernel, EIG_T, smem));
        TN_REQUIRE(occ >= 1, "eig_top: tridiagonal kernel does not fit on an SM");
        TrdArgs a{G, n, d, e, tau, y, dpart, bar};
        void* args[] = {&a};
        TN_CHECK_CUDA(cudaLaunchCooperativeKernel((void*)hetrd_kernel, dim3(B1), dim3(EIG_T), args,
                                                  smem, ctx->stream));
        ctx->count();
    } else {
        TN_CHECK_CUDA(cudaMemcpyAsync(d, G, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    const int t = (int)n;
    tri_bounds_kernel<<<1, EIG_T, 0, ctx->stream>>>(d, e, t, bounds, d32, e2f, e2);
    ctx->count();
    // one warp (eight eigenvalues) per block: the serial Sturm loops spread over the SMs
    bisect_kernel<<<nblk(want * BIS_W, 32), 32, 0, ctx->stream>>>(d, e2, d32, e2f, t, (int)want,
                                                                 bounds, lam_desc, lam_asc);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    separate_shifts_kernel<<<1, 32, 0, ctx->stream>>>(lam_desc, (int)want, bounds, shift);
    ctx->count();
    stein_kernel<<<nblk(want, 32), 32, 0, ctx->stream>>>(d, e, t, (int)want, shift, bounds, f1, f2,
                                                        f3, fl, pv, zw, Z);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    if (want > 1) {
        const unsigned B4 = (unsigned)std::min<int64_t>(ctx->sm_count, want);
        const size_t smem = sizeof(double) * nd;  // <= 32 KiB for n <= 4096
        TN_CHECK_CUDA(cudaMemsetAsync(bw, 0, 2 * sizeof(unsigned), ctx->stream));  // keep the error word
        int64_t tt = n, kk = want;
        void* args[] = {&Z, &tt, &kk, &qtau, &rdiag, &bar};
        TN_CHECK_CUDA(cudaLaunchCooperativeKernel((void*)qr_kernel, dim3(B4), dim3(EIG_T), args, smem,
                                                  ctx->stream));
        ctx->count();
        qr_form_kernel<<<nblk(want * 32, 128), 128, 0, ctx->stream>>>(Z, n, want, qtau, rdiag, Q);
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    } else {
        TN_CHECK_CUDA(cudaMemcpyAsync(Q, Z, sizeof(double) * nd, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    const int64_t ngroups = (n - 1 + BT_G - 1) / BT_G;
    if (ngroups > 0) {
        wy_factor_kernel<<<nblk(ngroups * 32, 128), 128, 0, ctx->stream>>>(G, n, tau, ngroups, Tw);
        ctx->count();
    }
    // seven warps per block: about one block per SM at the bulk DMRG shape
    backtransform_kernel<<<nblk(want * 32, 224), 224, 0, ctx->stream>>>(G, n, Tw, ngroups, Q, want,
                                                                        X);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

}  // namespace tn
