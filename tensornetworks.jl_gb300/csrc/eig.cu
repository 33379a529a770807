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

namespace tn {

namespace {

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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block (blockDim.x a multiple of 32, at most 1024); the result
// is valid in every thread.  The warp totals are added as a tree: a serial
// chain of dependent FP64 additions costs tens of cycles per link on GB300.
__device__ double block_sum(double v, double* ws) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    __syncthreads();
    if (lane == 0) ws[w] = v;
    __syncthreads();
    double t = lane < nw ? ws[lane] : 0.0;
    t = warp_sum(t);
    return __shfl_sync(0xffffffffu, t, 0);
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
// Number of eigenvalues of T below x: sign changes of the leading principal
// minors q_k = det(T[0:k, 0:k] - x I), q_k = (d_k - x) q_{k-1} - e_{k-1}^2
// q_{k-2} (Sylvester's inertia: a sign change is a negative LDL^T pivot
// q_k / q_{k-1}).  No division: two dependent FP64 operations per step, where
// the pivot form waits on a division.  Both minors are rescaled by an exact
// power of two when they leave [2^-400, 2^400]; an exact zero becomes the
// pivot -pivmin (LAPACK dstebz's guard).
__device__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e2, int t,
                           double x, double pivmin) {
    double q1 = 1.0, q0 = d[0] - x;  // q_{k-1}, q_k
    if (fabs(q0) < pivmin) q0 = -pivmin;
    int cnt = q0 < 0.0;
    for (int k = 1; k < t; ++k) {
        double q = fma(-e2[k - 1], q1, (d[k] - x) * q0);
        const long long bq = __double_as_longlong(q);
        if ((bq << 1) == 0) q = -pivmin * q0;  // +-0
        cnt += (__double_as_longlong(q) ^ __double_as_longlong(q0)) < 0;
        q1 = q0;
        q0 = q;
        // biased exponent of q_k: rescale both minors outside [2^-400, 2^400]
        const int ex = (int)((__double_as_longlong(q0) >> 52) & 0x7ff);
        if (ex > 1023 + 400) {
            q0 *= 0x1p-400;
            q1 *= 0x1p-400;
        } else if (ex < 1023 - 400 && ((__double_as_longlong(q1) >> 52) & 0x7ff) < 1023 - 400) {
            q0 *= 0x1p400;
            q1 *= 0x1p400;
        }
    }
    return cnt;
}

// The same count on FP32 copies (d, e^2): exact for a matrix within a few
// FP32 ulps of |T| of T, 64 times the FP64 issue rate on GB300.
__device__ int sturm_count_f(const float* __restrict__ d, const float* __restrict__ e2, int t,
                             float x, float pivmin) {
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int cnt = q < 0.f;
    for (int k = 1; k < t; ++k) {
        q = (d[k] - x) - __fdividef(e2[k - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        cnt += q < 0.f;
    }
    return cnt;
}

// The g-th largest eigenvalue (number t-1-g ascending) to eps * |T|:
// lam_desc[g], and lam_asc[want-1-g].  bounds = (low, high, pivmin, |T|,
// FP32 pivmin).  Four lanes share one eigenvalue: each round they count at
// the four inner points of a five-way split of the interval, so a round cuts
// it 5x (the eigenvalues' serial Sturm loops are latency bound, and four
// lanes per eigenvalue keep four times as many warps busy).  FP32 counts
// first narrow the interval to 64 FP32 ulps of |T|; it is widened by that
// much again, both ends are checked with FP64 counts (the full interval is
// restored if a check fails), and FP64 rounds finish.
constexpr int BIS_W = 4;
__global__ void bisect_kernel(const double* __restrict__ d, const double* __restrict__ e2,
                              const float* __restrict__ d32, const float* __restrict__ e2f, int t,
                              int want, const double* __restrict__ bounds,
                              double* __restrict__ lam_desc, double* __restrict__ lam_asc) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = gt / BIS_W, m = gt % BIS_W;
    const unsigned grp = 0xFu << ((threadIdx.x & 31) & ~(BIS_W - 1));
    if (g >= want) return;  // whole groups leave together (want is per group)
    const int idx = t - 1 - g;
    const double eps = 2.220446049250313e-16, pivmin = bounds[2], tn = bounds[3];
    const double abstol = eps * tn;
    double lo = bounds[0], hi = bounds[1];
    {
        const float pf = (float)bounds[4];
        float lf = __double2float_rd(lo), hf = __double2float_ru(hi);
        const float tolf = 64.f * 1.1920929e-7f * (float)tn;
        for (int it = 0; it < 64 && hf - lf > tolf; ++it) {
            const float h = (hf - lf) * (1.f / (BIS_W + 1));
            const float x = lf + h * (float)(m + 1);
            const int below = sturm_count_f(d32, e2f, t, x, pf) <= idx;  // eigenvalue >= x
            // new interval: between the last point with count <= idx and the next
            float nl = lf, nh = hf;
#pragma unroll
            for (int u = 0; u < BIS_W; ++u) {
                const int bu = __shfl_sync(grp, below, u, BIS_W);
                const float xu = lf + h * (float)(u + 1);
                if (bu) nl = xu;
                else if (nh == hf) nh = xu;
            }
            if (!(nl < nh) || (nl == lf && nh == hf)) break;
            lf = nl;
            hf = nh;
        }
        const double widen = 64.0 * 1.1920929e-7 * tn;
        const double a = fmax(lo, (double)lf - widen), b = fmin(hi, (double)hf + widen);
        const double xc = m == 0 ? a : b;
        const int ok = m < 2 ? (m == 0 ? sturm_count(d, e2, t, xc, pivmin) <= idx
                                       : sturm_count(d, e2, t, xc, pivmin) > idx)
                             : 1;
        const int oka = __shfl_sync(grp, ok, 0, BIS_W), okb = __shfl_sync(grp, ok, 1, BIS_W);
        lo = oka ? a : lo;
        hi = okb ? b : hi;
    }
    for (int it = 0; it < 128; ++it) {
        const double tol = 2.0 * eps * fmax(fabs(lo), fabs(hi)) + abstol + pivmin;
        if (hi - lo <= tol) break;
        const double h = (hi - lo) * (1.0 / (BIS_W + 1));
        const double x = lo + h * (double)(m + 1);
        const int below = sturm_count(d, e2, t, x, pivmin) <= idx;
        double nl = lo, nh = hi;
#pragma unroll
        for (int u = 0; u < BIS_W; ++u) {
            const int bu = __shfl_sync(grp, below, u, BIS_W);
            const double xu = lo + h * (double)(u + 1);
            if (bu) nl = xu;
            else if (nh == hi) nh = xu;
        }
        if (!(nl < nh) || (nl == lo && nh == hi)) break;
        lo = nl;
        hi = nh;
    }
    if (m == 0) {
        const double v = 0.5 * (lo + hi);
        lam_desc[g] = v;
        lam_asc[want - 1 - g] = v;
    }
}

// ---- 3. inverse iteration ----------------------------------------------------
__device__ __forceinline__ double hash_uniform(uint64_t a, uint64_t b) {
    // splitmix64 of (a, b) mapped to (-1, 1)
    uint64_t z = a * 0x9E3779B97F4A7C15ull + b + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

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
    const double s = shift[g];
    // pivot floor eps |T|, kept far above the denormals so that 1/tiny is finite
    const double tiny = fmax(2.220446049250313e-16 * bounds[3], 1e-290);
    const size_t W = (size_t)want;
    auto guard = [&](double x) { return fabs(x) < tiny ? (x < 0.0 ? -tiny : tiny) : x; };
    // partially pivoted LU of the tridiagonal T - s I (the scheme of LAPACK
    // dlagtf): row k of U holds (1/u1, u2, u3) at columns (k, k+1, k+2)
    double a = d[0] - s, bsup = t > 1 ? e[0] : 0.0;
    for (int k = 0; k < t - 1; ++k) {
        const double cs = e[k];          // subdiagonal entry below the pivot
        const double dn = d[k + 1] - s;  // next diagonal
        const double bn = k + 2 < t ? e[k + 1] : 0.0;
        const size_t o = (size_t)k * W + g;
        if (fabs(a) >= fabs(cs)) {  // keep row k
            const double pa = guard(a);
            const double mult = cs / pa;
            fu1[o] = 1.0 / pa;
            fu2[o] = bsup;
            fu3[o] = 0.0;
            fl[o] = mult;
            piv[o] = 0;
            a = dn - mult * bsup;
            bsup = bn;
        } else {  // interchange rows k and k+1
            const double mult = a / cs;
            fu1[o] = 1.0 / cs;
            fu2[o] = dn;
            fu3[o] = bn;
            fl[o] = mult;
            piv[o] = 1;
            a = bsup - mult * dn;
            bsup = -mult * bn;
        }
    }
    {
        const size_t o = (size_t)(t - 1) * W + g;
        fu1[o] = 1.0 / guard(a);
        fu2[o] = 0.0;
        fu3[o] = 0.0;
    }
    for (int k = 0; k < t; ++k) zw[(size_t)k * W + g] = hash_uniform((uint64_t)g + 1, (uint64_t)k);
    for (int it = 0; it < 3; ++it) {
        // forward: the row interchanges and multipliers
        double zk = zw[g];
#pragma unroll 4
        for (int k = 0; k < t - 1; ++k) {
            const size_t o = (size_t)k * W + g;
            const double mult = fl[o];
            const double zn = zw[o + W];
            if (piv[o]) {
                zw[o] = zn;
                zk = zk - mult * zn;
            } else {
                zw[o] = zk;
                zk = zn - mult * zk;
            }
        }
        zw[(size_t)(t - 1) * W + g] = zk;
        // backward: U z = rhs, then scale to unit max-norm
        double z1 = 0.0, z2 = 0.0, nrm = 0.0;  // z[k+1], z[k+2]
#pragma unroll 4
        for (int k = t - 1; k >= 0; --k) {
            const size_t o = (size_t)k * W + g;
            const double r = (zw[o] - fu2[o] * z1 - fu3[o] * z2) * fu1[o];
            zw[o] = r;
            z2 = z1;
            z1 = r;
            nrm = fmax(nrm, fabs(r));
        }
        const double inv = nrm > 0.0 ? 1.0 / nrm : 1.0;
        for (int k = 0; k < t; ++k) zw[(size_t)k * W + g] *= inv;
    }
    double s2 = 0.0;
    for (int k = 0; k < t; ++k) {
        const double v = zw[(size_t)k * W + g];
        s2 += v * v;
    }
    const double inv = s2 > 0.0 ? 1.0 / sqrt(s2) : 0.0;
    double* z = Z + (size_t)g * t;
    for (int k = 0; k < t; ++k) z[k] = zw[(size_t)k * W + g] * inv;
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
    const int64_t c = k - 1 - w;  // column c costs c+1 reflectors: the heaviest start first
    double* q = Q + c * t;
    for (int64_t i = lane; i < t; i += 32) q[i] = (i == c) ? 1.0 : 0.0;
    __syncwarp();
    for (int64_t j = c; j >= 0; --j) {
        const double tau = qtau[j];
        if (tau == 0.0) continue;
        const double* v = Zr + j * t;  // v[j] = 1 implicit
        double s0 = (lane == 0) ? q[j] : 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int64_t i = j + 1 + lane;
        for (; i + 96 < t; i += 128) {
            s0 = fma(v[i], q[i], s0);
            s1 = fma(v[i + 32], q[i + 32], s1);
            s2 = fma(v[i + 64], q[i + 64], s2);
            s3 = fma(v[i + 96], q[i + 96], s3);
        }
        for (; i < t; i += 32) s0 = fma(v[i], q[i], s0);
        double s = warp_sum((s0 + s1) + (s2 + s3));
        s = __shfl_sync(0xffffffffu, s, 0) * tau;
        for (int64_t i = j + lane; i < t; i += 32) q[i] -= s * (i == j ? 1.0 : v[i]);
        __syncwarp();
    }
    // R's diagonal carries the sign that maps the input column onto Q's column
    if (rdiag[c] < 0.0)
        for (int64_t i = lane; i < t; i += 32) q[i] = -q[i];
}

// ---- 5. back-transformation ----------------------------------------------------
// Reflector j of step 1: v_j[j+1] = 1, v_j[j+2:] = A[j+2:, j], zero above.
__device__ __forceinline__ cplx refl(const cplx* __restrict__ A, int64_t n, int64_t j, int64_t i) {
    return i == j + 1 ? cmk(1, 0) : (i > j + 1 ? A[i + n * j] : cmk(0, 0));
}

constexpr int BT_G = 4;  // reflectors per compact-WY group

// Group q covers reflectors a = q*BT_G .. a+BT_G-1 (those < n-1):
// H_a H_{a+1} ... = I - V T V^H with T upper triangular (LAPACK zlarft,
// forward, columnwise): T[r][r] = tau_r, T[0:r, r] = -tau_r T[0:r, 0:r] V^H v_r.
// One warp per group; T is stored column-major, 16 entries per group.
__global__ void wy_factor_kernel(const cplx* __restrict__ A, int64_t n, const cplx* __restrict__ tau,
                                 int64_t ngroups, cplx* __restrict__ Tg) {
    const int lane = threadIdx.x & 31;
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= ngroups) return;
    const int64_t a = q * BT_G;
    const int nr = (int)min((int64_t)BT_G, (n - 1) - a);
    // S[c][r] = v_c^H v_r for c < r
    double sre[BT_G][BT_G], sim[BT_G][BT_G];
#pragma unroll
    for (int c = 0; c < BT_G; ++c)
#pragma unroll
        for (int r = 0; r < BT_G; ++r) sre[c][r] = sim[c][r] = 0.0;
    for (int64_t i = a + 1 + lane; i < n; i += 32) {
        cplx v[BT_G];
#pragma unroll
        for (int r = 0; r < BT_G; ++r) v[r] = r < nr ? refl(A, n, a + r, i) : cmk(0, 0);
#pragma unroll
        for (int c = 0; c < BT_G; ++c)
#pragma unroll
            for (int r = c + 1; r < BT_G; ++r) {
                sre[c][r] += v[c].x * v[r].x + v[c].y * v[r].y;
                sim[c][r] += v[c].x * v[r].y - v[c].y * v[r].x;
            }
    }
#pragma unroll
    for (int c = 0; c < BT_G; ++c)
#pragma unroll
        for (int r = c + 1; r < BT_G; ++r) {
            sre[c][r] = warp_sum(sre[c][r]);
            sim[c][r] = warp_sum(sim[c][r]);
        }
    if (lane != 0) return;
    cplx T[BT_G][BT_G];
#pragma unroll
    for (int c = 0; c < BT_G; ++c)
#pragma unroll
        for (int r = 0; r < BT_G; ++r) T[c][r] = cmk(0, 0);
    for (int r = 0; r < nr; ++r) {
        const cplx tr = tau[a + r];
        T[r][r] = tr;
        cplx z[BT_G];
        for (int c = 0; c < r; ++c) z[c] = cmul(cmk(-tr.x, -tr.y), cmk(sre[c][r], sim[c][r]));
        for (int c = 0; c < r; ++c) {  // T[0:r, r] = T[0:r, 0:r] z
            cplx acc = cmk(0, 0);
            for (int u = c; u < r; ++u) acc = cfma(T[c][u], z[u], acc);
            T[c][r] = acc;
        }
    }
    for (int c = 0; c < BT_G; ++c)
        for (int r = 0; r < BT_G; ++r) Tg[q * BT_G * BT_G + c + BT_G * r] = T[c][r];
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
    cplx* x = X + c * n;
    const double* z = Z + c * n;
    for (int64_t i = lane; i < n; i += 32) x[i] = cmk(z[i], 0.0);
    __syncwarp();
    for (int64_t q = ngroups - 1; q >= 0; --q) {
        const int64_t a = q * BT_G;
        const int nr = (int)min((int64_t)BT_G, (n - 1) - a);
        double sr[BT_G], si[BT_G];
#pragma unroll
        for (int r = 0; r < BT_G; ++r) sr[r] = si[r] = 0.0;
        for (int64_t i = a + 1 + lane; i < n; i += 32) {
            const cplx xi = x[i];
#pragma unroll
            for (int r = 0; r < BT_G; ++r) {
                if (r < nr) {
                    const cplx v = refl(A, n, a + r, i);
                    sr[r] += v.x * xi.x + v.y * xi.y;  // conj(v) x
                    si[r] += v.x * xi.y - v.y * xi.x;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < BT_G; ++r) {
            sr[r] = __shfl_sync(0xffffffffu, warp_sum(sr[r]), 0);
            si[r] = __shfl_sync(0xffffffffu, warp_sum(si[r]), 0);
        }
        // coefficients u = T s
        const cplx* T = Tg + q * BT_G * BT_G;
        cplx u[BT_G];
#pragma unroll
        for (int r = 0; r < BT_G; ++r) {
            cplx acc = cmk(0, 0);
#pragma unroll
            for (int v = r; v < BT_G; ++v) acc = cfma(T[r + BT_G * v], cmk(sr[v], si[v]), acc);
            u[r] = acc;
        }
        for (int64_t i = a + 1 + lane; i < n; i += 32) {
            cplx xi = x[i];
#pragma unroll
            for (int r = 0; r < BT_G; ++r)
                if (r < nr) xi = csub(xi, cmul(u[r], refl(A, n, a + r, i)));
            x[i] = xi;
        }
        __syncwarp();
    }
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
    const double sep = 10.0 * 2.220446049250313e-16 * fmax(bounds[3], 1e-290);
    double prev = 0.0;
    for (int g = 0; g < want; ++g) {
        double s = lam[g];
        if (g > 0 && s > prev - sep) s = prev - sep;
        shift[g] = s;
        prev = s;
    }
}

// Gershgorin interval, pivot guards and |T| (bounds[0..4]), and FP32 copies
// of d and e^2 for the bisection's first phase; one block.
__global__ void tri_bounds_kernel(const double* __restrict__ d, const double* __restrict__ e,
                                  int t, double* __restrict__ out, float* __restrict__ d32,
                                  float* __restrict__ e2f, double* __restrict__ e2) {
    __shared__ double slo[EIG_T], shi[EIG_T], sm[EIG_T];
    double lo = 1e300, hi = -1e300, me = 0.0;
    for (int k = threadIdx.x; k < t; k += blockDim.x) {
        const double r = (k > 0 ? fabs(e[k - 1]) : 0.0) + (k + 1 < t ? fabs(e[k]) : 0.0);
        lo = fmin(lo, d[k] - r);
        hi = fmax(hi, d[k] + r);
        d32[k] = (float)d[k];
        if (k + 1 < t) {
            me = fmax(me, e[k] * e[k]);
            e2f[k] = (float)(e[k] * e[k]);
            e2[k] = e[k] * e[k];
        }
    }
    slo[threadIdx.x] = lo;
    shi[threadIdx.x] = hi;
    sm[threadIdx.x] = me;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            slo[threadIdx.x] = fmin(slo[threadIdx.x], slo[threadIdx.x + s]);
            shi[threadIdx.x] = fmax(shi[threadIdx.x], shi[threadIdx.x + s]);
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double eps = 2.220446049250313e-16;
        const double nrm = fmax(fabs(slo[0]), fabs(shi[0]));
        const double w = 2.0 * eps * nrm * t + 1e-300;
        out[0] = slo[0] - w;
        out[1] = shi[0] + w;
        out[2] = fmax(2.2250738585072014e-308 * fmax(1.0, sm[0]), 1e-300);  // pivmin
        out[3] = nrm;
        out[4] = 1.1754944e-38 * fmax(1.0, fmin(sm[0], 1e30));  // FP32 pivmin
    }
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
