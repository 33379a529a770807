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

// Sum over the block; the result is valid in every thread.
__device__ double block_sum(double v, double* ws) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) ws[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
    return t;
}

__device__ __forceinline__ cplx crecip(cplx a) {
    // 1 / a with the larger component as the divisor (Smith's method)
    if (fabs(a.x) >= fabs(a.y)) {
        const double r = a.y / a.x, den = a.x + a.y * r;
        return cmk(1.0 / den, -r / den);
    }
    const double r = a.x / a.y, den = a.x * r + a.y;
    return cmk(r / den, -1.0 / den);
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

__global__ void __launch_bounds__(EIG_T) hetrd_kernel(TrdArgs p) {
    extern __shared__ cplx sv[];
    const int64_t n = p.n;
    cplx* vp = sv;          // v of the previous step (its update is pending)
    cplx* wp = sv + n;      // w of the previous step
    cplx* vc = sv + 2 * n;  // v of this step
    cplx* red = sv + 3 * n; // per-thread partial row sums
    __shared__ double ws[32];
    __shared__ cplx s_c[3];
    const int T = blockDim.x, tid = threadIdx.x;
    const int B = gridDim.x, b = blockIdx.x;
    unsigned passed = 0;
    bool pend = false;
    for (int64_t j = 0; j + 1 < n; ++j) {
        // column j with the pending update: vc[j] = diagonal, vc[j+1:] = x
        const cplx vpj = pend ? vp[j] : cmk(0, 0), wpj = pend ? wp[j] : cmk(0, 0);
        double nrm2 = 0.0;
        for (int64_t i = j + tid; i < n; i += T) {
            cplx a = __ldcg(p.A + i + n * j);
            if (pend) a = csub(a, cadd(cmul(wp[i], cconj(vpj)), cmul(vp[i], cconj(wpj))));
            vc[i] = a;
            if (i >= j + 2) nrm2 += a.x * a.x + a.y * a.y;
        }
        nrm2 = block_sum(nrm2, ws);  // synchronises: vc visible
        if (tid == 0) {
            // reflector with H^H x = beta e_1, beta real (LAPACK zlarfg's convention)
            const cplx al = vc[j + 1];
            cplx tau = cmk(0, 0), scale = cmk(0, 0);
            double beta = al.x;
            if (nrm2 != 0.0 || al.y != 0.0) {
                beta = -copysign(sqrt(al.x * al.x + al.y * al.y + nrm2), al.x);
                tau = cmk((beta - al.x) / beta, -al.y / beta);
                scale = crecip(cmk(al.x - beta, al.y));
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
            cplx acc = cmk(0, 0);
            if (tid < cs * cr) {
                const int64_t i = r0 + tid % cr;
                const cplx vpi = pend ? vp[i] : cmk(0, 0), wpi = pend ? wp[i] : cmk(0, 0);
                for (int64_t l = j + 1 + tid / cr; l < n; l += cs) {
                    cplx a = __ldcg(p.A + i + n * l);
                    if (pend) {
                        a = csub(a, cadd(cmul(wpi, cconj(vp[l])), cmul(vpi, cconj(wp[l]))));
                        p.A[i + n * l] = a;
                    }
                    acc = cfma(a, vc[l], acc);
                }
            }
            red[tid] = acc;
            __syncthreads();
            if (tid < cr) {
                cplx s = cmk(0, 0);
                for (int q = 0; q < cs; ++q) s = cadd(s, red[tid + q * cr]);
                const cplx yi = cmul(tau, s);
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
        // w = y - (tau/2) (y^H v) v, the same in every block (fixed order)
        if (tid == 0) {
            cplx s = cmk(0, 0);
            for (int q = 0; q < B; ++q) s = cadd(s, __ldcg(p.dpart + q));
            s_c[2] = cmul(cmk(-0.5 * tau.x, -0.5 * tau.y), s);
        }
        __syncthreads();
        const cplx al2 = s_c[2];
        for (int64_t i = j + 1 + tid; i < n; i += T) wp[i] = cfma(al2, vc[i], __ldcg(p.y + i));
        // block 0 keeps the reflector below the subdiagonal of column j
        if (b == 0)
            for (int64_t i = j + 2 + tid; i < n; i += T) p.A[i + n * j] = vc[i];
        cplx* t = vp;
        vp = vc;
        vc = t;
        pend = true;
        __syncthreads();
    }
    if (b == 0 && tid == 0) {
        cplx a = __ldcg(p.A + (n - 1) + n * (n - 1));
        if (pend)
            a = csub(a, cadd(cmul(wp[n - 1], cconj(vp[n - 1])), cmul(vp[n - 1], cconj(wp[n - 1]))));
        p.d[n - 1] = a.x;
    }
}

// ---- 2. bisection ------------------------------------------------------------
// Number of eigenvalues of T below x (LDL^T pivots, LAPACK dstebz's guard).
__device__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e, int t,
                           double x, double pivmin) {
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0;
    for (int k = 1; k < t; ++k) {
        q = (d[k] - x) - e[k - 1] * e[k - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += q < 0.0;
    }
    return cnt;
}

// The g-th largest eigenvalue (number t-1-g ascending) to eps * |T|:
// lam_desc[g], and lam_asc[want-1-g].  bounds = (low, high, pivmin, |T|).
__global__ void bisect_kernel(const double* __restrict__ d, const double* __restrict__ e, int t,
                              int want, const double* __restrict__ bounds,
                              double* __restrict__ lam_desc, double* __restrict__ lam_asc) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= want) return;
    const int idx = t - 1 - g;
    const double eps = 2.220446049250313e-16, pivmin = bounds[2], abstol = eps * bounds[3];
    double lo = bounds[0], hi = bounds[1];
    for (int it = 0; it < 256; ++it) {
        const double tol = 2.0 * eps * fmax(fabs(lo), fabs(hi)) + abstol + pivmin;
        if (hi - lo <= tol) break;
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count(d, e, t, mid, pivmin) > idx)
            hi = mid;
        else
            lo = mid;
    }
    const double v = 0.5 * (lo + hi);
    lam_desc[g] = v;
    lam_asc[want - 1 - g] = v;
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
    // dlagtf): row k of U holds (u1, u2, u3) at columns (k, k+1, k+2)
    double a = d[0] - s, bsup = t > 1 ? e[0] : 0.0;
    for (int k = 0; k < t - 1; ++k) {
        const double cs = e[k];          // subdiagonal entry below the pivot
        const double dn = d[k + 1] - s;  // next diagonal
        const double bn = k + 2 < t ? e[k + 1] : 0.0;
        const size_t o = (size_t)k * W + g;
        if (fabs(a) >= fabs(cs)) {  // keep row k
            const double pa = guard(a);
            const double mult = cs / pa;
            fu1[o] = pa;
            fu2[o] = bsup;
            fu3[o] = 0.0;
            fl[o] = mult;
            piv[o] = 0;
            a = dn - mult * bsup;
            bsup = bn;
        } else {  // interchange rows k and k+1
            const double mult = a / cs;
            fu1[o] = cs;
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
        fu1[o] = guard(a);
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
            const double r = (zw[o] - fu2[o] * z1 - fu3[o] * z2) / fu1[o];
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
            double s = 0.0;
            for (int64_t i = j + lane; i < t; i += 32) s += sq[i] * zc[i];
            s = warp_sum(s);
            s = __shfl_sync(0xffffffffu, s, 0) * tau;
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
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= k) return;
    double* q = Q + c * t;
    for (int64_t i = lane; i < t; i += 32) q[i] = (i == c) ? 1.0 : 0.0;
    __syncwarp();
    for (int64_t j = c; j >= 0; --j) {
        const double tau = qtau[j];
        if (tau == 0.0) continue;
        const double* v = Zr + j * t;  // v[j] = 1 implicit
        double s = 0.0;
        for (int64_t i = j + lane; i < t; i += 32) s += (i == j ? 1.0 : v[i]) * q[i];
        s = warp_sum(s);
        s = __shfl_sync(0xffffffffu, s, 0) * tau;
        for (int64_t i = j + lane; i < t; i += 32) q[i] -= s * (i == j ? 1.0 : v[i]);
        __syncwarp();
    }
    // R's diagonal carries the sign that maps the input column onto Q's column
    if (rdiag[c] < 0.0)
        for (int64_t i = lane; i < t; i += 32) q[i] = -q[i];
}

// ---- 5. back-transformation ----------------------------------------------------
// X[:, c] = H_0 ... H_{n-2} [z_c], z_c real (t = n rows), one warp per
// column.  Reflector j: v_j[j+1] = 1, v_j[j+2:] = A[j+2:, j].
__global__ void backtransform_kernel(const cplx* __restrict__ A, int64_t n,
                                     const cplx* __restrict__ tau, const double* __restrict__ Z,
                                     int64_t k, cplx* __restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= k) return;
    cplx* x = X + c * n;
    const double* z = Z + c * n;
    for (int64_t i = lane; i < n; i += 32) x[i] = cmk(z[i], 0.0);
    __syncwarp();
    for (int64_t j = n - 2; j >= 0; --j) {
        const cplx tj = tau[j];
        if (tj.x == 0.0 && tj.y == 0.0) continue;
        const cplx* v = A + j * n;
        // s = v^H x over rows j+1..n-1
        double sr = 0.0, si = 0.0;
        for (int64_t i = j + 1 + lane; i < n; i += 32) {
            const cplx vi = (i == j + 1) ? cmk(1, 0) : v[i];
            const cplx xi = x[i];
            sr += vi.x * xi.x + vi.y * xi.y;
            si += vi.x * xi.y - vi.y * xi.x;
        }
        sr = __shfl_sync(0xffffffffu, warp_sum(sr), 0);
        si = __shfl_sync(0xffffffffu, warp_sum(si), 0);
        const cplx s = cmul(tj, cmk(sr, si));  // H x = x - tau v (v^H x)
        for (int64_t i = j + 1 + lane; i < n; i += 32) {
            const cplx vi = (i == j + 1) ? cmk(1, 0) : v[i];
            x[i] = csub(x[i], cmul(s, vi));
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

// Gershgorin interval and the pivot guard of T, one block.
__global__ void tri_bounds_kernel(const double* __restrict__ d, const double* __restrict__ e,
                                  int t, double* __restrict__ out) {
    __shared__ double slo[EIG_T], shi[EIG_T], sm[EIG_T];
    double lo = 1e300, hi = -1e300, me = 0.0;
    for (int k = threadIdx.x; k < t; k += blockDim.x) {
        const double r = (k > 0 ? fabs(e[k - 1]) : 0.0) + (k + 1 < t ? fabs(e[k]) : 0.0);
        lo = fmin(lo, d[k] - r);
        hi = fmax(hi, d[k] + r);
        if (k + 1 < t) me = fmax(me, e[k] * e[k]);
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
    const unsigned B1 = (unsigned)std::min<int64_t>(ctx->sm_count, std::max<int64_t>(1, n / 8));
    TN_REQUIRE((n - 1 + B1 - 1) / B1 <= EIG_T, "eig_top: too few blocks for the row partition");
    ProfScope ps(ctx, 2, 16.0 / 3.0 * n * n * n + 8.0 * n * n * want, 16.0 * n * n);
    const size_t nd = (size_t)n, nw = nd * (size_t)want;
    // scratch layout, 256-byte aligned pieces
    const size_t sizes[] = {sizeof(double) * nd,     sizeof(double) * nd,    sizeof(cplx) * nd,
                            sizeof(cplx) * nd,       sizeof(cplx) * B1,      sizeof(double) * 8,
                            sizeof(double) * want,   sizeof(double) * want,  sizeof(double) * want,
                            sizeof(double) * want,   sizeof(double) * nw,    sizeof(double) * nw,
                            sizeof(double) * nw,     sizeof(double) * nw,    sizeof(double) * nw,
                            sizeof(double) * nw,     sizeof(double) * nw,    nw};
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
    tri_bounds_kernel<<<1, EIG_T, 0, ctx->stream>>>(d, e, t, bounds);
    ctx->count();
    bisect_kernel<<<nblk(want, 128), 128, 0, ctx->stream>>>(d, e, t, (int)want, bounds, lam_desc,
                                                           lam_asc);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    separate_shifts_kernel<<<1, 32, 0, ctx->stream>>>(lam_desc, (int)want, bounds, shift);
    ctx->count();
    stein_kernel<<<nblk(want, 64), 64, 0, ctx->stream>>>(d, e, t, (int)want, shift, bounds, f1, f2,
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
    backtransform_kernel<<<nblk(want * 32, 128), 128, 0, ctx->stream>>>(G, n, tau, Q, want, X);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

}  // namespace tn
