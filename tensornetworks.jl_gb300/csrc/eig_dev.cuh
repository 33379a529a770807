// Device helpers shared by the Hermitian eigensolvers: the grid-wide one of
// the truncated split (eig.cu) and the one-block one inside the trajectory
// engine (qjmc_engine.cu).
#pragma once

#include "common.cuh"

namespace tn {
namespace eigdev {

constexpr int BIS_W = 4;  // lanes per eigenvalue in the bisection
constexpr int BT_G = 4;   // reflectors per compact-WY group of the back-transformation

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block (blockDim.x a multiple of 32, at most 1024); the result
// is valid in every thread.  The warp totals are added as a tree: a serial
// chain of dependent FP64 additions costs tens of cycles per link on GB300.
__device__ __forceinline__ double block_sum(double v, double* ws) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    __syncthreads();
    if (lane == 0) ws[w] = v;
    __syncthreads();
    double t = lane < nw ? ws[lane] : 0.0;
    t = warp_sum(t);
    return __shfl_sync(0xffffffffu, t, 0);
}

// Number of eigenvalues of the symmetric tridiagonal T (diagonal d, squared
// off-diagonal e2) below x: sign changes of the leading principal minors
// q_k = det(T[0:k, 0:k] - x I), q_k = (d_k - x) q_{k-1} - e_{k-1}^2 q_{k-2}
// (Sylvester's inertia: a sign change is a negative LDL^T pivot q_k /
// q_{k-1}).  No division: two dependent FP64 operations per step, where the
// pivot form waits on a division.  Both minors are rescaled by an exact power
// of two when they leave [2^-400, 2^400]; an exact zero becomes the pivot
// -pivmin (LAPACK dstebz's guard).
__device__ __forceinline__ int sturm_count(const double* __restrict__ d,
                                           const double* __restrict__ e2, int t, double x,
                                           double pivmin) {
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
__device__ __forceinline__ int sturm_count_f(const float* __restrict__ d,
                                             const float* __restrict__ e2, int t, float x,
                                             float pivmin) {
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

// splitmix64 of (a, b) mapped to (-1, 1): the start vectors of inverse
// iteration
__device__ __forceinline__ double hash_uniform(uint64_t a, uint64_t b) {
    uint64_t z = a * 0x9E3779B97F4A7C15ull + b + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

// Householder reflector j of the tridiagonal reduction of the n x n matrix
// A: v_j[j+1] = 1, v_j[j+2:] = A[j+2:, j], zero above.
__device__ __forceinline__ cplx refl(const cplx* __restrict__ A, int64_t n, int64_t j, int64_t i) {
    return i == j + 1 ? cmk(1, 0) : (i > j + 1 ? A[i + n * j] : cmk(0, 0));
}

// The g-th largest eigenvalue by one group of BIS_W lanes (lane m of the
// group, shuffle mask grp); see bisect_kernel.
// W lanes (2 or 4) cut the interval (W+1)-fold per round: fewer lanes do
// less FP64 work per eigenvalue, more lanes finish in fewer rounds.
template <int W>
__device__ __forceinline__ void bisect_group_w(int g, int m, unsigned grp,
                                               const double* __restrict__ d,
                                               const double* __restrict__ e2,
                                               const float* __restrict__ d32,
                                               const float* __restrict__ e2f, int t, int want,
                                               const double* __restrict__ bounds,
                                               double* __restrict__ lam_desc,
                                               double* __restrict__ lam_asc) {
    const int idx = t - 1 - g;
    const double eps = 2.220446049250313e-16, pivmin = bounds[2], tn = bounds[3];
    const double abstol = eps * tn;
    double lo = bounds[0], hi = bounds[1];
    {
        const float pf = (float)bounds[4];
        float lf = __double2float_rd(lo), hf = __double2float_ru(hi);
        const float tolf = 64.f * 1.1920929e-7f * (float)tn;
        for (int it = 0; it < 64 && hf - lf > tolf; ++it) {
            const float h = (hf - lf) * (1.f / (W + 1));
            const float x = lf + h * (float)(m + 1);
            const int below = sturm_count_f(d32, e2f, t, x, pf) <= idx;  // eigenvalue >= x
            // new interval: between the last point with count <= idx and the next
            float nl = lf, nh = hf;
#pragma unroll
            for (int u = 0; u < W; ++u) {
                const int bu = __shfl_sync(grp, below, u, W);
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
        const int oka = __shfl_sync(grp, ok, 0, W), okb = __shfl_sync(grp, ok, 1, W);
        lo = oka ? a : lo;
        hi = okb ? b : hi;
    }
    for (int it = 0; it < 128; ++it) {
        const double tol = 2.0 * eps * fmax(fabs(lo), fabs(hi)) + abstol + pivmin;
        if (hi - lo <= tol) break;
        const double h = (hi - lo) * (1.0 / (W + 1));
        const double x = lo + h * (double)(m + 1);
        const int below = sturm_count(d, e2, t, x, pivmin) <= idx;
        double nl = lo, nh = hi;
#pragma unroll
        for (int u = 0; u < W; ++u) {
            const int bu = __shfl_sync(grp, below, u, W);
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

__device__ __forceinline__ void bisect_group(int g, int m, unsigned grp, const double* __restrict__ d,
                                             const double* __restrict__ e2,
                                             const float* __restrict__ d32,
                                             const float* __restrict__ e2f, int t, int want,
                                             const double* __restrict__ bounds,
                                             double* __restrict__ lam_desc,
                                             double* __restrict__ lam_asc) {
    bisect_group_w<BIS_W>(g, m, grp, d, e2, d32, e2f, t, want, bounds, lam_desc, lam_asc);
}

// Inverse iteration for vector g; see stein_kernel.
__device__ __forceinline__ void stein_vector(int g, const double* __restrict__ d,
                                             const double* __restrict__ e, int t, int want,
                                             const double* __restrict__ shift,
                                             const double* __restrict__ bounds,
                                             double* __restrict__ fu1, double* __restrict__ fu2,
                                             double* __restrict__ fu3, double* __restrict__ fl,
                                             unsigned char* __restrict__ piv,
                                             double* __restrict__ zw, double* __restrict__ Z) {
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

// Column k-1-w of Q from the QR reflectors, by one warp (lane); see
// qr_form_kernel.
__device__ __forceinline__ void qr_form_column(int64_t w, int lane, const double* __restrict__ Zr,
                                               int64_t t, int64_t k,
                                               const double* __restrict__ qtau,
                                               const double* __restrict__ rdiag,
                                               double* __restrict__ Q) {
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

// Compact-WY factor of reflector group q by one warp (lane); see
// wy_factor_kernel.
__device__ __forceinline__ void wy_group(int64_t q, int lane, const cplx* __restrict__ A, int64_t n,
                                         const cplx* __restrict__ tau,
                                         cplx* __restrict__ Tg) {
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
                sre[c][r] = fma(v[c].x, v[r].x, fma(v[c].y, v[r].y, sre[c][r]));
                sim[c][r] = fma(v[c].x, v[r].y, fma(-v[c].y, v[r].x, sim[c][r]));
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

// Column c of X = Q_trd Z by one warp (lane); see backtransform_kernel.
__device__ __forceinline__ void bt_column(int64_t c, int lane, const cplx* __restrict__ A, int64_t n,
                                          const cplx* __restrict__ Tg, int64_t ngroups,
                                          const double* __restrict__ Z,
                                          cplx* __restrict__ X) {
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
                    const cplx v = refl(A, n, a + r, i);  // conj(v) x as two FMA chains
                    sr[r] = fma(v.x, xi.x, fma(v.y, xi.y, sr[r]));
                    si[r] = fma(v.x, xi.y, fma(-v.y, xi.x, si[r]));
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
                if (r < nr) {  // x -= u v, fused
                    const cplx v = refl(A, n, a + r, i);
                    xi.x = fma(-u[r].x, v.x, fma(u[r].y, v.y, xi.x));
                    xi.y = fma(-u[r].x, v.y, fma(-u[r].y, v.x, xi.y));
                }
            x[i] = xi;
        }
        __syncwarp();
    }

}

// Shifts for inverse iteration: descending eigenvalues pulled apart so that
// consecutive shifts differ by at least sep (LAPACK dstein's perturbation);
// one thread.
__device__ __forceinline__ void separate_shifts_serial(const double* __restrict__ lam, int want,
                                                       const double* __restrict__ bounds,
                                                       double* __restrict__ shift) {
    const double sep = 10.0 * 2.220446049250313e-16 * fmax(bounds[3], 1e-290);
    double prev = 0.0;
    for (int g = 0; g < want; ++g) {
        double s = lam[g];
        if (g > 0 && s > prev - sep) s = prev - sep;
        shift[g] = s;
        prev = s;
    }

}

// Gershgorin interval, pivot guards and |T| (out[0..4]), and FP32 copies of
// d and e^2 for the bisection's first phase; all threads of one block, with
// blockDim.x-entry shared arrays slo, shi, sm.
__device__ __forceinline__ void tri_bounds_block(const double* __restrict__ d,
                                                 const double* __restrict__ e, int t,
                                                 double* __restrict__ out, float* __restrict__ d32,
                                                 float* __restrict__ e2f, double* __restrict__ e2,
                                                 double* slo, double* shi, double* sm) {
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

}  // namespace eigdev
}  // namespace tn
