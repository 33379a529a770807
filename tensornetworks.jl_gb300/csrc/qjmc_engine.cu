// Quantum-jump trajectories as one persistent launch
// (src/algorithms/mps/qjmc.jl:28-220, one trajectory per qjmc_simulation call
// there).
//
// Every block of the launch owns one trajectory at a time and runs it to its
// end on the device, with no host round trip: the gate rows of applygates!
// (structures/mps/gatelist.jl:191-227) with the truncating centre moves before
// each gate, every truncated split through a one-block FP64 Hermitian
// eigensolver of the Gram matrix (the steps of eig.cu, run by one block), the
// norm, the emission rates from one-site reduced density matrices, the
// uniform draws (per-trajectory Philox4x32-10 streams or the caller's
// arrays), the jump and the observables.  Bond dimensions live in shared
// memory and the site tensors in a per-block slot of fixed capacity, so no
// step needs the host to size a tensor, and trajectories of different bond
// dimension advance independently.
//
// GB300 issues FP64 at two FMAs per clock per SM.  A block's contractions,
// Gram products, tridiagonal reduction and back-transformation keep that pipe
// busy from L1/L2-resident operands (a slot's scratch is a few MB), and four
// 128-thread blocks per SM overlap one block's latency-bound phases
// (bisection, inverse iteration, keep rule, reductions) with the others' FMA
// phases.
#include <cmath>
#include <memory>

#include "eig_dev.cuh"
#include "mps.cuh"
#include "philox.cuh"

namespace tn {

std::vector<cplx> inner_terms(Ctx* ctx, const tn_mps* bra, const tn_mps* ket,
                              const std::vector<Term>& terms);

namespace {

using namespace eigdev;

constexpr int QT = 128;        // threads per trajectory block
constexpr int QJ_GMAX = 256;   // largest Gram order: d x bond dimension
constexpr int QJ_NMAX = 1024;  // most sites
constexpr int QJ_DMAX = 4;     // largest physical dimension

// per-trajectory status words
enum : int { QE_OK = 0, QE_CAPACITY = 1, QE_DRAWS = 2, QE_JUMPS = 3, QE_NOCHANNEL = 4 };

struct QjParams {
    int N, d, nsteps, save_every, nobs, njump, maxj, nrows_out;
    int classical;  // 0: jump decision from the norm lost in the step (qjmc.jl:65-86)
    double dt, cutoff;
    int maxdim, mindim;
    int nrows;  // gate rows
    const int *row_start, *row_len, *gsite, *gns;
    const cplx* const* gM;  // gate matrices, small_apply form M[I + d^n J]
    const int* jsite;
    const cplx *jL, *jLdL;  // njump x d x d, small_apply form M[i + d o] = op[o, i]
    const double* jw;       // |coefficient|^2 of each channel
    const int* osite;
    const cplx* oO;  // nobs x d x d, small_apply form
    const cplx* const* psi0;
    const int* psi0_dims;
    int psi0_center;
    const double* draws;  // ntraj x ndraws, or null for the Philox streams
    int64_t ndraws;
    uint64_t seed;
    uint32_t first_traj;
    int ntraj;
    cplx* mps_pool;
    int64_t mps_slot;        // complex entries per slot
    const int64_t* cap_off;  // N site offsets within a slot
    const int* cap;          // N+1 bond capacities
    char* scr_pool;
    int64_t scr_slot;  // bytes per slot
    int gmax;          // Gram order bound of a slot's scratch
    cplx* obs_traj;    // ntraj x nrows_out x nobs; row 0 is the host's
    int* njumps;
    int* jump_ch;       // ntraj x maxj, 1-based channel
    double* jump_time;  // ntraj x maxj
    int* err;           // ntraj status words
    int64_t* used;      // ntraj draws consumed
    double* flops;      // ntraj algorithmic FP64 flops
};

// ---- a slot's scratch -----------------------------------------------------------
struct Scr {
    cplx *th, *th2, *G, *V, *tmp, *tau, *wyT, *rho;
    double *Z, *Q, *f1, *f2, *f3, *fl, *zw;
    double *d, *e, *e2, *shift, *qtau, *rdiag, *lamd, *lama, *bounds;
    float *d32, *e2f;
    unsigned char* piv;
};

struct Bump {
    char* base;
    size_t off;
    __host__ __device__ char* take(size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return p;
    }
};

// Carves the scratch of one slot (Gram order <= g, N sites, dimension d)
// from base; returns its size in bytes (base may be null).
__host__ __device__ inline size_t scr_layout(char* base, int g, int N, int d, Scr& s) {
    Bump b{base, 0};
    const size_t gg = (size_t)g * g;
    s.th = (cplx*)b.take(sizeof(cplx) * gg);
    s.th2 = (cplx*)b.take(sizeof(cplx) * gg);
    s.G = (cplx*)b.take(sizeof(cplx) * gg);
    s.V = (cplx*)b.take(sizeof(cplx) * gg);
    s.tmp = (cplx*)b.take(sizeof(cplx) * gg);
    s.Z = (double*)b.take(sizeof(double) * gg);
    s.Q = (double*)b.take(sizeof(double) * gg);
    s.f1 = (double*)b.take(sizeof(double) * gg);
    s.f2 = (double*)b.take(sizeof(double) * gg);
    s.f3 = (double*)b.take(sizeof(double) * gg);
    s.fl = (double*)b.take(sizeof(double) * gg);
    s.zw = (double*)b.take(sizeof(double) * gg);
    s.piv = (unsigned char*)b.take(gg);
    s.d = (double*)b.take(sizeof(double) * g);
    s.e = (double*)b.take(sizeof(double) * g);
    s.e2 = (double*)b.take(sizeof(double) * g);
    s.shift = (double*)b.take(sizeof(double) * g);
    s.qtau = (double*)b.take(sizeof(double) * g);
    s.rdiag = (double*)b.take(sizeof(double) * g);
    s.lamd = (double*)b.take(sizeof(double) * g);
    s.lama = (double*)b.take(sizeof(double) * g);
    s.bounds = (double*)b.take(sizeof(double) * 8);
    s.d32 = (float*)b.take(sizeof(float) * g);
    s.e2f = (float*)b.take(sizeof(float) * g);
    s.tau = (cplx*)b.take(sizeof(cplx) * g);
    s.wyT = (cplx*)b.take(sizeof(cplx) * ((size_t)g / BT_G + 1) * BT_G * BT_G);
    s.rho = (cplx*)b.take(sizeof(cplx) * (size_t)N * d * d);
    return b.off;
}

// ---- block state -------------------------------------------------------------
struct Sh {
    int dims[QJ_NMAX + 1];
    int center;
    int flag;  // status of the running trajectory
    int k;     // broadcast of a kept dimension
    double sc[4];
    cplx c[4];
    double rd[2][QT];  // block reductions: one value per thread, summed by warp 0
    double res[2];
    cplx buf[4 * QJ_GMAX + QT];  // tridiagonal-reduction vectors; bounds, QR and BT scratch
};

// Block sums through shared memory: every thread stores its value, warp 0
// adds eight per lane and one warp_sum, and the total comes back through
// shared memory.  Twelve FP64 warp-instructions per sum where a shuffle
// butterfly in every warp takes eighty, on a pipe that issues two FP64
// lane-operations per clock per SM.
__device__ __forceinline__ double bsum(double v, Sh& sh) {
    sh.rd[0][threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double a = 0.0, b = 0.0;
#pragma unroll
        for (int q = 0; q < QT / 32; q += 2) {
            a += sh.rd[0][threadIdx.x + 32 * q];
            b += sh.rd[0][threadIdx.x + 32 * (q + 1)];
        }
        a = warp_sum(a + b);
        if (threadIdx.x == 0) sh.res[0] = a;
    }
    __syncthreads();
    return sh.res[0];
}

__device__ __forceinline__ void bsum2(double u, double v, Sh& sh, double& su, double& sv) {
    sh.rd[0][threadIdx.x] = u;
    sh.rd[1][threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 64) {
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        double a = 0.0, b = 0.0;
#pragma unroll
        for (int q = 0; q < QT / 32; q += 2) {
            a += sh.rd[w][l + 32 * q];
            b += sh.rd[w][l + 32 * (q + 1)];
        }
        a = warp_sum(a + b);
        if (l == 0) sh.res[w] = a;
    }
    __syncthreads();
    su = sh.res[0];
    sv = sh.res[1];
}

struct TruncD {
    double cutoff;
    int maxdim, mindim;
};

struct Traj {
    const QjParams* p;
    Sh* sh;
    cplx* mps;
    Scr s;
    uint64_t used;    // draws consumed (the same in every thread)
    uint32_t trajno;  // Philox stream number
    int t;            // trajectory index within the launch
    TruncD tr;
    double fl;  // algorithmic FP64 flops so far (the same in every thread)
    __device__ cplx* A(int i) const { return mps + p->cap_off[i - 1]; }
    __device__ int dl(int i) const { return sh->dims[i - 1]; }
    __device__ int dr(int i) const { return sh->dims[i]; }
};

__device__ __forceinline__ void set_flag(Sh& sh, int f) {
    if (threadIdx.x == 0 && sh.flag == QE_OK) sh.flag = f;
    __syncthreads();
}

__device__ __forceinline__ void bcopy(cplx* __restrict__ dst, const cplx* __restrict__ src, int n) {
    for (int e = threadIdx.x; e < n; e += QT) dst[e] = src[e];
    __syncthreads();
}

// ---- block contractions (FP64, one thread per output element) ------------------
enum { ON = 0, OC = 1, OR = 2, OT = 3 };

template <int OP>
__device__ __forceinline__ cplx opA(const cplx* __restrict__ A, int lda, int i, int l) {
    if (OP == ON) return A[i + lda * l];
    if (OP == OC) return cconj(A[l + lda * i]);
    return cconj(A[i + lda * l]);  // OR
}
template <int OP>
__device__ __forceinline__ cplx opB(const cplx* __restrict__ B, int ldb, int l, int j) {
    if (OP == ON) return B[l + ldb * j];
    if (OP == OC) return cconj(B[j + ldb * l]);
    return B[j + ldb * l];  // OT
}

// C (m x n, ldc) = op(A) op(B), inner dimension k; two partial sums per
// element keep two independent FMA chains in flight.
template <int OA, int OB>
__device__ __noinline__ void bgemm(int m, int n, int k, const cplx* __restrict__ A, int lda,
                      const cplx* __restrict__ B, int ldb, cplx* __restrict__ C, int ldc) {
    for (int e = threadIdx.x; e < m * n; e += QT) {
        const int i = e % m, j = e / m;
        double r0 = 0.0, i0 = 0.0, r1 = 0.0, i1 = 0.0;
        int l = 0;
        for (; l + 1 < k; l += 2) {
            const cplx a0 = opA<OA>(A, lda, i, l), b0 = opB<OB>(B, ldb, l, j);
            const cplx a1 = opA<OA>(A, lda, i, l + 1), b1 = opB<OB>(B, ldb, l + 1, j);
            r0 = fma(a0.x, b0.x, fma(-a0.y, b0.y, r0));
            i0 = fma(a0.x, b0.y, fma(a0.y, b0.x, i0));
            r1 = fma(a1.x, b1.x, fma(-a1.y, b1.y, r1));
            i1 = fma(a1.x, b1.y, fma(a1.y, b1.x, i1));
        }
        if (l < k) {
            const cplx a0 = opA<OA>(A, lda, i, l), b0 = opB<OB>(B, ldb, l, j);
            r0 = fma(a0.x, b0.x, fma(-a0.y, b0.y, r0));
            i0 = fma(a0.x, b0.y, fma(a0.y, b0.x, i0));
        }
        C[i + ldc * j] = cmk(r0 + r1, i0 + i1);
    }
    __syncthreads();
}

// Hermitian Gram matrix of th (m x n): th th^H (left) or th^H th, both
// triangles, real diagonal; the lower triangle is computed.
__device__ __noinline__ void bgram(bool left, int m, int n, const cplx* __restrict__ th, cplx* __restrict__ G) {
    const int g = left ? m : n, k = left ? n : m;
    for (int e = threadIdx.x; e < g * g; e += QT) {
        const int i = e % g, j = e / g;
        if (i < j) continue;
        double r0 = 0.0, i0 = 0.0, r1 = 0.0, i1 = 0.0;
        if (left) {  // sum_l th[i,l] conj(th[j,l])
            int l = 0;
            for (; l + 1 < k; l += 2) {
                const cplx a0 = th[i + m * l], b0 = th[j + m * l];
                const cplx a1 = th[i + m * (l + 1)], b1 = th[j + m * (l + 1)];
                r0 = fma(a0.x, b0.x, fma(a0.y, b0.y, r0));
                i0 = fma(a0.y, b0.x, fma(-a0.x, b0.y, i0));
                r1 = fma(a1.x, b1.x, fma(a1.y, b1.y, r1));
                i1 = fma(a1.y, b1.x, fma(-a1.x, b1.y, i1));
            }
            if (l < k) {
                const cplx a0 = th[i + m * l], b0 = th[j + m * l];
                r0 = fma(a0.x, b0.x, fma(a0.y, b0.y, r0));
                i0 = fma(a0.y, b0.x, fma(-a0.x, b0.y, i0));
            }
        } else {  // sum_l conj(th[l,i]) th[l,j]
            const cplx* ci = th + (size_t)m * i;
            const cplx* cj = th + (size_t)m * j;
            int l = 0;
            for (; l + 1 < k; l += 2) {
                const cplx a0 = ci[l], b0 = cj[l], a1 = ci[l + 1], b1 = cj[l + 1];
                r0 = fma(a0.x, b0.x, fma(a0.y, b0.y, r0));
                i0 = fma(a0.x, b0.y, fma(-a0.y, b0.x, i0));
                r1 = fma(a1.x, b1.x, fma(a1.y, b1.y, r1));
                i1 = fma(a1.x, b1.y, fma(-a1.y, b1.x, i1));
            }
            if (l < k) {
                const cplx a0 = ci[l], b0 = cj[l];
                r0 = fma(a0.x, b0.x, fma(a0.y, b0.y, r0));
                i0 = fma(a0.x, b0.y, fma(-a0.y, b0.x, i0));
            }
        }
        const cplx v = cmk(r0 + r1, i0 + i1);
        if (i == j) {
            G[i + g * j] = cmk(v.x, 0.0);
        } else {
            G[i + g * j] = v;
            G[j + g * i] = cconj(v);
        }
    }
    __syncthreads();
}

// out[a + na J + na nJ c] = sum_I in[a + na I + na nI c] M[I + nI J]
// (small_apply on contiguous tensors)
__device__ __noinline__ void bapply(const cplx* __restrict__ in, cplx* __restrict__ out,
                       const cplx* __restrict__ M, int nI, int nJ, int na, int nc) {
    const int total = na * nJ * nc;
    for (int e = threadIdx.x; e < total; e += QT) {
        const int a = e % na, J = (e / na) % nJ, c = e / (na * nJ);
        const cplx* x = in + a + (size_t)na * nI * c;
        double re = 0.0, im = 0.0;
        for (int I = 0; I < nI; ++I) {
            const cplx v = x[(size_t)na * I], w = M[I + nI * J];
            re = fma(v.x, w.x, fma(-v.y, w.y, re));
            im = fma(v.x, w.y, fma(v.y, w.x, im));
        }
        out[e] = cmk(re, im);
    }
    __syncthreads();
}

// ---- one-block Hermitian eigensolver (the steps of eig.cu) ------------------------
// Householder reduction of the n x n Hermitian A (both triangles) to a real
// tridiagonal (d, e), reflectors below the subdiagonal of A and their scalars
// in tau.  One pass per step applies the pending rank-2 update and forms the
// matvec, as hetrd_kernel does with one block.
__device__ __noinline__ void hetrd_blk(cplx* __restrict__ A, int n, double* __restrict__ d,
                          double* __restrict__ e, cplx* __restrict__ tau, Sh& sh) {
    cplx* vp = sh.buf;
    cplx* wp = sh.buf + QJ_GMAX;
    cplx* vc = sh.buf + 2 * QJ_GMAX;
    cplx* red = sh.buf + 3 * QJ_GMAX;
    cplx* ys = sh.buf + 3 * QJ_GMAX + QT;
    const int tid = threadIdx.x;
    bool pend = false;
    double nrm2 = 0.0;
    for (int i = tid; i < n; i += QT) {
        const cplx a = A[i];
        vc[i] = a;
        if (i >= 2) nrm2 = fma(a.x, a.x, fma(a.y, a.y, nrm2));
    }
    nrm2 = bsum(nrm2, sh);
    for (int j = 0; j + 1 < n; ++j) {
        if (tid == 0) {
            // reflector with H^H x = beta e_1, beta real (LAPACK zlarfg's convention)
            const cplx al = vc[j + 1];
            cplx tv = cmk(0, 0), scale = cmk(0, 0);
            double beta = al.x;
            if (nrm2 != 0.0 || al.y != 0.0) {
                beta = -copysign(sqrt(al.x * al.x + al.y * al.y + nrm2), al.x);
                const double rb = 1.0 / beta;
                tv = cmk((beta - al.x) * rb, -al.y * rb);
                const double ur = al.x - beta, ui = al.y, rd = 1.0 / (ur * ur + ui * ui);
                scale = cmk(ur * rd, -ui * rd);
            }
            sh.c[0] = tv;
            sh.c[1] = scale;
            d[j] = vc[j].x;
            e[j] = beta;
            tau[j] = tv;
        }
        __syncthreads();
        const cplx tv = sh.c[0], scale = sh.c[1];
        for (int i = j + 2 + tid; i < n; i += QT) vc[i] = cmul(vc[i], scale);
        if (tid == 0) vc[j + 1] = cmk(1, 0);
        __syncthreads();
        // rows and columns j+1..n-1, up to QT rows per pass: pending update,
        // then y = tau A v
        const int m = n - j - 1;
        double dre = 0.0, dim = 0.0;
        for (int rb = 0; rb < m; rb += QT) {
            const int cr = min(m - rb, QT), cs = QT / cr;
            double ar = 0.0, ai = 0.0;
            if (tid < cs * cr) {
                const int i = j + 1 + rb + tid % cr;
                const cplx vpi = pend ? vp[i] : cmk(0, 0), wpi = pend ? wp[i] : cmk(0, 0);
                for (int l = j + 1 + tid / cr; l < n; l += cs) {
                    cplx a = A[i + (size_t)n * l];
                    if (pend) {
                        const cplx vl = vp[l], wl = wp[l];
                        a.x = fma(-wpi.x, vl.x, fma(-wpi.y, vl.y, fma(-vpi.x, wl.x, fma(-vpi.y, wl.y, a.x))));
                        a.y = fma(-wpi.y, vl.x, fma(wpi.x, vl.y, fma(-vpi.y, wl.x, fma(vpi.x, wl.y, a.y))));
                        A[i + (size_t)n * l] = a;
                    }
                    const cplx x = vc[l];
                    ar = fma(a.x, x.x, fma(-a.y, x.y, ar));
                    ai = fma(a.x, x.y, fma(a.y, x.x, ai));
                }
            }
            red[tid] = cmk(ar, ai);
            __syncthreads();
            int span = 1;
            while (span < cs) span <<= 1;
            for (int h = span >> 1; h > 0; h >>= 1) {
                if (tid < h * cr && tid + h * cr < cs * cr) red[tid] = cadd(red[tid], red[tid + h * cr]);
                __syncthreads();
            }
            if (tid < cr) {
                const cplx yi = cmul(tv, red[tid]);
                ys[rb + tid] = yi;
                const cplx t = cmul(cconj(yi), vc[j + 1 + rb + tid]);  // y^H v
                dre += t.x;
                dim += t.y;
            }
            __syncthreads();
        }
        bsum2(dre, dim, sh, dre, dim);
        // w = y - (tau/2) (y^H v) v
        const cplx al2 = cmul(cmk(-0.5 * tv.x, -0.5 * tv.y), cmk(dre, dim));
        for (int r = tid; r < m; r += QT) wp[j + 1 + r] = cfma(al2, vc[j + 1 + r], ys[r]);
        for (int i = j + 2 + tid; i < n; i += QT) A[i + (size_t)n * j] = vc[i];
        cplx* t = vp;  // v_j becomes the pending vector
        vp = vc;
        vc = t;
        pend = true;
        __syncthreads();
        // column j+1 with this step's update (v_{j+1} = 1)
        const cplx wj1 = wp[j + 1];
        nrm2 = 0.0;
        for (int r = tid; r < m; r += QT) {
            const int i = j + 1 + r;
            const cplx vi = vp[i], wi = wp[i];
            cplx a = A[i + (size_t)n * (j + 1)];
            a.x -= wi.x + (vi.x * wj1.x + vi.y * wj1.y);
            a.y -= wi.y + (vi.y * wj1.x - vi.x * wj1.y);
            vc[i] = a;
            if (i >= j + 3) nrm2 = fma(a.x, a.x, fma(a.y, a.y, nrm2));
        }
        nrm2 = bsum(nrm2, sh);
    }
    if (tid == 0) d[n - 1] = vc[n - 1].x;
    __syncthreads();
}

// Householder QR of Z (t x k, real, descending eigenvalues) by one block:
// reflectors in place, scalars qtau, R's diagonal rdiag (qr_kernel's steps).
// One thread per trailing column: its dot product and update run down the
// column without shuffles.
__device__ void qr_blk(double* __restrict__ Z, int t, int k, double* __restrict__ qtau,
                       double* __restrict__ rdiag, Sh& sh) {
    double* sq = reinterpret_cast<double*>(sh.buf);
    const int tid = threadIdx.x;
    for (int j = 0; j < k; ++j) {
        const double* zj = Z + (size_t)j * t;
        double nrm2 = 0.0;
        for (int i = j + tid; i < t; i += QT) {
            const double v = zj[i];
            sq[i] = v;
            if (i > j) nrm2 = fma(v, v, nrm2);
        }
        nrm2 = bsum(nrm2, sh);
        if (tid == 0) {
            const double al = sq[j];
            double tv = 0.0, beta = al, scale = 0.0;
            if (nrm2 != 0.0) {
                beta = -copysign(sqrt(al * al + nrm2), al);
                tv = (beta - al) / beta;
                scale = 1.0 / (al - beta);
            }
            sh.sc[0] = tv;
            sh.sc[1] = scale;
            sq[j] = 1.0;
            qtau[j] = tv;
            rdiag[j] = beta;
        }
        __syncthreads();
        const double tv = sh.sc[0], scale = sh.sc[1];
        for (int i = j + 1 + tid; i < t; i += QT) sq[i] *= scale;
        __syncthreads();
        for (int i = j + 1 + tid; i < t; i += QT) Z[i + (size_t)j * t] = sq[i];
        if (tv != 0.0) {
            for (int c = j + 1 + tid; c < k; c += QT) {
                double* zc = Z + (size_t)c * t;
                double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;  // four FMA chains
                int i = j;
                for (; i + 3 < t; i += 4) {
                    s0 = fma(sq[i], zc[i], s0);
                    s1 = fma(sq[i + 1], zc[i + 1], s1);
                    s2 = fma(sq[i + 2], zc[i + 2], s2);
                    s3 = fma(sq[i + 3], zc[i + 3], s3);
                }
                for (; i < t; ++i) s0 = fma(sq[i], zc[i], s0);
                const double f = ((s0 + s1) + (s2 + s3)) * tv;
                for (int i2 = j; i2 < t; ++i2) zc[i2] = fma(-f, sq[i2], zc[i2]);
            }
        }
        __syncthreads();
    }
}

// Column c of the explicit Q (t x k) from qr_blk's reflectors, by one
// thread: H_0 ... H_c e_c, signed like the input column (qr_form_kernel).
__device__ __forceinline__ void qr_form_thread(int c, const double* __restrict__ Zr, int t,
                                               const double* __restrict__ qtau,
                                               const double* __restrict__ rdiag,
                                               double* __restrict__ Q) {
    double* q = Q + (size_t)c * t;
    for (int i = 0; i < t; ++i) q[i] = (i == c) ? 1.0 : 0.0;
    for (int j = c; j >= 0; --j) {
        const double tv = qtau[j];
        if (tv == 0.0) continue;
        const double* v = Zr + (size_t)j * t;  // v[j] = 1 implicit
        double s0 = q[j], s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int i = j + 1;
        for (; i + 3 < t; i += 4) {
            s0 = fma(v[i], q[i], s0);
            s1 = fma(v[i + 1], q[i + 1], s1);
            s2 = fma(v[i + 2], q[i + 2], s2);
            s3 = fma(v[i + 3], q[i + 3], s3);
        }
        for (; i < t; ++i) s0 = fma(v[i], q[i], s0);
        const double f = ((s0 + s1) + (s2 + s3)) * tv;
        q[j] -= f;
        for (int i2 = j + 1; i2 < t; ++i2) q[i2] = fma(-f, v[i2], q[i2]);
    }
    if (rdiag[c] < 0.0)
        for (int i = 0; i < t; ++i) q[i] = -q[i];
}

// Compact-WY factor T of reflector group q by one thread (wy_factor_kernel's
// T[r][r] = tau_r, T[0:r, r] = -tau_r T[0:r, 0:r] V^H v_r).
__device__ __forceinline__ void wy_thread(int q, const cplx* __restrict__ A, int n,
                                          const cplx* __restrict__ tau, cplx* __restrict__ Tg) {
    const int a = q * BT_G;
    const int nr = min(BT_G, (n - 1) - a);
    cplx S[BT_G][BT_G];
#pragma unroll
    for (int c = 0; c < BT_G; ++c)
#pragma unroll
        for (int r = 0; r < BT_G; ++r) S[c][r] = cmk(0, 0);
    for (int i = a + 1; i < n; ++i) {
        cplx v[BT_G];
#pragma unroll
        for (int r = 0; r < BT_G; ++r) v[r] = r < nr ? refl(A, n, a + r, i) : cmk(0, 0);
#pragma unroll
        for (int c = 0; c < BT_G; ++c)
#pragma unroll
            for (int r = c + 1; r < BT_G; ++r) {
                S[c][r].x = fma(v[c].x, v[r].x, fma(v[c].y, v[r].y, S[c][r].x));
                S[c][r].y = fma(v[c].x, v[r].y, fma(-v[c].y, v[r].x, S[c][r].y));
            }
    }
    cplx T[BT_G][BT_G];
#pragma unroll
    for (int c = 0; c < BT_G; ++c)
#pragma unroll
        for (int r = 0; r < BT_G; ++r) T[c][r] = cmk(0, 0);
    for (int r = 0; r < nr; ++r) {
        const cplx tr = tau[a + r];
        T[r][r] = tr;
        cplx z[BT_G];
        for (int c = 0; c < r; ++c) z[c] = cmul(cmk(-tr.x, -tr.y), S[c][r]);
        for (int c = 0; c < r; ++c) {
            cplx acc = cmk(0, 0);
            for (int u = c; u < r; ++u) acc = cfma(T[c][u], z[u], acc);
            T[c][r] = acc;
        }
    }
    for (int c = 0; c < BT_G; ++c)
        for (int r = 0; r < BT_G; ++r) Tg[q * BT_G * BT_G + c + BT_G * r] = T[c][r];
}

// X = H_0 ... H_{n-2} Q (n x k, Q real) by the whole block, one reflector
// group at a time from the last: S = V^H X (a thread per (reflector,
// column) pair, each a dot product down the column), U = T S (a thread per
// column), X -= V U (a thread per element).  No shuffles.
__device__ void bt_blk(const cplx* __restrict__ A, int n, const cplx* __restrict__ Tg,
                       const double* __restrict__ Q, int k, cplx* __restrict__ X, Sh& sh) {
    cplx* S = sh.buf;  // BT_G x k, k <= QJ_GMAX
    const int tid = threadIdx.x;
    for (int e = tid; e < n * k; e += QT) X[e] = cmk(Q[e], 0.0);
    __syncthreads();
    const int ngroups = (n - 1 + BT_G - 1) / BT_G;
    for (int q = ngroups - 1; q >= 0; --q) {
        const int a = q * BT_G;
        const int nr = min(BT_G, (n - 1) - a);
        for (int p = tid; p < nr * k; p += QT) {
            const int r = p % nr, c = p / nr;
            const cplx* x = X + (size_t)c * n;
            double sr0 = 0.0, si0 = 0.0, sr1 = 0.0, si1 = 0.0;
            int i = a + 1 + r;  // v_r[i] = 0 above a + r + 1
            {
                const cplx xi = x[i];  // v_r[a + r + 1] = 1
                sr0 = xi.x;
                si0 = xi.y;
                ++i;
            }
            for (; i + 1 < n; i += 2) {
                const cplx v0 = A[i + (size_t)n * (a + r)], x0 = x[i];
                const cplx v1 = A[i + 1 + (size_t)n * (a + r)], x1 = x[i + 1];
                sr0 = fma(v0.x, x0.x, fma(v0.y, x0.y, sr0));
                si0 = fma(v0.x, x0.y, fma(-v0.y, x0.x, si0));
                sr1 = fma(v1.x, x1.x, fma(v1.y, x1.y, sr1));
                si1 = fma(v1.x, x1.y, fma(-v1.y, x1.x, si1));
            }
            if (i < n) {
                const cplx v0 = A[i + (size_t)n * (a + r)], x0 = x[i];
                sr0 = fma(v0.x, x0.x, fma(v0.y, x0.y, sr0));
                si0 = fma(v0.x, x0.y, fma(-v0.y, x0.x, si0));
            }
            S[r + BT_G * c] = cmk(sr0 + sr1, si0 + si1);
        }
        __syncthreads();
        const cplx* T = Tg + q * BT_G * BT_G;
        for (int c = tid; c < k; c += QT) {  // U = T S, T upper triangular
            cplx s[BT_G], u[BT_G];
#pragma unroll
            for (int r = 0; r < BT_G; ++r) s[r] = r < nr ? S[r + BT_G * c] : cmk(0, 0);
#pragma unroll
            for (int r = 0; r < BT_G; ++r) {
                cplx acc = cmk(0, 0);
#pragma unroll
                for (int v = r; v < BT_G; ++v) acc = cfma(T[r + BT_G * v], s[v], acc);
                u[r] = acc;
            }
#pragma unroll
            for (int r = 0; r < BT_G; ++r)
                if (r < nr) S[r + BT_G * c] = u[r];
        }
        __syncthreads();
        const int rows = n - (a + 1);
        for (int e = tid; e < rows * k; e += QT) {
            const int i = a + 1 + e % rows, c = e / rows;
            cplx xi = X[i + (size_t)n * c];
#pragma unroll
            for (int r = 0; r < BT_G; ++r) {
                if (r < nr && i >= a + r + 1) {
                    const cplx v = refl(A, n, a + r, i), u = S[r + BT_G * c];
                    xi.x = fma(-u.x, v.x, fma(u.y, v.y, xi.x));
                    xi.y = fma(-u.x, v.y, fma(-u.y, v.x, xi.y));
                }
            }
            X[i + (size_t)n * c] = xi;
        }
        __syncthreads();
    }
}

// Top `want` eigenpairs of the n x n Hermitian G (both triangles; destroyed):
// s.lama[want-1-g] and s.V[:, g] (n x want) hold the g-th largest.
__device__ __noinline__ void eig_blk(Traj& T, cplx* G, int n, int want) {
    Scr& s = T.s;
    Sh& sh = *T.sh;
    const int tid = threadIdx.x, lane = tid & 31;
    if (n >= 2) {
        hetrd_blk(G, n, s.d, s.e, s.tau, sh);
    } else {
        if (tid == 0) s.d[0] = G[0].x;
        __syncthreads();
    }
    {
        double* b3 = reinterpret_cast<double*>(sh.buf);
        tri_bounds_block(s.d, s.e, n, s.bounds, s.d32, s.e2f, s.e2, b3, b3 + QT, b3 + 2 * QT);
        __syncthreads();
    }
    // two lanes per eigenvalue: 27 % fewer FP64 Sturm counts than four
    for (int base = 0; base < want * 2; base += QT) {
        const int gt = base + tid, g = gt / 2, m = gt % 2;
        const unsigned grp = 0x3u << (lane & ~1);
        if (g < want)
            bisect_group_w<2>(g, m, grp, s.d, s.e2, s.d32, s.e2f, n, want, s.bounds, s.lamd, s.lama);
    }
    __syncthreads();
    if (tid == 0) separate_shifts_serial(s.lamd, want, s.bounds, s.shift);
    __syncthreads();
    for (int g = tid; g < want; g += QT)
        stein_vector(g, s.d, s.e, n, want, s.shift, s.bounds, s.f1, s.f2, s.f3, s.fl, s.piv, s.zw,
                     s.Z);
    __syncthreads();
    if (want > 1) {
        qr_blk(s.Z, n, want, s.qtau, s.rdiag, sh);
        for (int c = tid; c < want; c += QT) qr_form_thread(c, s.Z, n, s.qtau, s.rdiag, s.Q);
    } else {
        for (int i = tid; i < n; i += QT) s.Q[i] = s.Z[i];
    }
    const int ngroups = (n - 1 + BT_G - 1) / BT_G;
    for (int q = tid; q < ngroups; q += QT) wy_thread(q, G, n, s.tau, s.wyT);
    __syncthreads();
    bt_blk(G, n, s.wyT, s.Q, want, s.V, sh);
}

// Keep rule (src/tensors.jl:200-215) on the ascending top eigenvalues lam
// (want of them) with the Gram trace for the weight below them.
__device__ __noinline__ int keep_blk(const double* __restrict__ lam, int want, double trace, const TruncD& tr,
                        Sh& sh) {
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int i = 0; i < want; ++i) acc += fmax(lam[i], 0.0);  // smallest first
        const double rest = fmax(trace - acc, 0.0), total = acc + rest;
        int cnt = 0;
        double tail = rest;
        for (int i = want - 1; i >= 0; --i) {  // descending index i: lam[want-1-i]
            tail += fmax(lam[want - 1 - i], 0.0);
            if (tail / total > tr.cutoff) ++cnt;  // NaN (total 0) compares false
        }
        const int mind = min(tr.mindim, want);
        int maxd = (tr.maxdim == 0 || tr.maxdim > want) ? want : tr.maxdim;
        if (maxd == 0) maxd = 1;
        if (tr.cutoff != 0.0) maxd = min(maxd, cnt > 0 ? cnt : 1);
        sh.k = max(maxd, mind);
    }
    __syncthreads();
    return sh.k;
}

// Truncated split of th (m x n, ld m; scratch) (trunc_split): X (m x k) to Xo
// (ld m), Y (k x n) to Yo (ld k); returns k, or -1 past the capacity kcap.
__device__ __noinline__ int split_blk(Traj& T, const cplx* th, int m, int n, bool left_iso, const TruncD& tr,
                         cplx* Xo, cplx* Yo, int kcap) {
    Scr& s = T.s;
    Sh& sh = *T.sh;
    const int g = left_iso ? m : n, sz = min(m, n);
    bgram(left_iso, m, n, th, s.G);
    T.fl += 4.0 * g * (g + 1) * (double)(left_iso ? n : m);  // lower triangle
    double trace = 0.0;
    for (int i = threadIdx.x; i < g; i += QT) trace += s.G[i + (size_t)g * i].x;
    trace = bsum(trace, sh);
    const int maxd = (tr.maxdim <= 0 || tr.maxdim > sz) ? sz : tr.maxdim;
    const int want = min(sz, max(maxd, tr.mindim));
    eig_blk(T, s.G, g, want);
    T.fl += 16.0 / 3.0 * g * g * (double)g + 8.0 * g * g * (double)want;  // LAPACK count
    const int k = keep_blk(s.lama, want, trace, tr, sh);
    if (k > kcap) {
        set_flag(sh, QE_CAPACITY);
        return -1;
    }
    if (left_iso) {  // X = V_k, Y = V_k^H th
        for (int e = threadIdx.x; e < m * k; e += QT) Xo[e] = s.V[e];
        bgemm<OC, ON>(k, n, m, s.V, m, th, m, Yo, k);
        T.fl += 8.0 * k * n * (double)m;
    } else {  // X = th V_k, Y = V_k^H
        bgemm<ON, ON>(m, k, n, th, m, s.V, n, Xo, m);
        T.fl += 8.0 * m * k * (double)n;
        for (int e = threadIdx.x; e < k * n; e += QT) {
            const int r = e % k, c = e / k;
            Yo[r + k * c] = cconj(s.V[c + (size_t)n * r]);
        }
        __syncthreads();
    }
    return k;
}

// ---- gauge moves, gates, norm (gmps.jl:29-112, gatelist.jl:137-171) -------------
__device__ __noinline__ void moveright(Traj& T, int idx, const TruncD& tr) {
    const QjParams& p = *T.p;
    if (!(0 < idx && idx < p.N)) return;
    const int d = p.d, Dl = T.dl(idx), Dr = T.dr(idx), Dr2 = T.dr(idx + 1);
    bcopy(T.s.th, T.A(idx), Dl * d * Dr);
    const int k = split_blk(T, T.s.th, Dl * d, Dr, true, tr, T.A(idx), T.s.tmp, p.cap[idx]);
    if (k < 0) return;
    bgemm<ON, ON>(k, d * Dr2, Dr, T.s.tmp, k, T.A(idx + 1), Dr, T.s.th2, k);
    T.fl += 8.0 * k * d * Dr2 * (double)Dr;
    bcopy(T.A(idx + 1), T.s.th2, k * d * Dr2);
    if (threadIdx.x == 0) T.sh->dims[idx] = k;
    __syncthreads();
}

__device__ __noinline__ void moveleft(Traj& T, int idx, const TruncD& tr) {
    const QjParams& p = *T.p;
    if (!(1 < idx && idx <= p.N)) return;
    const int d = p.d, Dl = T.dl(idx), Dr = T.dr(idx), Dl0 = T.dl(idx - 1);
    bcopy(T.s.th, T.A(idx), Dl * d * Dr);
    const int k = split_blk(T, T.s.th, Dl, d * Dr, false, tr, T.s.tmp, T.A(idx), p.cap[idx - 1]);
    if (k < 0) return;
    bgemm<ON, ON>(Dl0 * d, k, Dl, T.A(idx - 1), Dl0 * d, T.s.tmp, Dl, T.s.th2, Dl0 * d);
    T.fl += 8.0 * Dl0 * d * k * (double)Dl;
    bcopy(T.A(idx - 1), T.s.th2, Dl0 * d * k);
    if (threadIdx.x == 0) T.sh->dims[idx - 1] = k;
    __syncthreads();
}

__device__ void movecenter(Traj& T, int idx, const TruncD& tr) {
    const int N = T.p->N;
    Sh& sh = *T.sh;
    const int c = sh.center;
    if (c == 0) {
        for (int i = 1; i <= idx - 1 && !sh.flag; ++i) moveright(T, i, tr);
        for (int i = 1; i <= N - idx && !sh.flag; ++i) moveleft(T, N + 1 - i, tr);
    } else if (idx > c) {
        for (int i = c; i <= idx - 1 && !sh.flag; ++i) moveright(T, i, tr);
    } else if (idx < c) {
        for (int i = 1; i <= c - idx && !sh.flag; ++i) moveleft(T, c + 1 - i, tr);
    }
    __syncthreads();
    if (threadIdx.x == 0) sh.center = idx;
    __syncthreads();
}

__device__ __noinline__ void gate2(Traj& T, int site, const cplx* M, bool direction, const TruncD& tr) {
    const QjParams& p = *T.p;
    const int d = p.d, d2 = d * d, Dl = T.dl(site), Dm = T.dr(site), Dr = T.dr(site + 1);
    bgemm<ON, ON>(Dl * d, d * Dr, Dm, T.A(site), Dl * d, T.A(site + 1), Dm, T.s.th, Dl * d);
    bapply(T.s.th, T.s.th2, M, d2, d2, Dl, Dr);
    T.fl += 8.0 * Dl * d * d * (double)Dr * Dm + 8.0 * Dl * Dr * (double)d2 * d2;
    const int k = split_blk(T, T.s.th2, Dl * d, d * Dr, !direction, tr, T.A(site), T.A(site + 1),
                            p.cap[site]);
    if (k < 0) return;
    if (threadIdx.x == 0) {
        T.sh->dims[site] = k;
        T.sh->center = direction ? site : site + 1;
    }
    __syncthreads();
}

__device__ void site_op(Traj& T, int site, const cplx* M) {
    const int d = T.p->d, Dl = T.dl(site), Dr = T.dr(site);
    bapply(T.A(site), T.s.tmp, M, d, d, Dl, Dr);
    T.fl += 8.0 * Dl * Dr * (double)d * d;
    bcopy(T.A(site), T.s.tmp, Dl * d * Dr);
}

__device__ void gate1(Traj& T, int site, const cplx* M, bool direction) {
    site_op(T, site, M);
    const int nxt = site + 1 - 2 * (direction ? 1 : 0);
    if (0 < nxt && nxt <= T.p->N) movecenter(T, nxt, TruncD{0.0, 0, 1});
}

__device__ void applygates(Traj& T) {
    const QjParams& p = *T.p;
    Sh& sh = *T.sh;
    for (int r = 0; r < p.nrows && !sh.flag; ++r) {
        const int s0 = p.row_start[r], len = p.row_len[r];
        if (len == 0) continue;
        const int first = p.gsite[s0];
        const int last = p.gsite[s0 + len - 1] + p.gns[s0 + len - 1] - 1;
        const int c = sh.center;
        const bool direction = !(abs(c - first) < abs(c - last));
        for (int i = 0; i < len && !sh.flag; ++i) {
            const int gi = s0 + (direction ? len - 1 - i : i);
            const int ctr = direction ? p.gsite[gi] + p.gns[gi] - 1 : p.gsite[gi];
            movecenter(T, ctr, T.tr);
            if (sh.flag) break;
            if (p.gns[gi] == 1)
                gate1(T, p.gsite[gi], p.gM[gi], direction);
            else
                gate2(T, p.gsite[gi], p.gM[gi], direction, T.tr);
        }
    }
}

// Normalises the centre tensor; returns the squared norm before scaling.
__device__ __noinline__ double normalize(Traj& T) {
    Sh& sh = *T.sh;
    if (sh.center == 0) movecenter(T, 1, TruncD{0.0, 0, 1});
    const int c = sh.center, n = T.dl(c) * T.p->d * T.dr(c);
    cplx* A = T.A(c);
    double n2 = 0.0;
    for (int e = threadIdx.x; e < n; e += QT) n2 = fma(A[e].x, A[e].x, fma(A[e].y, A[e].y, n2));
    n2 = bsum(n2, sh);
    const double inv = 1.0 / sqrt(n2);
    for (int e = threadIdx.x; e < n; e += QT) A[e] = cmk(A[e].x * inv, A[e].y * inv);
    __syncthreads();
    return n2;
}

// rho[s + D s'] = sum_{a,b} conj(A[a,s,b]) Y[a,s',b] (A, Y: Dl x D x Dr); the
// D x D partial sums stay in registers (compile-time indices).
template <int D>
__device__ __noinline__ void rho_contract_t(const cplx* __restrict__ A, const cplx* __restrict__ Y, int Dl,
                               int Dr, cplx* __restrict__ rho, Sh& sh) {
    double acc[2 * D * D];
#pragma unroll
    for (int q = 0; q < 2 * D * D; ++q) acc[q] = 0.0;
    for (int e = threadIdx.x; e < Dl * Dr; e += QT) {
        const int a = e % Dl, b = e / Dl;
        const cplx* ab = A + a + (size_t)Dl * D * b;
        const cplx* yb = Y + a + (size_t)Dl * D * b;
        cplx x[D], y[D];
#pragma unroll
        for (int s = 0; s < D; ++s) {
            x[s] = ab[Dl * s];
            y[s] = yb[Dl * s];
        }
#pragma unroll
        for (int s = 0; s < D; ++s)
#pragma unroll
            for (int s2 = 0; s2 < D; ++s2) {
                const int q = s + D * s2;
                acc[2 * q] = fma(x[s].x, y[s2].x, fma(x[s].y, y[s2].y, acc[2 * q]));
                acc[2 * q + 1] = fma(x[s].x, y[s2].y, fma(-x[s].y, y[s2].x, acc[2 * q + 1]));
            }
    }
    // 8 sums at a time through shared memory: 64 threads add QT/8 each, 8 add 8
    double* part = reinterpret_cast<double*>(sh.buf);  // QT x 8 values, then 64 partials
#pragma unroll
    for (int q0 = 0; q0 < 2 * D * D; q0 += 8) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q0 + q < 2 * D * D) part[threadIdx.x + QT * q] = acc[q0 + q];
        __syncthreads();
        double v = 0.0;
        if (threadIdx.x < 64) {
            const int q = threadIdx.x & 7, h = threadIdx.x >> 3, per = QT / 8;
            double a = 0.0, b = 0.0;
            for (int i = h * per; i < h * per + per; i += 2) {
                a += part[i + QT * q];
                b += part[i + 1 + QT * q];
            }
            v = a + b;
        }
        __syncthreads();
        if (threadIdx.x < 64) part[threadIdx.x] = v;
        __syncthreads();
        if (threadIdx.x < 8 && q0 + (int)threadIdx.x < 2 * D * D) {
            double t = 0.0;
            for (int h = 0; h < 8; ++h) t += part[threadIdx.x + 8 * h];
            reinterpret_cast<double*>(rho)[q0 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

__device__ void rho_contract(const cplx* A, const cplx* Y, int Dl, int d, int Dr, cplx* rho,
                             Sh& sh) {
    switch (d) {
        case 1: rho_contract_t<1>(A, Y, Dl, Dr, rho, sh); break;
        case 2: rho_contract_t<2>(A, Y, Dl, Dr, rho, sh); break;
        case 3: rho_contract_t<3>(A, Y, Dl, Dr, rho, sh); break;
        default: rho_contract_t<4>(A, Y, Dl, Dr, rho, sh); break;
    }
}

// One-site reduced density matrices of every site (s.rho, d x d each) of the
// normalised MPS in canonical form about its centre c >= 1: left blocks are
// the identity left of c and right blocks right of it.
__device__ __noinline__ void rho_all(Traj& T) {
    const QjParams& p = *T.p;
    Sh& sh = *T.sh;
    const int N = p.N, d = p.d, c = sh.center;
    cplx* B = T.s.G;    // running block
    cplx* Bn = T.s.th;  // next block
    cplx* Y = T.s.V;
    {  // rightward from c with L = I
        const int D = T.dl(c);
        for (int e = threadIdx.x; e < D * D; e += QT) B[e] = cmk(e % (D + 1) == 0 ? 1.0 : 0.0, 0.0);
        __syncthreads();
    }
    for (int i = c; i <= N; ++i) {
        const int Dl = T.dl(i), Dr = T.dr(i);
        bgemm<ON, ON>(Dl, d * Dr, Dl, B, Dl, T.A(i), Dl, Y, Dl);
        rho_contract(T.A(i), Y, Dl, d, Dr, T.s.rho + (size_t)(i - 1) * d * d, sh);
        T.fl += 8.0 * Dl * Dl * (double)d * Dr + 8.0 * Dl * Dr * (double)d * d;
        if (i < N) {
            bgemm<OC, ON>(Dr, Dr, Dl * d, T.A(i), Dl * d, Y, Dl * d, Bn, Dr);
            T.fl += 8.0 * Dr * Dr * (double)Dl * d;
            cplx* t = B;
            B = Bn;
            Bn = t;
        }
    }
    {  // leftward from c with R = I
        const int D = T.dr(c);
        for (int e = threadIdx.x; e < D * D; e += QT) B[e] = cmk(e % (D + 1) == 0 ? 1.0 : 0.0, 0.0);
        __syncthreads();
    }
    for (int i = c; i >= 1; --i) {
        const int Dl = T.dl(i), Dr = T.dr(i);
        bgemm<ON, OT>(Dl * d, Dr, Dr, T.A(i), Dl * d, B, Dr, Y, Dl * d);
        T.fl += 8.0 * Dl * d * Dr * (double)Dr;
        if (i < c) {
            rho_contract(T.A(i), Y, Dl, d, Dr, T.s.rho + (size_t)(i - 1) * d * d, sh);
            T.fl += 8.0 * Dl * Dr * (double)d * d;
        }
        if (i > 1) {
            bgemm<OR, OT>(Dl, Dl, d * Dr, T.A(i), Dl, Y, Dl, Bn, Dl);
            T.fl += 8.0 * Dl * Dl * (double)d * Dr;
            cplx* t = B;
            B = Bn;
            Bn = t;
        }
    }
}

// sum_{s,s'} rho[s + d s'] O[s, s'] with M the small_apply form (O[s, s'] = M[s' + d s])
__device__ __forceinline__ cplx expect(const cplx* rho, const cplx* M, int d) {
    cplx acc = cmk(0, 0);
    for (int s = 0; s < d; ++s)
        for (int s2 = 0; s2 < d; ++s2) acc = cfma(rho[s + d * s2], M[s2 + d * s], acc);
    return acc;
}

__device__ bool draw(Traj& T, double& u) {
    const QjParams& p = *T.p;
    if (p.draws) {
        if ((int64_t)T.used >= p.ndraws) return false;
        u = p.draws[(size_t)T.t * p.ndraws + T.used];
    } else {
        u = philox_uniform(p.seed, T.trajno, T.used);
    }
    ++T.used;
    return true;
}

// Emission rates |c_j|^2 |<L_j^dag L_j>| (qjmc.jl:170-220) from s.rho; every
// thread computes the same values.
__device__ double rate(const Traj& T, int j) {
    const QjParams& p = *T.p;
    const int d = p.d;
    const cplx v = expect(T.s.rho + (size_t)(p.jsite[j] - 1) * d * d, p.jLdL + (size_t)j * d * d, d);
    return p.jw[j] * sqrt(v.x * v.x + v.y * v.y);
}

__device__ void run_traj(const QjParams& p, Sh& sh, int t, int slot) {
    Traj T;
    T.p = &p;
    T.sh = &sh;
    T.mps = p.mps_pool + (size_t)slot * p.mps_slot;
    scr_layout(p.scr_pool + (size_t)slot * p.scr_slot, p.gmax, p.N, p.d, T.s);
    T.used = 0;
    T.trajno = p.first_traj + (uint32_t)t;
    T.t = t;
    T.tr = TruncD{p.cutoff, p.maxdim, p.mindim};
    T.fl = 0.0;
    const int N = p.N, d = p.d;
    for (int i = 1; i <= N; ++i) {
        const int n = p.psi0_dims[i - 1] * d * p.psi0_dims[i];
        cplx* dst = T.A(i);
        const cplx* src = p.psi0[i - 1];
        for (int e = threadIdx.x; e < n; e += QT) dst[e] = src[e];
    }
    for (int i = threadIdx.x; i <= N; i += QT) sh.dims[i] = p.psi0_dims[i];
    if (threadIdx.x == 0) {
        sh.center = p.psi0_center;
        sh.flag = QE_OK;
    }
    __syncthreads();
    double time = 0.0;
    int nj = 0, row = 1;
    for (int step = 1; step <= p.nsteps; ++step) {
        applygates(T);
        if (sh.flag) break;
        double u;
        if (!draw(T, u)) {  // qjmc.jl:64; the jump decision when not classical
            set_flag(sh, QE_DRAWS);
            break;
        }
        const double n2 = normalize(T);
        if (sh.flag) break;
        bool want = false, rho_fresh = false;
        double er = 0.0;
        if (p.classical) {
            rho_all(T);
            rho_fresh = true;
            for (int j = 0; j < p.njump; ++j) er += rate(T, j);
            const double prob = exp(-er * p.dt);
            double u2;
            if (!draw(T, u2)) {
                set_flag(sh, QE_DRAWS);
                break;
            }
            want = u2 > prob;
        } else {
            want = u > n2;  // the squared norm of the unnormalised state
            if (want) {
                rho_all(T);
                rho_fresh = true;
                for (int j = 0; j < p.njump; ++j) er += rate(T, j);
            }
        }
        if (want) {
            double r;
            if (!draw(T, r)) {
                set_flag(sh, QE_DRAWS);
                break;
            }
            int idx = -1;
            double cum = 0.0;
            for (int j = 0; j < p.njump; ++j) {
                cum += rate(T, j);
                if (r < cum / er) {
                    idx = j;
                    break;
                }
            }
            if (idx < 0) {
                set_flag(sh, QE_NOCHANNEL);
                break;
            }
            __syncthreads();  // every thread has read s.rho
            const TruncD none{0.0, 0, 1};
            movecenter(T, 1, none);
            site_op(T, p.jsite[idx], p.jL + (size_t)idx * d * d);
            movecenter(T, N, none);
            movecenter(T, 1, T.tr);
            if (sh.flag) break;
            normalize(T);
            if (nj >= p.maxj) {
                set_flag(sh, QE_JUMPS);
                break;
            }
            if (threadIdx.x == 0) {
                p.jump_ch[(size_t)t * p.maxj + nj] = idx + 1;
                p.jump_time[(size_t)t * p.maxj + nj] = time + p.dt;
            }
            ++nj;
            rho_fresh = false;
        }
        time += p.dt;
        if (step % p.save_every == 0 && p.nobs > 0) {
            if (!rho_fresh) rho_all(T);
            for (int k = threadIdx.x; k < p.nobs; k += QT)
                p.obs_traj[((size_t)t * p.nrows_out + row) * p.nobs + k] =
                    expect(T.s.rho + (size_t)(p.osite[k] - 1) * d * d, p.oO + (size_t)k * d * d, d);
            ++row;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        p.err[t] = sh.flag;
        p.njumps[t] = nj;
        p.used[t] = (int64_t)T.used;
        p.flops[t] = T.fl;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(QT, 4) qjmc_engine_kernel(QjParams p) {
    __shared__ Sh sh;
    for (int t = blockIdx.x; t < p.ntraj; t += gridDim.x) run_traj(p, sh, t, blockIdx.x);
}

// obs_avg[row, k] = sum_t obs_traj[t, row, k] / ntraj for rows >= 1, trajectory order
__global__ void obs_reduce_kernel(const cplx* __restrict__ obs_traj, int ntraj, int nrows, int nobs,
                                  cplx* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (nrows - 1) * nobs) return;
    const int row = 1 + e / nobs, k = e % nobs;
    double re = 0.0, im = 0.0;
    for (int t = 0; t < ntraj; ++t) {
        const cplx v = obs_traj[((size_t)t * nrows + row) * nobs + k];
        re += v.x;
        im += v.y;
    }
    out[(size_t)row * nobs + k] = cmk(re / ntraj, im / ntraj);
}

template <class T>
DBuf upload(Ctx* ctx, const std::vector<T>& v) {
    DBuf b(ctx, sizeof(T) * std::max<size_t>(v.size(), 1));
    if (!v.empty())
        TN_CHECK_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice,
                                      ctx->stream));
    return b;
}

// small_apply form M[i + d o] = op[o, i] of an interleaved column-major d x d operator
std::vector<cplx> apply_form(const double* op, int d) {
    std::vector<cplx> M((size_t)d * d);
    for (int o = 0; o < d; ++o)
        for (int i = 0; i < d; ++i) {
            const double* e = op + 2 * (o + (size_t)d * i);
            M[i + (size_t)d * o] = cmk(e[0], e[1]);
        }
    return M;
}

}  // namespace

// Host side of the engine: capacities, slots, operator uploads, one launch of
// qjmc_engine_kernel and one of the trajectory-order reduction.
void qjmc_ensemble(const tn_mps* psi0, const tn_gates* g, int njump, const int* jsites,
                   const double* jops, const double* jcoeffs, int nsteps, double dt, int ntraj,
                   const double* draws, int64_t ndraws_per_traj, uint64_t seed, uint32_t first_traj,
                   const Trunc& t, int save_every, int nobs, const int* obs_sites,
                   const double* obs_ops, double* obs_avg, int* njumps_per_traj, int max_jumps,
                   int* jumps, double* jumptimes, int blocks_per_sm, double* stats,
                   bool classical) {
    Ctx* ctx = psi0->ctx;
    const int N = psi0->N, d = psi0->d;
    TN_REQUIRE(g->N == N && g->d == d, "GateList and MPS do not match.");
    TN_REQUIRE(d <= QJ_DMAX, "the trajectory engine takes physical dimensions up to 4");
    TN_REQUIRE(N >= 1 && N <= QJ_NMAX, "the trajectory engine takes up to 1024 sites");
    TN_REQUIRE(t.maxdim >= 1, "the trajectory engine needs maxdim >= 1 (it sizes the slots)");
    TN_REQUIRE(t.mindim >= 1 && t.mindim <= t.maxdim, "mindim must lie in [1, maxdim]");
    TN_REQUIRE(ntraj >= 1 && nsteps >= 0 && save_every >= 1, "bad trajectory counts");
    TN_REQUIRE(njump >= 1 && nobs >= 0 && max_jumps >= 0, "bad operator counts");
    TN_REQUIRE(draws == nullptr || ndraws_per_traj >= 1, "need at least one draw per trajectory");
    TN_REQUIRE(blocks_per_sm >= 1 && blocks_per_sm <= 8, "blocks_per_sm must lie in [1, 8]");
    for (size_t i = 0; i < g->nsites.size(); ++i)
        TN_REQUIRE(g->nsites[i] == 1 || g->nsites[i] == 2,
                   "the trajectory engine applies one- and two-site gates");
    for (int j = 0; j < njump; ++j)
        TN_REQUIRE(jsites[j] >= 1 && jsites[j] <= N, "jump site out of range");
    for (int k = 0; k < nobs; ++k)
        TN_REQUIRE(obs_sites[k] >= 1 && obs_sites[k] <= N, "observable site out of range");
    // bond capacities: maxdim, or the initial state's bond where larger
    std::vector<int> cap(N + 1);
    int capmax = 1;
    for (int i = 0; i <= N; ++i) {
        const int64_t b = psi0->dims[i];
        cap[i] = (i == 0 || i == N) ? (int)b : (int)std::max<int64_t>(t.maxdim, b);
        capmax = std::max(capmax, cap[i]);
    }
    TN_REQUIRE((int64_t)d * capmax <= QJ_GMAX,
               "the trajectory engine takes d x bond dimension up to 256");
    const int gmax = d * capmax;
    std::vector<int64_t> cap_off(N);
    int64_t off = 0;
    for (int i = 1; i <= N; ++i) {
        cap_off[i - 1] = off;
        off += (int64_t)cap[i - 1] * d * cap[i];
    }
    const int64_t mps_slot = (off + 15) / 16 * 16;
    Scr dummy;
    const int64_t scr_slot = (int64_t)scr_layout(nullptr, gmax, N, d, dummy);
    int slots = (int)std::min<int64_t>(ntraj, (int64_t)ctx->sm_count * blocks_per_sm);
    {
        // slots beyond what fits in 80 % of the free device memory run as
        // later waves of the same blocks instead
        size_t free_b = 0, total_b = 0;
        TN_CHECK_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const double per_slot = (double)sizeof(cplx) * mps_slot + (double)scr_slot;
        const int64_t fit = (int64_t)(0.8 * (double)free_b / per_slot);
        TN_REQUIRE(fit >= 1, "one trajectory slot does not fit in the free device memory");
        slots = (int)std::min<int64_t>(slots, fit);
    }
    const int nrows_out = nsteps / save_every + 1;

    // gates
    std::vector<int> row_start(g->row_start.begin(), g->row_start.end());
    std::vector<int> row_len(g->row_len.begin(), g->row_len.end());
    std::vector<int> gsite(g->sites.begin(), g->sites.end()), gns(g->nsites.begin(), g->nsites.end());
    std::vector<const cplx*> gM(g->M.size());
    for (size_t i = 0; i < g->M.size(); ++i) gM[i] = g->M[i].c();
    // jump channels and observables
    std::vector<cplx> jL, jLdL, oO;
    std::vector<double> jw(njump);
    std::vector<int> js(jsites, jsites + njump), os(obs_sites, obs_sites + nobs);
    for (int j = 0; j < njump; ++j) {
        const double* op = jops + 2 * (size_t)d * d * j;
        std::vector<cplx> a = apply_form(op, d);
        std::vector<double> ldl(2 * (size_t)d * d, 0.0);
        for (int i = 0; i < d; ++i)  // (L^dag L)[i, l] = sum_k conj(L[k, i]) L[k, l]
            for (int l = 0; l < d; ++l) {
                double re = 0.0, im = 0.0;
                for (int k = 0; k < d; ++k) {
                    const double ar = op[2 * (k + d * i)], ai = -op[2 * (k + d * i) + 1];
                    const double br = op[2 * (k + d * l)], bi = op[2 * (k + d * l) + 1];
                    re += ar * br - ai * bi;
                    im += ar * bi + ai * br;
                }
                ldl[2 * (i + (size_t)d * l)] = re;
                ldl[2 * (i + (size_t)d * l) + 1] = im;
            }
        std::vector<cplx> b = apply_form(ldl.data(), d);
        jL.insert(jL.end(), a.begin(), a.end());
        jLdL.insert(jLdL.end(), b.begin(), b.end());
        const double cr = jcoeffs[2 * j], ci = jcoeffs[2 * j + 1];
        jw[j] = cr * cr + ci * ci;
    }
    for (int k = 0; k < nobs; ++k) {
        std::vector<cplx> a = apply_form(obs_ops + 2 * (size_t)d * d * k, d);
        oO.insert(oO.end(), a.begin(), a.end());
    }
    std::vector<const cplx*> p0(N);
    std::vector<int> p0dims(N + 1);
    for (int i = 1; i <= N; ++i) p0[i - 1] = psi0->site(i);
    for (int i = 0; i <= N; ++i) p0dims[i] = (int)psi0->dims[i];

    DBuf d_rs = upload(ctx, row_start), d_rl = upload(ctx, row_len), d_gs = upload(ctx, gsite),
         d_gn = upload(ctx, gns), d_gM = upload(ctx, gM), d_js = upload(ctx, js),
         d_jL = upload(ctx, jL), d_jLdL = upload(ctx, jLdL), d_jw = upload(ctx, jw),
         d_os = upload(ctx, os), d_oO = upload(ctx, oO), d_p0 = upload(ctx, p0),
         d_p0d = upload(ctx, p0dims), d_coff = upload(ctx, cap_off), d_cap = upload(ctx, cap);
    DBuf d_draws;
    if (draws) {
        d_draws = DBuf(ctx, sizeof(double) * (size_t)ntraj * ndraws_per_traj);
        TN_CHECK_CUDA(cudaMemcpyAsync(d_draws.p, draws, d_draws.bytes, cudaMemcpyHostToDevice,
                                      ctx->stream));
    }
    // jump records: max_jumps per trajectory, or one per step when none are returned
    const int maxj = max_jumps > 0 ? max_jumps : nsteps + 1;
    DBuf mps_pool(ctx, sizeof(cplx) * (size_t)mps_slot * slots);
    DBuf scr_pool(ctx, (size_t)scr_slot * slots);
    DBuf obs_traj(ctx, sizeof(cplx) * (size_t)ntraj * nrows_out * std::max(nobs, 1));
    DBuf d_nj(ctx, sizeof(int) * ntraj), d_jc(ctx, sizeof(int) * (size_t)ntraj * maxj),
        d_jt(ctx, sizeof(double) * (size_t)ntraj * maxj), d_err(ctx, sizeof(int) * ntraj),
        d_used(ctx, sizeof(int64_t) * ntraj), d_fl(ctx, sizeof(double) * ntraj), d_avg(ctx, sizeof(cplx) * (size_t)nrows_out * std::max(nobs, 1));

    QjParams p{};
    p.N = N;
    p.d = d;
    p.nsteps = nsteps;
    p.save_every = save_every;
    p.nobs = nobs;
    p.njump = njump;
    p.maxj = maxj;
    p.nrows_out = nrows_out;
    p.classical = classical ? 1 : 0;
    p.dt = dt;
    p.cutoff = t.cutoff;
    p.maxdim = (int)t.maxdim;
    p.mindim = (int)t.mindim;
    p.nrows = (int)row_start.size();
    p.row_start = d_rs.as<int>();
    p.row_len = d_rl.as<int>();
    p.gsite = d_gs.as<int>();
    p.gns = d_gn.as<int>();
    p.gM = d_gM.as<const cplx*>();
    p.jsite = d_js.as<int>();
    p.jL = d_jL.c();
    p.jLdL = d_jLdL.c();
    p.jw = d_jw.d();
    p.osite = d_os.as<int>();
    p.oO = d_oO.c();
    p.psi0 = d_p0.as<const cplx*>();
    p.psi0_dims = d_p0d.as<int>();
    p.psi0_center = psi0->center;
    p.draws = draws ? d_draws.d() : nullptr;
    p.ndraws = ndraws_per_traj;
    p.seed = seed;
    p.first_traj = first_traj;
    p.ntraj = ntraj;
    p.mps_pool = mps_pool.c();
    p.mps_slot = mps_slot;
    p.cap_off = d_coff.as<int64_t>();
    p.cap = d_cap.as<int>();
    p.scr_pool = scr_pool.as<char>();
    p.scr_slot = scr_slot;
    p.gmax = gmax;
    p.obs_traj = obs_traj.c();
    p.njumps = d_nj.as<int>();
    p.jump_ch = d_jc.as<int>();
    p.jump_time = d_jt.d();
    p.err = d_err.as<int>();
    p.used = d_used.as<int64_t>();
    p.flops = d_fl.d();
    cudaEvent_t e0 = ctx->ev_get(), e1 = ctx->ev_get();
    TN_CHECK_CUDA(cudaEventRecord(e0, ctx->stream));
    qjmc_engine_kernel<<<slots, QT, 0, ctx->stream>>>(p);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    TN_CHECK_CUDA(cudaEventRecord(e1, ctx->stream));
    if (nobs > 0 && nrows_out > 1) {
        const int n = (nrows_out - 1) * nobs;
        obs_reduce_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(obs_traj.c(), ntraj, nrows_out,
                                                                   nobs, d_avg.c());
        ctx->count();
        TN_CHECK_CUDA(cudaGetLastError());
    }
    std::vector<int> err(ntraj), nj(ntraj);
    TN_CHECK_CUDA(cudaMemcpyAsync(err.data(), d_err.p, sizeof(int) * ntraj, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    TN_CHECK_CUDA(cudaMemcpyAsync(nj.data(), d_nj.p, sizeof(int) * ntraj, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    if (nobs > 0 && nrows_out > 1)
        TN_CHECK_CUDA(cudaMemcpyAsync(obs_avg + 2 * (size_t)nobs, d_avg.c() + nobs,
                                      sizeof(cplx) * (size_t)(nrows_out - 1) * nobs,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    if (jumps && max_jumps > 0)
        TN_CHECK_CUDA(cudaMemcpyAsync(jumps, d_jc.p, sizeof(int) * (size_t)ntraj * max_jumps,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    if (jumptimes && max_jumps > 0)
        TN_CHECK_CUDA(cudaMemcpyAsync(jumptimes, d_jt.p, sizeof(double) * (size_t)ntraj * max_jumps,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> fl(ntraj);
    TN_CHECK_CUDA(cudaMemcpyAsync(fl.data(), d_fl.p, sizeof(double) * ntraj, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    ctx->sync();
    float ms = 0.f;
    TN_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    ctx->ev_pool.push_back(e0);
    ctx->ev_pool.push_back(e1);
    if (stats) {
        double f = 0.0;
        for (double v : fl) f += v;
        stats[0] = f;
        stats[1] = ms;
        stats[2] = (double)ntraj * nsteps;
        stats[3] = slots;
    }
    for (int i = 0; i < ntraj; ++i) {
        switch (err[i]) {
            case QE_OK: break;
            case QE_CAPACITY:
                throw Error(TN_ERR_INVALID, "trajectory " + std::to_string(i) +
                                                ": a bond outgrew its slot capacity");
            case QE_DRAWS:
                throw Error(TN_ERR_INVALID, "trajectory " + std::to_string(i) +
                                                ": uniform draw stream exhausted");
            case QE_JUMPS:
                throw Error(TN_ERR_INVALID, "trajectory " + std::to_string(i) +
                                                ": jump record capacity exceeded");
            default:
                throw Error(TN_ERR_INVALID, "trajectory " + std::to_string(i) +
                                                ": no jump channel selected (all rates zero)");
        }
    }
    if (njumps_per_traj)
        for (int i = 0; i < ntraj; ++i) njumps_per_traj[i] = nj[i];
    // row 0: the initial state's expectation values, the same in every trajectory
    if (nobs > 0) {
        std::vector<DBuf> ops(nobs);
        std::vector<Term> terms(nobs);
        for (int k = 0; k < nobs; ++k) {
            upload_op_matrix(ctx, obs_ops + 2 * (size_t)d * d * k, d, ops[k]);
            terms[k].first = obs_sites[k];
            terms[k].len = 1;
            terms[k].dops = {ops[k].c()};
            terms[k].coeff = cmk(1, 0);
        }
        std::vector<cplx> v = inner_terms(ctx, psi0, psi0, terms);
        for (int k = 0; k < nobs; ++k) {
            obs_avg[2 * k] = v[k].x;
            obs_avg[2 * k + 1] = v[k].y;
        }
    }
}

}  // namespace tn
