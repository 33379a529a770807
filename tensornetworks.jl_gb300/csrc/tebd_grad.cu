// Hand-written adjoint of a TEBD evolution: gradient of a final-time one-site
// expectation value with respect to every gate of step-dependent gate lists.
//
// Forward (one step, as src/algorithms/mps/tebd.jl:61-84 with the gate
// schedule of applygates!, structures/mps/gatelist.jl:191-227):
//   truncating gauge moves (gmps.jl:60-112) before each gate, the gate
//   contraction (gatelist.jl:137-171), the truncated two-site split
//   (gmps.jl:199-267, keep rule tensors.jl:200-215), then normalize!.
// The objective is f = <psi|O|psi> / <psi|psi> with O on one site, evaluated
// at the orthogonality centre after non-truncating gauge moves.
//
// Backward rules (cotangents xbar = df/dRe x + i df/dIm x, df = Re<xbar, dx>):
//   C = A B               : Abar = Cbar B^H, Bbar = A^H Cbar
//   out = in . M (leg)    : inbar = outbar . M^H, Mbar = sum conj(in) outbar
//   c' = c / |c|          : cbar = (c'bar - Re<c', c'bar> c') / |c|
//   truncated split       : through the Gram eigendecomposition G = V diag(l) V^H
//     (left_iso: G = M M^H, X = top-k columns of V, Y = X^H M;
//      else:     G = M^H M, Vk = top-k columns, X = M Vk, Y = Vk^H)
//     Gbar = V (F o V^H Vbar) Vk^H with F_ij = x / (x^2 + eta lmax^2),
//     x = l_j - l_i, for i discarded and j kept, and 0 for kept-kept pairs:
//     the state depends on the kept subspace only, so the gauge block drops.
// Memory: the state is checkpointed every `every` steps; each segment is
// recomputed with its tape (inputs of every contraction, the Gram
// eigenvectors of every split) and then reversed.
#include <cmath>

#include "mps.cuh"

namespace tn {
namespace {

const cplx ONE = {1.0, 0.0};
const cplx ZERO = {0.0, 0.0};

inline int blocks_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    return (int)(b < 1 ? 1 : b);
}

// D[i + g j] = C[i + g j] * F(lam[g-1-j] - lam[i]) for discarded rows i < g-k,
// 0 for kept rows; F(x) = x / (x^2 + eta lmax^2)
__global__ void gap_weight_kernel(const cplx* __restrict__ C, const double* __restrict__ lam,
                                  int64_t g, int64_t k, double eta, cplx* __restrict__ D) {
    const double lmax = fmax(fabs(lam[g - 1]), 1e-300);
    const double e2 = eta * lmax * lmax;
    const int64_t total = g * k;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % g, j = idx / g;
        cplx v = cmk(0, 0);
        if (i < g - k) {
            const double x = lam[g - 1 - j] - lam[i];
            const double f = x / (x * x + e2);
            v = cmk(C[idx].x * f, C[idx].y * f);
        }
        D[idx] = v;
    }
}

// S = A + A^H (n x n)
__global__ void herm_sum_kernel(const cplx* __restrict__ A, int64_t n, cplx* __restrict__ S) {
    const int64_t total = n * n;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        const cplx a = A[idx], b = A[j + n * i];
        S[idx] = cmk(a.x + b.x, a.y - b.y);
    }
}

// y = (y - r x) * s
__global__ void axpy_scale_kernel(cplx* __restrict__ y, const cplx* __restrict__ x, double r,
                                  double s, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const cplx a = y[i], b = x[i];
        y[i] = cmk((a.x - r * b.x) * s, (a.y - r * b.y) * s);
    }
}

// y += a x (complex a)
__global__ void zaxpy_kernel(cplx* __restrict__ y, const cplx* __restrict__ x, cplx a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = cfma(a, x[i], y[i]);
}

// Mbar[I + nI J] += sum_{a,c} conj(in[a + lda I + ldc c]) * bar[a + lda J + ldcb c]
// one block per (I, J); deterministic warp-shuffle reduction
__global__ void __launch_bounds__(256) leg_grad_kernel(const cplx* __restrict__ in,
                                                       const cplx* __restrict__ bar, int nI,
                                                       int nJ, int64_t na, int64_t nc, int64_t lda,
                                                       int64_t ldc, int64_t ldcb,
                                                       cplx* __restrict__ Mbar) {
    __shared__ double sr[8], si[8];
    const int I = blockIdx.x % nI, J = blockIdx.x / nI;
    double re = 0.0, im = 0.0;
    for (int64_t idx = threadIdx.x; idx < na * nc; idx += blockDim.x) {
        const int64_t a = idx % na, c = idx / na;
        const cplx x = in[a + lda * I + ldc * c], y = bar[a + lda * J + ldcb * c];
        re = fma(x.x, y.x, fma(x.y, y.y, re));   // Re(conj(x) y)
        im = fma(x.x, y.y, fma(-x.y, y.x, im));  // Im(conj(x) y)
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_down_sync(0xffffffffu, re, o);
        im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sr[threadIdx.x >> 5] = re;
        si[threadIdx.x >> 5] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            tr += sr[w];
            ti += si[w];
        }
        Mbar[I + nI * J] = cadd(Mbar[I + nI * J], cmk(tr, ti));
    }
}

void check_launch(Ctx* ctx) {
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

cplx dot(Ctx* ctx, const cplx* x, const cplx* y, int64_t n) {  // sum conj(x) y
    cplx* d = ctx->s_coef.c(ctx, 16);
    const cplx* V[1] = {x};
    multi_dot(ctx, V, 1, y, n, d);
    cplx h;
    TN_CHECK_CUDA(cudaMemcpyAsync(&h, d, sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    return h;
}

DBuf dcopy(Ctx* ctx, const cplx* src, int64_t n) {
    DBuf b(ctx, sizeof(cplx) * std::max<int64_t>(n, 1));
    zcopy(ctx, b.c(), src, n);
    return b;
}

// ---- tape ------------------------------------------------------------------
struct SplitRec {
    int64_t m = 0, n = 0, k = 0, g = 0;
    bool left_iso = true;
    DBuf M, V, lam;  // input, all Gram eigenvectors (ascending), eigenvalues
};

enum class Kind { MoveR, MoveL, Gate2, Gate1, Normalize };

struct Op {
    Kind kind = Kind::MoveR;
    int site = 0;
    int64_t Dl = 0, Dm = 0, Dr = 0;
    SplitRec sp;
    DBuf a, b, theta;        // saved inputs (see each rule)
    const cplx* Mh = nullptr;  // gate M^H (small_apply form)
    cplx* gbar = nullptr;      // gate cotangent accumulator (small_apply form)
    int nI = 0;
    double norm = 0.0;
};
using Tape = std::vector<Op>;

// Truncated split with the full Gram eigensystem (same keep rule and
// projections as trunc_split).  rec != null keeps M, V and the eigenvalues.
int64_t split_full(Ctx* ctx, DBuf&& Min, int64_t m, int64_t n, const Trunc& t, bool left_iso,
                   DBuf& X, DBuf& Y, SplitRec* rec) {
    const int64_t sz = std::min(m, n), g = left_iso ? m : n;
    const cplx* M = Min.c();
    DBuf G(ctx, sizeof(cplx) * g * g), lam(ctx, sizeof(double) * (g + sz));
    if (left_iso)
        zgemm(ctx, OP_N, OP_C, m, m, n, ONE, M, m, 0, M, m, 0, ZERO, G.c(), m, 0, 1, true);
    else
        zgemm(ctx, OP_C, OP_N, n, n, m, ONE, M, m, 0, M, m, 0, ZERO, G.c(), n, 0, 1, true);
    heev_full(ctx, G.c(), g, lam.d());
    const KeepResult kr = keep_rule(ctx, lam.d(), g, sz, t.cutoff, t.maxdim, t.mindim, nullptr);
    const int64_t k = kr.k;
    X = DBuf(ctx, sizeof(cplx) * m * k);
    Y = DBuf(ctx, sizeof(cplx) * k * n);
    if (left_iso) {
        take_top_eigvecs(ctx, G.c(), m, k, X.c());
        zgemm(ctx, OP_C, OP_N, k, n, m, ONE, X.c(), m, 0, M, m, 0, ZERO, Y.c(), k, 0);
    } else {
        DBuf Vk(ctx, sizeof(cplx) * n * k);
        take_top_eigvecs(ctx, G.c(), n, k, Vk.c());
        zgemm(ctx, OP_N, OP_N, m, k, n, ONE, M, m, 0, Vk.c(), n, 0, ZERO, X.c(), m, 0);
        conj_transpose(ctx, Vk.c(), n, k, Y.c());
    }
    if (rec) {
        rec->m = m;
        rec->n = n;
        rec->k = k;
        rec->g = g;
        rec->left_iso = left_iso;
        rec->M = std::move(Min);
        rec->V = std::move(G);
        rec->lam = std::move(lam);
    }
    return k;
}

// Mbar (m x n) from Xbar (m x k), Ybar (k x n)
void split_back(Ctx* ctx, const SplitRec& r, const cplx* Xbar, const cplx* Ybar, double eta,
                DBuf& Mbar) {
    const int64_t m = r.m, n = r.n, k = r.k, g = r.g;
    const cplx* M = r.M.c();
    Mbar = DBuf(ctx, sizeof(cplx) * m * n);
    DBuf Vk(ctx, sizeof(cplx) * g * k), Vbar(ctx, sizeof(cplx) * g * k);
    take_top_eigvecs(ctx, r.V.c(), g, k, Vk.c());
    if (r.left_iso) {
        // Y = X^H M: Mbar = X Ybar; Xbar_tot = Xbar + M Ybar^H
        zgemm(ctx, OP_N, OP_N, m, n, k, ONE, Vk.c(), m, 0, Ybar, k, 0, ZERO, Mbar.c(), m, 0);
        zcopy(ctx, Vbar.c(), Xbar, m * k);
        zgemm(ctx, OP_N, OP_C, m, k, n, ONE, M, m, 0, Ybar, k, 0, ONE, Vbar.c(), m, 0);
    } else {
        // X = M Vk, Y = Vk^H: Mbar = Xbar Vk^H; Vbar = M^H Xbar + Ybar^H
        zgemm(ctx, OP_N, OP_C, m, n, k, ONE, Xbar, m, 0, Vk.c(), n, 0, ZERO, Mbar.c(), m, 0);
        conj_transpose(ctx, Ybar, k, n, Vbar.c());
        zgemm(ctx, OP_C, OP_N, n, k, m, ONE, M, m, 0, Xbar, m, 0, ONE, Vbar.c(), n, 0);
    }
    // C = V^H Vbar (g x k), D = F o C, Gbar = V D Vk^H, S = Gbar + Gbar^H
    DBuf Cm(ctx, sizeof(cplx) * g * k), D(ctx, sizeof(cplx) * g * k);
    zgemm(ctx, OP_C, OP_N, g, k, g, ONE, r.V.c(), g, 0, Vbar.c(), g, 0, ZERO, Cm.c(), g, 0);
    gap_weight_kernel<<<blocks_for(g * k), 256, 0, ctx->stream>>>(Cm.c(), r.lam.d(), g, k, eta,
                                                                  D.c());
    check_launch(ctx);
    DBuf T(ctx, sizeof(cplx) * g * k), Gb(ctx, sizeof(cplx) * g * g), S(ctx, sizeof(cplx) * g * g);
    zgemm(ctx, OP_N, OP_N, g, k, g, ONE, r.V.c(), g, 0, D.c(), g, 0, ZERO, T.c(), g, 0);
    zgemm(ctx, OP_N, OP_C, g, g, k, ONE, T.c(), g, 0, Vk.c(), g, 0, ZERO, Gb.c(), g, 0);
    herm_sum_kernel<<<blocks_for(g * g), 256, 0, ctx->stream>>>(Gb.c(), g, S.c());
    check_launch(ctx);
    if (r.left_iso)  // G = M M^H: Mbar += S M
        zgemm(ctx, OP_N, OP_N, m, n, m, ONE, S.c(), m, 0, M, m, 0, ONE, Mbar.c(), m, 0);
    else  // G = M^H M: Mbar += M S
        zgemm(ctx, OP_N, OP_N, m, n, n, ONE, M, m, 0, S.c(), n, 0, ONE, Mbar.c(), m, 0);
}

// ---- taped forward primitives ---------------------------------------------
struct Fwd {
    tn_mps* psi;
    Tape* tape;  // null: untaped
};

void t_moveright(Fwd& F, int idx, const Trunc& t) {
    tn_mps* psi = F.psi;
    if (!(0 < idx && idx < psi->N)) return;
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(idx), Dr = psi->dr(idx), Dr2 = psi->dr(idx + 1);
    Op op;
    op.kind = Kind::MoveR;
    op.site = idx;
    op.Dl = Dl;
    op.Dm = Dr;
    op.Dr = Dr2;
    DBuf X, Y;
    const int64_t k = split_full(ctx, std::move(psi->A[idx - 1]), Dl * d, Dr, t, true, X, Y,
                                 F.tape ? &op.sp : nullptr);
    DBuf next(ctx, sizeof(cplx) * k * d * Dr2);
    zgemm(ctx, OP_N, OP_N, k, d * Dr2, Dr, ONE, Y.c(), k, 0, psi->site(idx + 1), Dr, 0, ZERO,
          next.c(), k, 0);
    if (F.tape) {
        op.a = std::move(Y);                  // absorbed factor (k x Dr)
        op.b = std::move(psi->A[idx]);        // old neighbour (Dr x d Dr2)
        F.tape->push_back(std::move(op));
    }
    psi->A[idx - 1] = std::move(X);
    psi->A[idx] = std::move(next);
    psi->dims[idx] = k;
}

void t_moveleft(Fwd& F, int idx, const Trunc& t) {
    tn_mps* psi = F.psi;
    if (!(1 < idx && idx <= psi->N)) return;
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    const int64_t Dl = psi->dl(idx), Dr = psi->dr(idx), Dl0 = psi->dl(idx - 1);
    Op op;
    op.kind = Kind::MoveL;
    op.site = idx;
    op.Dl = Dl0;
    op.Dm = Dl;
    op.Dr = Dr;
    DBuf X, Y;
    const int64_t k = split_full(ctx, std::move(psi->A[idx - 1]), Dl, d * Dr, t, false, X, Y,
                                 F.tape ? &op.sp : nullptr);
    DBuf prev(ctx, sizeof(cplx) * Dl0 * d * k);
    zgemm(ctx, OP_N, OP_N, Dl0 * d, k, Dl, ONE, psi->site(idx - 1), Dl0 * d, 0, X.c(), Dl, 0, ZERO,
          prev.c(), Dl0 * d, 0);
    if (F.tape) {
        op.a = std::move(X);               // absorbed factor (Dl x k)
        op.b = std::move(psi->A[idx - 2]);  // old neighbour (Dl0 d x Dl)
        F.tape->push_back(std::move(op));
    }
    psi->A[idx - 1] = std::move(Y);
    psi->A[idx - 2] = std::move(prev);
    psi->dims[idx - 1] = k;
}

void t_movecenter(Fwd& F, int idx, const Trunc& t) {
    tn_mps* psi = F.psi;
    TN_REQUIRE(idx >= 1 && idx <= psi->N, "The index is out of range.");
    TN_REQUIRE(psi->center != 0, "tebd gradient: the state has no orthogonality centre");
    if (idx > psi->center) {
        for (int i = psi->center; i <= idx - 1; ++i) t_moveright(F, i, t);
    } else if (idx < psi->center) {
        const int c = psi->center;
        for (int i = 1; i <= c - idx; ++i) t_moveleft(F, c + 1 - i, t);
    }
    psi->center = idx;
}

void t_applygate(Fwd& F, int site, int ns, const cplx* M, const cplx* Mh, cplx* gbar,
                 bool direction, const Trunc& t) {
    tn_mps* psi = F.psi;
    Ctx* ctx = psi->ctx;
    const int d = psi->d;
    if (ns == 1) {
        const int64_t Dl = psi->dl(site), Dr = psi->dr(site);
        DBuf out(ctx, sizeof(cplx) * Dl * d * Dr);
        small_apply(ctx, psi->site(site), out.c(), M, d, d, Dl, Dr, Dl, Dl * d, Dl, Dl * d);
        if (F.tape) {
            Op op;
            op.kind = Kind::Gate1;
            op.site = site;
            op.Dl = Dl;
            op.Dr = Dr;
            op.Mh = Mh;
            op.gbar = gbar;
            op.nI = d;
            op.a = std::move(psi->A[site - 1]);
            F.tape->push_back(std::move(op));
        }
        psi->A[site - 1] = std::move(out);
        // replacesite1 (gmps.jl:204-213): non-truncating move to the neighbour
        const int nxt = site + 1 - 2 * (direction ? 1 : 0);
        if (0 < nxt && nxt <= psi->N) t_movecenter(F, nxt, no_trunc());
        return;
    }
    const int64_t Dl = psi->dl(site), Dm = psi->dr(site), Dr = psi->dr(site + 1);
    const int d2 = d * d;
    DBuf theta(ctx, sizeof(cplx) * Dl * d2 * Dr), theta2(ctx, sizeof(cplx) * Dl * d2 * Dr);
    zgemm(ctx, OP_N, OP_N, Dl * d, d * Dr, Dm, ONE, psi->site(site), Dl * d, 0, psi->site(site + 1),
          Dm, 0, ZERO, theta.c(), Dl * d, 0);
    small_apply(ctx, theta.c(), theta2.c(), M, d2, d2, Dl, Dr, Dl, Dl * d2, Dl, Dl * d2);
    Op op;
    op.kind = Kind::Gate2;
    op.site = site;
    op.Dl = Dl;
    op.Dm = Dm;
    op.Dr = Dr;
    DBuf X, Y;
    const int64_t k = split_full(ctx, std::move(theta2), Dl * d, d * Dr, t, !direction, X, Y,
                                 F.tape ? &op.sp : nullptr);
    if (F.tape) {
        op.Mh = Mh;
        op.gbar = gbar;
        op.nI = d2;
        op.a = std::move(psi->A[site - 1]);
        op.b = std::move(psi->A[site]);
        op.theta = std::move(theta);
        F.tape->push_back(std::move(op));
    }
    psi->A[site - 1] = std::move(X);
    psi->A[site] = std::move(Y);
    psi->dims[site] = k;
    psi->center = direction ? site : site + 1;
}

void t_normalize(Fwd& F) {
    tn_mps* psi = F.psi;
    Ctx* ctx = psi->ctx;
    const int c = psi->center;
    const double n = std::sqrt(znorm2(ctx, psi->site(c), psi->size(c)));
    zscale(ctx, psi->site(c), psi->size(c), cmk(1.0 / n, 0.0));
    if (F.tape) {
        Op op;
        op.kind = Kind::Normalize;
        op.site = c;
        op.norm = n;
        op.a = dcopy(ctx, psi->site(c), psi->size(c));
        F.tape->push_back(std::move(op));
    }
}

struct GateSet {  // one uploaded gate list with its adjoint buffers
    const tn_gates* g;
    std::vector<DBuf> Mh;    // M^H per gate
    std::vector<DBuf> gbar;  // cotangent per gate (small_apply form)
};

void t_applygates(Fwd& F, GateSet& gs, const Trunc& t) {
    tn_mps* psi = F.psi;
    const tn_gates* g = gs.g;
    for (size_t r = 0; r < g->row_len.size(); ++r) {
        const int s0 = g->row_start[r], len = g->row_len[r];
        if (len == 0) continue;
        const int first = g->sites[s0];
        const int last = g->sites[s0 + len - 1] + g->nsites[s0 + len - 1] - 1;
        const bool direction = !(std::abs(psi->center - first) < std::abs(psi->center - last));
        for (int i = 0; i < len; ++i) {
            const int gi = s0 + (direction ? len - 1 - i : i);
            const int ctr = direction ? g->sites[gi] + g->nsites[gi] - 1 : g->sites[gi];
            t_movecenter(F, ctr, t);
            t_applygate(F, g->sites[gi], g->nsites[gi], g->M[gi].c(),
                        gs.Mh.empty() ? nullptr : gs.Mh[gi].c(),
                        gs.gbar.empty() ? nullptr : gs.gbar[gi].c(), direction, t);
        }
    }
}

// ---- reverse sweep over a tape --------------------------------------------
// bar[i] holds the cotangent of site i (dims of the state at that point)
void reverse(Ctx* ctx, int d, Tape& tape, std::vector<DBuf>& bar, double eta) {
    for (size_t q = tape.size(); q-- > 0;) {
        Op& op = tape[q];
        switch (op.kind) {
            case Kind::Normalize: {
                const int c = op.site;
                const int64_t sz = (int64_t)(op.a.bytes / sizeof(cplx));
                const double r = dot(ctx, op.a.c(), bar[c - 1].c(), sz).x;  // Re<c', c'bar>
                axpy_scale_kernel<<<blocks_for(sz), 256, 0, ctx->stream>>>(bar[c - 1].c(), op.a.c(),
                                                                            r, 1.0 / op.norm, sz);
                check_launch(ctx);
                break;
            }
            case Kind::MoveR: {
                // M (Dl d x Dr) -> X, Y (k x Dr); next = Y B with B (Dr x d Dr2)
                const int i = op.site;
                const int64_t k = op.sp.k, Dr = op.Dm, dDr2 = d * op.Dr;
                DBuf Ybar(ctx, sizeof(cplx) * k * Dr), Bbar(ctx, sizeof(cplx) * Dr * dDr2);
                const cplx* Nbar = bar[i].c();
                zgemm(ctx, OP_N, OP_C, k, Dr, dDr2, ONE, Nbar, k, 0, op.b.c(), Dr, 0, ZERO, Ybar.c(),
                      k, 0);
                zgemm(ctx, OP_C, OP_N, Dr, dDr2, k, ONE, op.a.c(), k, 0, Nbar, k, 0, ZERO, Bbar.c(),
                      Dr, 0);
                DBuf Mbar;
                split_back(ctx, op.sp, bar[i - 1].c(), Ybar.c(), eta, Mbar);
                bar[i - 1] = std::move(Mbar);
                bar[i] = std::move(Bbar);
                break;
            }
            case Kind::MoveL: {
                // M (Dl x d Dr) -> X (Dl x k), Y; prev = P X with P (Dl0 d x Dl)
                const int i = op.site;
                const int64_t k = op.sp.k, Dl = op.Dm, dDl0 = d * op.Dl;
                DBuf Pbar(ctx, sizeof(cplx) * dDl0 * Dl), Xbar(ctx, sizeof(cplx) * Dl * k);
                const cplx* Nbar = bar[i - 2].c();
                zgemm(ctx, OP_N, OP_C, dDl0, Dl, k, ONE, Nbar, dDl0, 0, op.a.c(), Dl, 0, ZERO,
                      Pbar.c(), dDl0, 0);
                zgemm(ctx, OP_C, OP_N, Dl, k, dDl0, ONE, op.b.c(), dDl0, 0, Nbar, dDl0, 0, ZERO,
                      Xbar.c(), Dl, 0);
                DBuf Mbar;
                split_back(ctx, op.sp, Xbar.c(), bar[i - 1].c(), eta, Mbar);
                bar[i - 1] = std::move(Mbar);
                bar[i - 2] = std::move(Pbar);
                break;
            }
            case Kind::Gate1: {
                const int s = op.site;
                const int64_t Dl = op.Dl, Dr = op.Dr;
                DBuf inb(ctx, sizeof(cplx) * Dl * d * Dr);
                small_apply(ctx, bar[s - 1].c(), inb.c(), op.Mh, d, d, Dl, Dr, Dl, Dl * d, Dl,
                            Dl * d);
                if (op.gbar) {
                    leg_grad_kernel<<<d * d, 256, 0, ctx->stream>>>(op.a.c(), bar[s - 1].c(), d, d,
                                                                    Dl, Dr, Dl, Dl * d, Dl * d,
                                                                    op.gbar);
                    check_launch(ctx);
                }
                bar[s - 1] = std::move(inb);
                break;
            }
            case Kind::Gate2: {
                const int s = op.site;
                const int64_t Dl = op.Dl, Dm = op.Dm, Dr = op.Dr;
                const int d2 = d * d;
                DBuf T2bar;
                split_back(ctx, op.sp, bar[s - 1].c(), bar[s].c(), eta, T2bar);
                DBuf Tbar(ctx, sizeof(cplx) * Dl * d2 * Dr);
                small_apply(ctx, T2bar.c(), Tbar.c(), op.Mh, d2, d2, Dl, Dr, Dl, Dl * d2, Dl,
                            Dl * d2);
                if (op.gbar) {
                    leg_grad_kernel<<<d2 * d2, 256, 0, ctx->stream>>>(op.theta.c(), T2bar.c(), d2,
                                                                      d2, Dl, Dr, Dl, Dl * d2,
                                                                      Dl * d2, op.gbar);
                    check_launch(ctx);
                }
                DBuf A1bar(ctx, sizeof(cplx) * Dl * d * Dm), A2bar(ctx, sizeof(cplx) * Dm * d * Dr);
                zgemm(ctx, OP_N, OP_C, Dl * d, Dm, d * Dr, ONE, Tbar.c(), Dl * d, 0, op.b.c(), Dm, 0,
                      ZERO, A1bar.c(), Dl * d, 0);
                zgemm(ctx, OP_C, OP_N, Dm, d * Dr, Dl * d, ONE, op.a.c(), Dl * d, 0, Tbar.c(),
                      Dl * d, 0, ZERO, A2bar.c(), Dm, 0);
                bar[s - 1] = std::move(A1bar);
                bar[s] = std::move(A2bar);
                break;
            }
        }
        tape.pop_back();  // release the record's device memory as we go
    }
}

tn_mps* mps_clone(const tn_mps* src) {
    tn_mps* m = new tn_mps();
    m->ctx = src->ctx;
    m->N = src->N;
    m->d = src->d;
    m->dims = src->dims;
    m->center = src->center;
    m->A.resize(src->N);
    for (int i = 1; i <= src->N; ++i) m->A[i - 1] = dcopy(src->ctx, src->site(i), src->size(i));
    return m;
}

struct MpsOwner {
    tn_mps* p = nullptr;
    ~MpsOwner() { delete p; }
    void reset(tn_mps* q) {
        delete p;
        p = q;
    }
};

}  // namespace

// f = <psi|O|psi>/<psi|psi> after the steps; gate cotangents when grads != null
double tebd_grad(const tn_mps* psi0, const std::vector<const tn_gates*>& gls,
                 const std::vector<int>& step_gl, const Trunc& t, int every, int obs_site,
                 const double* obs_op, double eta, double* grads) {
    Ctx* ctx = psi0->ctx;
    const int N = psi0->N, d = psi0->d;
    const int nsteps = (int)step_gl.size();
    TN_REQUIRE(every >= 1, "checkpoint interval must be >= 1");
    TN_REQUIRE(obs_site >= 1 && obs_site <= N, "observable site out of range");
    TN_REQUIRE(eta >= 0.0, "broadening must be >= 0");
    for (int s : step_gl) TN_REQUIRE(s >= 0 && s < (int)gls.size(), "step gate-list index out of range");
    for (const tn_gates* g : gls)
        TN_REQUIRE(g && g->N == N && g->d == d, "GateList and MPS do not match.");
    const bool want = grads != nullptr;
    std::vector<GateSet> sets(gls.size());
    for (size_t l = 0; l < gls.size(); ++l) {
        sets[l].g = gls[l];
        if (!want) continue;
        const size_t ng = gls[l]->M.size();
        sets[l].Mh.resize(ng);
        sets[l].gbar.resize(ng);
        for (size_t i = 0; i < ng; ++i) {
            const int nI = gls[l]->nsites[i] == 1 ? d : d * d;
            sets[l].Mh[i] = DBuf(ctx, sizeof(cplx) * nI * nI);
            conj_transpose(ctx, gls[l]->M[i].c(), nI, nI, sets[l].Mh[i].c());
            sets[l].gbar[i] = DBuf(ctx, sizeof(cplx) * nI * nI);
            zfill(ctx, sets[l].gbar[i].c(), nI * nI, ZERO);
        }
    }
    DBuf Obs;
    upload_op_matrix(ctx, obs_op, d, Obs);
    MpsOwner cur;
    cur.reset(mps_clone(psi0));
    if (cur.p->center == 0) movecenter(cur.p, 1, no_trunc());  // tebd.jl:61 canonicalises
    const int nseg = (nsteps + every - 1) / every;
    // first pass: checkpoints at the start of every segment
    std::vector<MpsOwner> ckpt(std::max(nseg, 1));
    {
        Fwd F{cur.p, nullptr};
        for (int s = 0; s < nsteps; ++s) {
            if (want && s % every == 0) ckpt[s / every].reset(mps_clone(cur.p));
            if (want && s >= (nseg - 1) * every) break;  // the last segment is recomputed
            t_applygates(F, sets[step_gl[s]], t);
            t_normalize(F);
        }
    }
    // objective at the orthogonality centre moved (without truncation) to the site
    auto objective = [&](Fwd& F, std::vector<DBuf>* bar) {
        t_movecenter(F, obs_site, no_trunc());
        tn_mps* p = F.psi;
        const int64_t Dl = p->dl(obs_site), Dr = p->dr(obs_site), n = p->size(obs_site);
        DBuf Oc(ctx, sizeof(cplx) * n);
        small_apply(ctx, p->site(obs_site), Oc.c(), Obs.c(), d, d, Dl, Dr, Dl, Dl * d, Dl, Dl * d);
        const double nn = dot(ctx, p->site(obs_site), p->site(obs_site), n).x;
        const double f = dot(ctx, p->site(obs_site), Oc.c(), n).x / nn;
        if (bar) {
            // cbar = 2 (O c - f c) / <c|c>
            bar->clear();
            bar->resize(N);
            for (int i = 1; i <= N; ++i) {
                (*bar)[i - 1] = DBuf(ctx, sizeof(cplx) * p->size(i));
                zfill(ctx, (*bar)[i - 1].c(), p->size(i), ZERO);
            }
            zaxpy_kernel<<<blocks_for(n), 256, 0, ctx->stream>>>((*bar)[obs_site - 1].c(), Oc.c(),
                                                                 cmk(2.0 / nn, 0.0), n);
            check_launch(ctx);
            zaxpy_kernel<<<blocks_for(n), 256, 0, ctx->stream>>>(
                (*bar)[obs_site - 1].c(), p->site(obs_site), cmk(-2.0 * f / nn, 0.0), n);
            check_launch(ctx);
        }
        return f;
    };
    if (!want) {
        Fwd F{cur.p, nullptr};
        return objective(F, nullptr);
    }
    double f = 0.0;
    std::vector<DBuf> bar;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        cur.reset(mps_clone(ckpt[seg].p));
        ckpt[seg].reset(nullptr);
        Tape tape;
        Fwd F{cur.p, &tape};
        const int a = seg * every, b = std::min(nsteps, a + every);
        for (int s = a; s < b; ++s) {
            t_applygates(F, sets[step_gl[s]], t);
            t_normalize(F);
        }
        if (seg == nseg - 1) f = objective(F, &bar);
        reverse(ctx, d, tape, bar, eta);
    }
    if (nsteps == 0) {  // objective only: no gates to differentiate
        Fwd F{cur.p, nullptr};
        f = objective(F, nullptr);
    }
    // gate cotangents back to the upload layouts
    size_t off = 0;
    for (size_t l = 0; l < gls.size(); ++l) {
        const tn_gates* g = gls[l];
        for (size_t i = 0; i < g->M.size(); ++i) {
            const int ns = g->nsites[i];
            const int nI = ns == 1 ? d : d * d;
            std::vector<cplx> h((size_t)nI * nI);
            TN_CHECK_CUDA(cudaMemcpyAsync(h.data(), sets[l].gbar[i].c(), sizeof(cplx) * h.size(),
                                          cudaMemcpyDeviceToHost, ctx->stream));
            ctx->sync();
            if (ns == 1) {
                // M[i + d o] = op[o + d i]
                for (int o = 0; o < d; ++o)
                    for (int ii = 0; ii < d; ++ii) {
                        const cplx v = h[ii + (size_t)d * o];
                        grads[2 * (off + o + (size_t)d * ii)] = v.x;
                        grads[2 * (off + o + (size_t)d * ii) + 1] = v.y;
                    }
            } else {
                // M[(i1 + d i2) + d^2 (o1 + d o2)] = G[o1 + d (i1 + d (o2 + d i2))]
                const int d2 = d * d;
                for (int o1 = 0; o1 < d; ++o1)
                    for (int i1 = 0; i1 < d; ++i1)
                        for (int o2 = 0; o2 < d; ++o2)
                            for (int i2 = 0; i2 < d; ++i2) {
                                const size_t src = (i1 + d * i2) + (size_t)d2 * (o1 + d * o2);
                                const size_t dst = o1 + d * (i1 + d * (o2 + (size_t)d * i2));
                                grads[2 * (off + dst)] = h[src].x;
                                grads[2 * (off + dst) + 1] = h[src].y;
                            }
            }
            off += (size_t)nI * nI;
        }
    }
    return f;
}

}  // namespace tn
