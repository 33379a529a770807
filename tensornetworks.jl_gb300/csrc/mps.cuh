// Device-resident GMPS / MPO / GateList handles and the operations of the
// hot path (structures/mps/gmps.jl, projmps.jl, gatelist.jl).
#pragma once

#include <functional>

#include "common.cuh"

struct tn_ctx {
    tn::Ctx c;
};

// Rank-1 GMPS on the device: site i (1-based) is A[dims[i-1], d, dims[i]].
struct tn_mps {
    tn::Ctx* ctx = nullptr;
    int N = 0, d = 0;
    std::vector<int64_t> dims;  // N+1 bond dimensions
    std::vector<tn::DBuf> A;    // N site tensors
    int center = 0;
    cplx* site(int i) const { return A[i - 1].c(); }
    int64_t dl(int i) const { return dims[i - 1]; }
    int64_t dr(int i) const { return dims[i]; }
    int64_t size(int i) const { return dims[i - 1] * d * dims[i]; }
    int maxbonddim() const {
        int64_t D = 1;
        for (int i = 1; i < N; ++i) D = std::max(D, dims[i]);
        return (int)D;
    }
};

// Rank-2 GMPS (MPO) with the per-site operator matrices the contractions use.
struct tn_mpo {
    tn::Ctx* ctx = nullptr;
    int N = 0, d = 0;
    std::vector<int64_t> w;       // N+1 bond dimensions
    std::vector<tn::DBuf> W;      // [wl, d, d, wr]
    std::vector<tn::DBuf> Ml;     // left-env leg matrix  M[(w,s),(s',w')]
    std::vector<tn::DBuf> Mr;     // right-env leg matrix M[(s',w'),(w,s)]
    std::vector<tn::DBuf> W12;    // bond (i,i+1): M[(w,s1,s2),(s1',s2',w'')]
    std::vector<std::vector<double>> host;  // interleaved host copies
};

struct tn_gates {
    int N = 0, d = 0;
    std::vector<int> row_start, row_len;
    std::vector<int> sites, nsites;
    std::vector<tn::DBuf> M;  // small_apply matrices M[I=(i1,i2), J=(o1,o2)]
};

namespace tn {

struct Trunc {
    double cutoff = 0.0;
    int64_t maxdim = 0;
    int64_t mindim = 1;
};
inline Trunc no_trunc() { return Trunc{}; }

// gauge moves and normalisation (gmps.jl:29-112)
void moveright(tn_mps* psi, int idx, const Trunc& t);
void moveleft(tn_mps* psi, int idx, const Trunc& t);
void movecenter(tn_mps* psi, int idx, const Trunc& t);
cplx mps_norm(tn_mps* psi);
void mps_normalize(tn_mps* psi);
// two-site split (gmps.jl:199-267); theta [Dl,d,d,Dr]
SplitResult replacesites2(tn_mps* psi, const cplx* theta, int site, bool direction, bool normalize,
                          const Trunc& t, std::vector<double>* S = nullptr);
// one-site replacement (gmps.jl:204-213); takes ownership of A
void replacesite1(tn_mps* psi, DBuf&& A, int site, bool direction, bool normalize);
// theta[Dl,d,d,Dr] = A_site * A_site+1 into buf
void two_site(tn_mps* psi, int site, DBuf& buf);
std::vector<double> singular_values(tn_mps* psi, int site);

// environment updates (projmps.jl:50-95); W == nullptr selects the overlap form
void env_left(Ctx* ctx, const cplx* L, int64_t ca, int64_t wl, int64_t cb, const cplx* A,
              int64_t ca2, const tn_mpo* H, int site, const cplx* B, int64_t cb2, int d, cplx* out);
void env_right(Ctx* ctx, const cplx* R, int64_t ca2, int64_t wr, int64_t cb2, const cplx* A,
               int64_t ca, const tn_mpo* H, int site, const cplx* B, int64_t cb, int d, cplx* out);
// two-site H_eff * theta (projmps.jl:103-145) in the optimal order
void heff2_fp64(Ctx* ctx, const cplx* L, const cplx* W12, const cplx* R, int64_t cl, int64_t cr,
                int d, int64_t wl, int64_t wr, const cplx* theta, cplx* out);

// sum_i x_i y_i (no conjugation), left on device at dout
void bilinear_dot(Ctx* ctx, const cplx* x, const cplx* y, int64_t n, cplx* dout);

// per-term expectation values (mps.jl:87-134); ops: d x d per covered site
struct Term {
    int first, len;
    std::vector<const cplx*> dops;  // device operator matrices (small_apply form)
    cplx coeff;
};
std::vector<cplx> inner_terms(Ctx* ctx, const tn_mps* bra, const tn_mps* ket,
                              const std::vector<Term>& terms);

// Terms of dmrg(psi, Hs::GMPS...; coeffs) (dmrg.jl:128-154, projmpssum.jl):
// MPOs H[t] with coefficients hc[t] (ProjMPS(psi, H, psi; rank=2)) and MPS
// projectors coeff pc[p] |P[p]><P[p]| (ProjMPS(P, psi; rank=2, squared=true)).
struct DmrgTerms {
    std::vector<const tn_mpo*> H;
    std::vector<double> hc;
    std::vector<const tn_mps*> P;
    std::vector<double> pc;
};
void dmrg_run(tn_mps* psi, const DmrgTerms& terms, const tn_dmrg_opts& o, double* energy,
              tn_dmrg_stats* stats);

// TEBD adjoint (tebd_grad.cu): f = <O at obs_site> after the steps (step s
// applies gate list gls[step_gl[s]] then normalises); grads != null receives
// df/dconj(G) for every gate of every list in the upload layouts
double tebd_grad(const tn_mps* psi0, const std::vector<const tn_gates*>& gls,
                 const std::vector<int>& step_gl, const Trunc& t, int every, int obs_site,
                 const double* obs_op, double eta, double* grads);

// small_apply matrix of a d x d operator acting on the physical leg
void upload_op_matrix(Ctx* ctx, const double* op_interleaved, int d, DBuf& out);
void apply_site_op(tn_mps* psi, int site, const cplx* M);

}  // namespace tn
