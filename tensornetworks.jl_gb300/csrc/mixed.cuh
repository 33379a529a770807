// Mixed-precision (3xTF32 on tcgen05 tensor cores, FP32 accumulate in TMEM)
// two-site effective-Hamiltonian product.
#pragma once

#include "common.cuh"
#include "tc_gemm.cuh"

namespace tn {

// Per-bond operands of the mixed matvec and its scratch, kept between
// Lanczos iterations.
struct MixedWork {
    int64_t cl = 0, cr = 0, wl = 0, wr = 0;
    int d = 0;
    Scratch L, R, th, t1, t2, p3;  // operand planes, intermediates, partials
    TcPlanes Lp, Rp;           // prepared environment operands
};

// Converts the environment blocks L[a,w,b], R[c',w'',c] into the split-TF32,
// K-major planes the tensor-core GEMM reads.
void mixed_prepare_env(Ctx* ctx, MixedWork& mw, const cplx* L, const cplx* R, int64_t cl,
                       int64_t cr, int d, int64_t wl, int64_t wr);
// Environment updates with both GEMMs on the tensor cores (3xTF32), FP64 in
// and out; Ml / Mr are the MPO leg matrices of the site.
void mixed_env_left(Ctx* ctx, const cplx* L, int64_t ca, int64_t wl, int64_t cb, const cplx* A,
                    int64_t ca2, const cplx* Ml, int d, int64_t wr, const cplx* B, int64_t cb2,
                    cplx* out);
void mixed_env_right(Ctx* ctx, const cplx* R, int64_t ca2, int64_t wr, int64_t cb2, const cplx* A,
                     int64_t ca, const cplx* Mr, int d, int64_t wl, const cplx* B, int64_t cb,
                     cplx* out);
// C (m x n) = op(A) B, op(A) = A (m x k) or A^H (A k x m), on the tensor cores.
void mixed_gemm(Ctx* ctx, int64_t m, int64_t n, int64_t k, const cplx* A, bool conj_a,
                const cplx* B, cplx* C);

// y = H_eff x for one bond, FP64 in and out, 3xTF32 products inside.
void mixed_heff2(Ctx* ctx, MixedWork& mw, const cplx* W12, int64_t cl, int64_t cr, int d,
                 int64_t wl, int64_t wr, const cplx* x, cplx* y);

}  // namespace tn
