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
// y = H_eff x for one bond, FP64 in and out, 3xTF32 products inside.
void mixed_heff2(Ctx* ctx, MixedWork& mw, const cplx* W12, int64_t cl, int64_t cr, int d,
                 int64_t wl, int64_t wr, const cplx* x, cplx* y);

}  // namespace tn
