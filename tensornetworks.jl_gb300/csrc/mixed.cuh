// Mixed-precision (3xTF32 on tcgen05 tensor cores, FP32 accumulate in TMEM)
// two-site effective-Hamiltonian product.
#pragma once

#include "common.cuh"

namespace tn {

// Per-bond operands of the mixed matvec, kept between Lanczos iterations.
struct MixedWork {
    const cplx* L = nullptr;  // identity of the prepared environment blocks
    const cplx* R = nullptr;
    int64_t cl = 0, cr = 0, wl = 0, wr = 0;
    int d = 0;
};

// Converts the environment blocks L[a,w,b], R[c',w'',c] into the split-TF32,
// K-major planes the tensor-core GEMM reads.  No-op when already prepared.
void mixed_prepare_env(Ctx* ctx, MixedWork& mw, const cplx* L, const cplx* R, int64_t cl,
                       int64_t cr, int d, int64_t wl, int64_t wr);
// y = H_eff x for one bond, FP64 in and out, 3xTF32 products inside.
void mixed_heff2(Ctx* ctx, MixedWork& mw, const cplx* W12, int64_t cl, int64_t cr, int d,
                 int64_t wl, int64_t wr, const cplx* x, cplx* y);

}  // namespace tn
