// Mixed-precision two-site H_eff product.
#include "mixed.cuh"

namespace tn {

void mixed_prepare_env(Ctx*, MixedWork&, const cplx*, const cplx*, int64_t, int64_t, int, int64_t,
                       int64_t) {
    throw Error(TN_ERR_INVALID, "mixed precision is not available yet in this build");
}

void mixed_heff2(Ctx*, MixedWork&, const cplx*, int64_t, int64_t, int, int64_t, int64_t,
                 const cplx*, cplx*) {
    throw Error(TN_ERR_INVALID, "mixed precision is not available yet in this build");
}

void mixed_unit_heff2(Ctx*, const cplx*, const cplx*, const cplx*, int64_t, int64_t, int, int64_t,
                      int64_t, const cplx*, cplx*) {
    throw Error(TN_ERR_INVALID, "mixed precision is not available yet in this build");
}

}  // namespace tn
