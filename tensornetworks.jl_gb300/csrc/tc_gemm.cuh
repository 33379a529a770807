// Complex GEMM on the 5th-generation tensor cores (tcgen05, TMEM accumulators,
// TMA-fed shared memory) with 3xTF32 split products and FP32 accumulation.
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace tn {

// Split-TF32 operand planes of a complex M x K (or N x K) matrix stored
// K-major (row r holds K contiguous values): four fp32 planes in the order
// re_hi, im_hi, re_lo, im_lo, each rows x ld with ld a multiple of 4.
struct TcPlanes {
    float* p = nullptr;
    int64_t rows = 0, K = 0, ld = 0;
    size_t plane() const { return (size_t)rows * ld; }
    size_t floats() const { return 4 * plane(); }
};

inline int64_t tc_ld(int64_t K) { return (K + 3) / 4 * 4; }

// Tensor-core FP32 accumulation rounds with a bias, so its relative error
// grows linearly with the number of accumulation steps.  The K loop is
// therefore cut into chunks of kchunk elements (one per blockIdx.z), each
// written as an FP32 partial; consumers sum the partials in FP64.
constexpr int64_t TC_KCHUNK = 128;
int tc_chunks(int64_t K, int64_t kchunk = TC_KCHUNK);

// Partials of C = op(A) * B^T, op(A) = A or conj(A): chunk z writes FP32
// planar re[z*chunk_stride + m + ldo*n], im at + plane_stride.  Returns the
// number of chunks.
int tc_cgemm_partials(Ctx* ctx, const TcPlanes& A, const TcPlanes& B, int64_t M, int64_t N,
                      int64_t K, bool conjA, int64_t kchunk, float* out, int64_t ldo,
                      int64_t plane_stride, int64_t chunk_stride);

// out[m + ldo*n] (+)= sum over chunks, FP64 interleaved column-major.
void tc_reduce_fp64(Ctx* ctx, const float* P, int S, int64_t M, int64_t N, int64_t ldp,
                    int64_t plane_stride, int64_t chunk_stride, cplx* out, int64_t ldo,
                    bool accumulate);

// Reads the device error flag the tensor-core kernels set when a bounded
// wait runs out; throws TN_ERR_TIMEOUT if it is set.
void tc_check_error(Ctx* ctx);

}  // namespace tn
