// tcgen05 complex GEMM, 3xTF32, FP32 accumulation in TMEM.
//
// Tile 128 x 128 per CTA (MMA M=128, N=128, K=8 per instruction), K staged in
// 32-float (128-byte) slices by TMA with the 128-byte swizzle, three-stage
// mbarrier pipeline.  Warp roles: warp 0 issues TMA loads, warp 1 allocates
// TMEM and one lane issues the MMAs, warps 2-5 drain TMEM in the epilogue.
//
// A complex product is four real products into two TMEM accumulators
// (Cr += Ar Br - Ai Bi, Ci += Ar Bi + Ai Br; the sign comes from the
// instruction descriptor's negate-A bit).  Each real product runs as three
// TF32 passes hi*hi + hi*lo + lo*hi over the split operand planes, which
// gives FP32-class accuracy from TF32 tensor cores.
//
// Every mbarrier wait is bounded by the global timer; a wait that runs out
// sets a device error flag, the kernel drains and releases TMEM, and the host
// reports TN_ERR_TIMEOUT.
#include <cudaTypedefs.h>

#include <cstring>

#include "tc_gemm.cuh"

namespace tn {

namespace {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 4;     // 16 KB, BM == BN
constexpr int STAGE_BYTES = 4 * TILE_BYTES; // A re, A im, B re, B im
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
// TMEM columns: hi*hi products accumulate in Cr (+0) and Ci (+128); the small
// hi*lo and lo*hi corrections in separate accumulators (+256, +384), so the
// large accumulators take only two additions per k-step.
constexpr uint32_t TMEM_COLS = 512;
constexpr uint64_t WAIT_NS = 2000000000ull; // 2 s bound on any wait

struct Params {
    int64_t M, N, K;
    int conjA;
    int kchunk_tiles;      // k-tiles per blockIdx.z chunk
    float* out;            // FP32 planar partials [z][re|im][n][m]
    int64_t ldo, plane_stride, chunk_stride;
    int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false when the global-timer limit runs out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    while (!mbar_try(bar, parity)) {
        if (gtimer() - t0 > WAIT_NS) return false;
    }
    return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// K-major operand tile, 128-byte swizzle: rows of 128 bytes, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1 (bits 46-48),
// swizzle mode 2 = 128B (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused when swizzled)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // fixed 0b001
    d |= (uint64_t)2 << 61;             // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::tf32: D fp32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), K-major A and B, N>>3 at bit 17, M>>4 at bit 24;
// bit 13 negates A.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n, bool negA) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (negA ? (1u << 13) : 0u) |
           ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

#define TN_TMEM_LD32(taddr, r)                                                                   \
    asm volatile(                                                                                \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "  \
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "   \
        "%28, %29, %30, %31}, [%32];"                                                            \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),    \
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),             \
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),          \
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),          \
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),          \
          "=r"(r[31])                                                                            \
        : "r"(taddr))

__global__ void __launch_bounds__(192, 1)
    tc_cgemm_kernel(const __grid_constant__ CUtensorMap mapA,
                    const __grid_constant__ CUtensorMap mapB, Params p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 1);
    int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
    const int ktotal = (int)((p.K + BK - 1) / BK);
    const int kbeg = (int)blockIdx.z * p.kchunk_tiles;
    const int ktiles = min(p.kchunk_tiles, ktotal - kbeg);  // >= 1 by construction
    const int niter = 3 * ktiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accf, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            int issued = 0;
            for (int it = 0; it < niter; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                if (!mbar_wait(&empty[s], ph ^ 1u)) {
                    atomicExch(abort_flag, 1);
                    break;
                }
                if (*(volatile int*)abort_flag) break;
                const int pass = it / ktiles, kt = kbeg + (it - pass * ktiles);
                const int selA = (pass == 2) ? 1 : 0;  // lo planes in the lo*hi pass
                const int selB = (pass == 1) ? 1 : 0;  // lo planes in the hi*lo pass
                uint8_t* st = smem + s * STAGE_BYTES;
                mbar_expect_tx(&full[s], STAGE_BYTES);
                const int x = kt * BK;
                tma_load_3d(st + 0 * TILE_BYTES, &mapA, &full[s], x, (int)m0, 2 * selA + 0);
                tma_load_3d(st + 1 * TILE_BYTES, &mapA, &full[s], x, (int)m0, 2 * selA + 1);
                tma_load_3d(st + 2 * TILE_BYTES, &mapB, &full[s], x, (int)n0, 2 * selB + 0);
                tma_load_3d(st + 3 * TILE_BYTES, &mapB, &full[s], x, (int)n0, 2 * selB + 1);
                ++issued;
            }
            // let the copies still in flight land before the CTA can retire
            for (int it = (issued > STAGES ? issued - STAGES : 0); it < issued; ++it)
                (void)mbar_wait(&full[it % STAGES], (uint32_t)(it / STAGES) & 1u);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            const uint32_t id_pos = idesc_tf32(BM, BN, false);
            const uint32_t id_neg = idesc_tf32(BM, BN, true);
            const uint32_t id_ai_bi = p.conjA ? id_pos : id_neg;  // Cr += -+ Ai Bi
            const uint32_t id_ai_br = p.conjA ? id_neg : id_pos;  // Ci += +- Ai Br
            for (int it = 0; it < niter; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                if (!mbar_wait(&full[s], ph)) {
                    atomicExch(abort_flag, 1);
                    break;
                }
                tc_fence_after();
                const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
                const uint64_t dAr = sw128_desc(base + 0 * TILE_BYTES);
                const uint64_t dAi = sw128_desc(base + 1 * TILE_BYTES);
                const uint64_t dBr = sw128_desc(base + 2 * TILE_BYTES);
                const uint64_t dBi = sw128_desc(base + 3 * TILE_BYTES);
                const int pass = it / ktiles;
                const uint32_t dr = tmem + (pass == 0 ? 0u : 256u), di = dr + 128u;
                const bool first = (it == 0) || (it == ktiles);  // first use of each pair
#pragma unroll
                for (int j = 0; j < BK / 8; ++j) {
                    const uint64_t o = (uint64_t)(j * 32) >> 4;  // 8 tf32 = 32 bytes along K
                    const uint32_t acc = (first && j == 0) ? 0u : 1u;
                    tc_mma(dr, dAr + o, dBr + o, id_pos, acc);
                    tc_mma(dr, dAi + o, dBi + o, id_ai_bi, 1u);
                    tc_mma(di, dAr + o, dBi + o, id_pos, acc);
                    tc_mma(di, dAi + o, dBr + o, id_ai_br, 1u);
                }
                tc_commit(&empty[s]);
            }
            tc_commit(accf);
        }
    } else {
        // ---- epilogue: warps 2..5, TMEM lane quarter = warp % 4 ----
        const int q = warp & 3;
        const int64_t m = m0 + 32 * q + lane;
        if (mbar_wait(accf, 0)) {
            tc_fence_after();
            const bool ok = !*(volatile int*)abort_flag;
            float* outz = p.out + (size_t)blockIdx.z * p.chunk_stride;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t a[32], b[32];
                const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0;
#pragma unroll 1
                for (int part = 0; part < 2; ++part) {  // 0: real, 1: imaginary
                    TN_TMEM_LD32(ta + 128 * part, a);
                    TN_TMEM_LD32(ta + 256 + 128 * part, b);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (!ok || m >= p.M) continue;
                    float* o = outz + (size_t)part * p.plane_stride + m;
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int64_t n = n0 + c0 + j;
                        if (n >= p.N) break;
                        o[p.ldo * n] = __uint_as_float(a[j]) + __uint_as_float(b[j]);
                    }
                }
            }
        } else {
            atomicExch(abort_flag, 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    }
    if (threadIdx.x == 0 && *(volatile int*)abort_flag) atomicExch(p.err, 1);
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

void make_map(const TcPlanes& t, CUtensorMap* map) {
    if (!g_encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        TN_CHECK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                       cudaEnableDefault, &q));
        TN_REQUIRE(q == cudaDriverEntryPointSuccess && fn, "cuTensorMapEncodeTiled unavailable");
        g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    TN_REQUIRE(t.ld % 4 == 0 && t.ld >= t.K, "tensor-core planes need ld % 4 == 0");
    TN_REQUIRE((reinterpret_cast<uintptr_t>(t.p) & 15) == 0, "tensor-core planes must be 16-byte aligned");
    TN_REQUIRE(t.rows < (1ll << 31) && t.K < (1ll << 31), "tensor-core operand too large");
    cuuint64_t dims[3] = {(cuuint64_t)t.K, (cuuint64_t)t.rows, 4};
    cuuint64_t strides[2] = {(cuuint64_t)t.ld * 4, (cuuint64_t)(t.plane() * 4)};
    cuuint32_t box[3] = {BK, BM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, t.p, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(TN_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

int* err_flag(Ctx* ctx) { return ctx->d_err; }

}  // namespace

void tc_check_error(Ctx* ctx) {
    int h = 0;
    TN_CHECK_CUDA(cudaMemcpyAsync(&h, err_flag(ctx), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (h) {
        TN_CHECK_CUDA(cudaMemsetAsync(err_flag(ctx), 0, sizeof(int), ctx->stream));
        throw Error(TN_ERR_TIMEOUT, "tensor-core GEMM: a bounded device wait ran out");
    }
}

int tc_chunks(int64_t K, int64_t kchunk) {
    const int64_t kc = std::max<int64_t>(BK, kchunk / BK * BK);
    return (int)((K + kc - 1) / kc);
}

int tc_cgemm_partials(Ctx* ctx, const TcPlanes& A, const TcPlanes& B, int64_t M, int64_t N,
                      int64_t K, bool conjA, int64_t kchunk, float* out, int64_t ldo,
                      int64_t plane_stride, int64_t chunk_stride) {
    if (M <= 0 || N <= 0) return 0;
    TN_REQUIRE(A.rows >= M && B.rows >= N && A.K == K && B.K == K, "tc_cgemm: operand shapes");
    TN_REQUIRE(K > 0, "tc_cgemm: empty contraction");
    const int64_t kc = std::max<int64_t>(BK, kchunk / BK * BK);
    const int S = tc_chunks(K, kchunk);
    TN_REQUIRE((N + BN - 1) / BN <= 65535 && S <= 65535, "tc_cgemm: grid");
    TN_REQUIRE(plane_stride >= ldo * N && ldo >= M && chunk_stride >= 2 * plane_stride,
               "tc_cgemm: output layout");
    TN_CHECK_CUDA(cudaFuncSetAttribute(tc_cgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       SMEM_BYTES));
    CUtensorMap ma, mb;
    make_map(A, &ma);
    make_map(B, &mb);
    Params p{M, N, K, conjA ? 1 : 0, (int)(kc / BK), out, ldo, plane_stride, chunk_stride,
             err_flag(ctx)};
    dim3 grid((unsigned)((M + BM - 1) / BM), (unsigned)((N + BN - 1) / BN), (unsigned)S);
    // algorithmic flops of the complex product (8 per complex multiply-add);
    // the tensor pipe executes three TF32 passes of them
    ProfScope ps(ctx, 0, 8.0 * M * N * (double)K,
                 4.0 * 4.0 * (double)(M + N) * K + 8.0 * M * N * S);
    tc_cgemm_kernel<<<grid, 192, SMEM_BYTES, ctx->stream>>>(ma, mb, p);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    return S;
}

namespace {
// out[m + ldo*n] (+)= sum_z P[z][re|im][m + ldp*n], summed in float-float (TwoSum), stored as FP64
__global__ void reduce_partials_fp64_kernel(const float* __restrict__ P, int S, int64_t M,
                                            int64_t N, int64_t ldp, int64_t plane,
                                            int64_t chunk, cplx* __restrict__ out, int64_t ldo,
                                            int accumulate) {
    const int64_t total = M * N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i % M, n = i / M;
        const int64_t off = m + ldp * n;
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        for (int z = 0; z < S; ++z) {
            ff_add(rh, rl, P[(size_t)z * chunk + off]);
            ff_add(ih, il, P[(size_t)z * chunk + plane + off]);
        }
        double re = (double)rh + (double)rl, im = (double)ih + (double)il;
        cplx* o = out + m + ldo * n;
        if (accumulate) {
            re += o->x;
            im += o->y;
        }
        *o = cmk(re, im);
    }
}
}  // namespace

void tc_reduce_fp64(Ctx* ctx, const float* P, int S, int64_t M, int64_t N, int64_t ldp,
                    int64_t plane_stride, int64_t chunk_stride, cplx* out, int64_t ldo,
                    bool accumulate) {
    if (M <= 0 || N <= 0) return;
    int64_t g = (M * N + 255) / 256;
    g = std::min<int64_t>(g, (int64_t)ctx->sm_count * 16);
    ProfScope ps(ctx, 5, 2.0 * M * N * S, 8.0 * M * N * S + 16.0 * M * N);
    reduce_partials_fp64_kernel<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, ctx->stream>>>(
        P, S, M, N, ldp, plane_stride, chunk_stride, out, ldo, accumulate ? 1 : 0);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
}

}  // namespace tn
