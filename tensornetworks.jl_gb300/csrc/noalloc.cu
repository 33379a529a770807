// Two-site effective-Hamiltonian product that allocates nothing.
//
// Some callers cannot call cudaMalloc.  A host that owns the device memory
// itself (a Julia or C++ program with its own arena and a fixed memory
// budget) hands the library buffers carved from that arena and does not let
// a library allocate behind its back; a long-running loop must not fail with
// an out-of-memory error halfway through a run because another process
// took the memory.  For them this entry point takes device pointers for all
// inputs and the output and keeps its intermediates (the L*theta product,
// the W12-leg product and the merged two-site MPO operator) in one
// file-scope static device array of fixed size, reserved when the library is
// loaded onto a GPU.
//
// Limits and sharing:
//  * the array holds TN_NOALLOC_SCRATCH_BYTES (64 MiB) on every GPU that loads
//    this library, until the process exits;
//  * intermediates must fit it: 16*chil*chir*d^2*(wl+wr) + 16*(wl*d^2)*(d^2*wr)
//    bytes (plus alignment padding), and the merged operator may have at most
//    4096 entries (it is staged whole in 64 KiB of shared memory); larger
//    problems are rejected with TN_ERR_INVALID before anything runs;
//  * every call uses the same array, which keeps the previous call's
//    contents; nothing in it needs to start at zero because every
//    intermediate is fully overwritten before it is read;
//  * calls whose GPU work overlaps (several streams, threads or contexts at
//    once) race on the array and must be serialised by the caller;
//  * like every entry point of the library, a call returns after its work has
//    finished on the context's stream;
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress, with the context's device made current; make that
//    first call before any stream capture.
#include <mutex>

#include "mps.cuh"

namespace tn {

constexpr size_t TN_NOALLOC_SCRATCH_BYTES = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[TN_NOALLOC_SCRATCH_BYTES];

namespace {

// W12[(w,s1,s2),(s1',s2',w'')] = sum_v W1[w,s1',s1,v] W2[v,s2',s2,w'']
__global__ void w12_kernel(const cplx* __restrict__ W1, const cplx* __restrict__ W2, int d,
                           int64_t wl, int64_t wm, int64_t wr, cplx* __restrict__ M) {
    const int64_t nI = wl * d * d, nJ = (int64_t)d * d * wr;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nI * nJ;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t I = e % nI, J = e / nI;
        const int64_t w = I % wl, s1 = (I / wl) % d, s2 = I / (wl * d);
        const int64_t p1 = J % d, p2 = (J / d) % d, w2 = J / (d * d);
        cplx acc = cmk(0, 0);
        for (int64_t v = 0; v < wm; ++v)
            acc = cfma(W1[w + wl * (p1 + d * (s1 + d * v))], W2[v + wm * (p2 + d * (s2 + d * w2))], acc);
        M[e] = acc;
    }
}

std::mutex g_addr_mu;
void* g_addr[64] = {nullptr};

// Device address of the static array on `device`, resolved once per device
// with that device current (the symbol names a different allocation on
// every GPU that loaded the library).
void* scratch_address(int device) {
    TN_REQUIRE(device >= 0 && device < 64, "device index out of range");
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[device]) {
        int cur = -1;
        TN_CHECK_CUDA(cudaGetDevice(&cur));
        TN_REQUIRE(cur == device, "the context's device must be current");
        void* p = nullptr;
        TN_CHECK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_addr[device] = p;
    }
    return g_addr[device];
}

// Accepts device memory of the context's GPU and managed memory; rejects
// host memory and other GPUs' memory.
void require_device_pointer(const void* p, const char* what, int device) {
    cudaPointerAttributes a;
    TN_CHECK_CUDA(cudaPointerGetAttributes(&a, p));
    TN_REQUIRE(a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged,
               std::string(what) + " must be a device pointer");
    TN_REQUIRE(a.type == cudaMemoryTypeManaged || a.device == device,
               std::string(what) + " lives on another GPU than the context's");
}

inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

void heff2_noalloc(Ctx* ctx, int64_t cl, int64_t cr, int d, int64_t wl, int64_t wm, int64_t wr,
                   const cplx* L, const cplx* W1, const cplx* W2, const cplx* R, const cplx* theta,
                   cplx* out) {
    TN_REQUIRE(cl >= 1 && cr >= 1 && d >= 1 && wl >= 1 && wm >= 1 && wr >= 1, "bad dimensions");
    const int64_t d2 = (int64_t)d * d;
    const size_t bT1 = align256(sizeof(cplx) * (size_t)cl * wl * d2 * cr);
    const size_t bT2 = align256(sizeof(cplx) * (size_t)cl * d2 * wr * cr);
    const size_t bW = align256(sizeof(cplx) * (size_t)(wl * d2) * (d2 * wr));
    TN_REQUIRE(bT1 + bT2 + bW <= TN_NOALLOC_SCRATCH_BYTES,
               "problem exceeds the 64 MiB static scratch of the allocation-free H_eff entry point");
    TN_REQUIRE((wl * d2) * (d2 * wr) <= 4096,
               "merged two-site operator above 4096 entries (64 KiB of shared memory)");
    // every launch below goes to the context's stream, and the array's
    // address is per device: make the context's device current first
    TN_CHECK_CUDA(cudaSetDevice(ctx->device));
    const void* ptrs[] = {L, W1, W2, R, theta, out};
    const char* names[] = {"L", "W1", "W2", "R", "theta", "out"};
    for (int i = 0; i < 6; ++i) require_device_pointer(ptrs[i], names[i], ctx->device);
    unsigned char* base = static_cast<unsigned char*>(scratch_address(ctx->device));
    cplx* T1 = reinterpret_cast<cplx*>(base);
    cplx* T2 = reinterpret_cast<cplx*>(base + bT1);
    cplx* W12 = reinterpret_cast<cplx*>(base + bT1 + bT2);
    const int64_t nW = (wl * d2) * (d2 * wr);
    w12_kernel<<<(unsigned)((nW + 255) / 256), 256, 0, ctx->stream>>>(W1, W2, d, wl, wm, wr, W12);
    ctx->count();
    TN_CHECK_CUDA(cudaGetLastError());
    const cplx one = cmk(1, 0), zero = cmk(0, 0);
    // the GEMMs run unsplit: split-K partials would come from the pool
    struct NoSplit {
        Ctx* c;
        bool old;
        ~NoSplit() { c->splitk = old; }
    } guard{ctx, ctx->splitk};
    ctx->splitk = false;
    // T1[(a w), (s1 s2 c)] = L[(a w), b] theta[b, (s1 s2 c)]
    zgemm(ctx, OP_N, OP_N, cl * wl, d2 * cr, cl, one, L, cl * wl, 0, theta, cl, 0, zero, T1, cl * wl, 0);
    // T2[a, (s1' s2' w''), c] = sum W12 T1
    small_apply(ctx, T1, T2, W12, (int)(wl * d2), (int)(d2 * wr), cl, cr, cl, cl * wl * d2, cl,
                cl * d2 * wr);
    // out[(a s1' s2'), c'] = T2[(a s1' s2'), (w'' c)] R[c', (w'' c)]^T
    zgemm(ctx, OP_N, OP_T, cl * d2, cr, wr * cr, one, T2, cl * d2, 0, R, cr, 0, zero, out, cl * d2, 0);
    ctx->sync();
}

}  // namespace tn
