// noalloc.cu -- Gram product G = A'A that allocates no device memory.
//
// Some callers cannot let a library allocate: a MATLAB MEX function whose
// device memory belongs to MATLAB's gpuArray memory manager (which caches
// freed blocks, so a cudaMalloc from outside it can fail even with room in the
// pool, and cudaFree synchronises the whole device), or an acquisition program
// that reserves the GPU's memory up front.  sid_gram_noalloc serves them: it
// computes the same FP32 SIMT Gram product as sid_gram(..., SID_PREC_FP32)
// without a context, keeping its split-K partial sums in the fixed device
// array below instead of a context workspace.
//
// Limits and sharing:
//   * the array holds kNoAllocScratchFloats floats (16 MiB); K is limited to
//     kNoAllocMaxK = 2048 so that at least one K x K partial fits, and the
//     split-K factor is capped to what fits;
//   * the array lives in every GPU that loads libsid until the process exits;
//   * all calls share it and it keeps the last call's contents: calls whose
//     kernels overlap on the GPU (different streams, or different host
//     threads) race on it and must be serialised by the caller;
//   * every call overwrites each partial it later reads, so nothing in the
//     array has to start at zero;
//   * the first call in a CUDA context looks the array's address up with
//     cudaGetSymbolAddress (host code cannot use the array's name as a device
//     address) and keeps it for that context; make that first call before any
//     stream capture.  The address is keyed by the driver's context ID, so a
//     device reset (MATLAB's reset(gpuDevice)) or a second context on the same
//     device looks it up again instead of reusing a stale address.
#include <cuda.h>

#include "ctx_cache.h"
#include "sid_internal.cuh"

namespace sid {

// FP32 SIMT GEMM kernels of gemm_simt.cu (launched through their host stubs)
__global__ void k_sgemm_tn(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C, int m,
                           int n, int k, int64_t lda, int64_t ldb, int64_t ldc, int kb_per, int64_t split_stride);
__global__ void k_splitk_reduce_simt(const float* __restrict__ part, int nsplit, int64_t split_stride, int m, int n,
                                     float* __restrict__ C, int64_t ldc, float alpha, float beta);

constexpr int64_t kNoAllocScratchFloats = 4 * 1024 * 1024;  // 16 MiB
constexpr int64_t kNoAllocMaxK = 2048;                      // 2048^2 floats = the whole array
constexpr int kNaBM = 128, kNaBN = 128, kNaBK = 16;         // tile of k_sgemm_tn

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

static CtxCache<float*> g_noalloc_cache;

using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Unique ID of the context current on this thread (binding the device's primary
// context first if the runtime has not yet done so on this thread).
static int current_context_id(unsigned long long* id)
{
    static std::once_flag once;
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    });
    if (!get_current || !get_id) {
        set_error("sid_gram_noalloc: cuCtxGetCurrent/cuCtxGetId are not available from the driver");
        return SID_ECUDA;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS) {
        set_error("sid_gram_noalloc: cuCtxGetCurrent failed");
        return SID_ECUDA;
    }
    if (!ctx) {
        // no context bound to this thread yet: a runtime call that needs one binds the primary context
        void* p = nullptr;
        SID_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (get_current(&ctx) != CUDA_SUCCESS || !ctx) {
            set_error("sid_gram_noalloc: no CUDA context is current");
            return SID_ECUDA;
        }
    }
    if (get_id(ctx, id) != CUDA_SUCCESS) {
        set_error("sid_gram_noalloc: cuCtxGetId failed");
        return SID_ECUDA;
    }
    return SID_OK;
}

// Device address of g_noalloc_scratch in the current context (looked up once per context).
static int noalloc_scratch(float** out)
{
    unsigned long long id = 0;
    SID_TRY(current_context_id(&id));
    return g_noalloc_cache.get(
        id,
        [](float** v) -> int {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_error("sid_gram_noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                          cudaGetErrorString(e));
                return SID_ECUDA;
            }
            *v = static_cast<float*>(p);
            return SID_OK;
        },
        out);
}

}  // namespace sid

using namespace sid;

extern "C" int sid_gram_noalloc(const float* A, int64_t P, int64_t K, float* G, void* stream)
{
    SID_REQUIRE(A && G, "sid_gram_noalloc: NULL argument");
    SID_REQUIRE(P > 0 && K > 0, "sid_gram_noalloc: empty matrix (P=%lld K=%lld)", (long long)P, (long long)K);
    SID_REQUIRE(K <= kNoAllocMaxK,
                "sid_gram_noalloc: K=%lld exceeds the fixed scratch limit of %lld components "
                "(use sid_gram with a context for larger problems)",
                (long long)K, (long long)kNoAllocMaxK);
    SID_REQUIRE(P <= INT32_MAX, "sid_gram_noalloc: P=%lld exceeds 2^31-1", (long long)P);
    float* scratch = nullptr;
    SID_TRY(noalloc_scratch(&scratch));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // split-K factor: enough CTAs to fill the GPU, capped by the scratch size
    const int64_t tiles = cdiv(K, kNaBM) * cdiv(K, kNaBN);
    const int64_t nkb = cdiv(P, kNaBK);
    const int64_t cap = kNoAllocScratchFloats / (K * K);
    int64_t splitk = 1;
    while (tiles * splitk < 4 * sm_count() && nkb / (splitk + 1) >= 16 && splitk + 1 <= cap) ++splitk;
    const int64_t kb_per = cdiv(nkb, splitk);
    splitk = cdiv(nkb, kb_per);
    const int64_t sstride = K * K;
    dim3 grid((unsigned)cdiv(K, kNaBM), (unsigned)cdiv(K, kNaBN), (unsigned)splitk);
    k_sgemm_tn<<<grid, 256, 0, st>>>(A, A, scratch, (int)K, (int)K, (int)P, P, P, K, (int)kb_per, sstride);
    SID_CHECK_LAUNCH();
    k_splitk_reduce_simt<<<1024, 256, 0, st>>>(scratch, (int)splitk, sstride, (int)K, (int)K, G, K, 1.f, 0.f);
    SID_CHECK_LAUNCH();
    return SID_OK;
}
