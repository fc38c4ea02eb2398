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
//   * the first call on a device looks the array's address up with
//     cudaGetSymbolAddress (host code cannot use the array's name as a device
//     address); make that first call before any stream capture.
#include <mutex>

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
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

static std::mutex g_noalloc_mu;
static float* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
static int noalloc_scratch(float** out)
{
    int dev = -1;
    SID_CUDA_TRY(cudaGetDevice(&dev));
    SID_REQUIRE(dev >= 0 && dev < kMaxDevices, "sid_gram_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("sid_gram_noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                      cudaGetErrorString(e));
            return SID_ECUDA;
        }
        g_noalloc_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return SID_OK;
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
    while (tiles * splitk < 4 * 152 && nkb / (splitk + 1) >= 16 && splitk + 1 <= cap) ++splitk;
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
