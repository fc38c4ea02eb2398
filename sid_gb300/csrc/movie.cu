// movie.cu -- whole-movie scans: the rank-1 background factorisation and the
// standard-deviation image (rank_1_factorization.m, compute_std_image.m).
//
// The movie Y is P x F, column-major (frame j is the contiguous column
// Y(:, j)), FP32 or FP16.  Both scans are HBM-bound:
//   column pass  t_j = sum_i s_i Y(i, j)            one CTA per frame
//   row pass     s_i = sum_j Y(i, j) t_j, and optionally A_i = sum_j Y(i,j)^2,
//                B_i = sum_j Y(i, j)                 one thread per pixel, t staged
//                                                    in shared memory by frame chunks
// Each byte of Y is read once per pass; the standard-deviation image needs A
// and B, which the last spatial update of the factorisation computes in the
// same pass.  Sums are FP32 over blocks of kSub terms, the blocks added as
// unevaluated FP32 pairs hi + lo (two-sum: FP64 accuracy on the FP32 pipes;
// GB300's FP64 rate is about 1/64 of FP32, and an FP64 add per block held the
// passes below the HBM rate).
#include <algorithm>
#include <cuda_fp16.h>

#include "sid_internal.cuh"

namespace sid {

namespace {

constexpr int kThreads = 256;
constexpr int kSub = 32;        // FP32 terms per pair addition
constexpr int kTChunk = 2048;   // frames of t staged per shared-memory round

__device__ __forceinline__ float ld(const float* p) { return __ldcs(p); }
__device__ __forceinline__ float ld(const __half* p) { return __half2float(__ldcs(p)); }

__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    const float l = (a.y + b.y) + e;
    const float hi = s + l;
    return make_float2(hi, l - (hi - s));
}

__device__ __forceinline__ float2 ff_add(float2 a, float b) { return ff_add(a, make_float2(b, 0.f)); }

__device__ __forceinline__ float2 warp_sum_ff(float2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
    return v;
}

// block sum of pairs, as FP64 in thread 0
__device__ __forceinline__ double block_sum_ff(float2 v, float2* red)
{
    v = warp_sum_ff(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        float2 t = red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = ff_add(t, red[w]);
        r = (double)t.x + (double)t.y;
    }
    return r;  // valid in thread 0
}

__device__ __forceinline__ double block_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    if (warp == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;  // valid in thread 0
}

// 8 consecutive movie values from a 16-byte aligned address
__device__ __forceinline__ void ld8(const __half* p, float (&v)[8])
{
    const uint4 w = __ldcs(reinterpret_cast<const uint4*>(p));
    const __half2* h = reinterpret_cast<const __half2*>(&w);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 f = __half22float2(h[q]);
        v[2 * q] = f.x;
        v[2 * q + 1] = f.y;
    }
}
__device__ __forceinline__ void ld8(const float* p, float (&v)[8])
{
    const float4 a = __ldcs(reinterpret_cast<const float4*>(p)), b = __ldcs(reinterpret_cast<const float4*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Four copies of s shifted by a = 0..3 elements: s4[a * ps + a + i] = s[i], so
// that s4 + a * ps + a + head is 16-byte aligned whenever head + a = 0 (mod 4).
__global__ void k_shift4(const float* __restrict__ s, int64_t P, int64_t ps, float* __restrict__ s4)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = s[i];
#pragma unroll
        for (int a = 0; a < 4; ++a) s4[a * ps + a + i] = v;
    }
}

// t_j = scale_s * sum_i s_i Y(i, j); s == nullptr means s_i = 1 (s4: the
// shifted copies of s).  Each frame column is read with 16-byte loads from its
// first 16-byte aligned element (a scalar head and tail around it), four
// vectors in flight per thread; the weights of the vectors come from the copy
// of s in which they are 16-byte aligned.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_col_pass(const T* __restrict__ Y, int64_t P, int64_t F, const float* __restrict__ s, const float* __restrict__ s4,
           int64_t ps, float scale_s, double* __restrict__ t)
{
    constexpr int U = 4;
    __shared__ float2 red[kThreads / 32];
    for (int64_t j = blockIdx.x; j < F; j += gridDim.x) {
        const T* col = Y + j * P;
        const int64_t head = std::min<int64_t>(P, (int64_t)(((16 - ((uintptr_t)col & 15)) & 15) / sizeof(T)));
        const int64_t nv = (P - head) / 8;
        float2 acc = make_float2(0.f, 0.f);
        float part = 0.f;
        for (int64_t i = threadIdx.x; i < head; i += kThreads) part = fmaf(s ? s[i] : 1.f, ld(col + i), part);
        for (int64_t i = head + nv * 8 + threadIdx.x; i < P; i += kThreads) part = fmaf(s ? s[i] : 1.f, ld(col + i), part);
        acc = ff_add(acc, part);
        const T* body = col + head;
        const int a = (int)((4 - head % 4) % 4);
        const float* sb = s ? s4 + a * ps + a + head : nullptr;
        for (int64_t v0 = threadIdx.x; v0 < nv; v0 += (int64_t)U * kThreads) {
            float y[U][8];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t v = v0 + (int64_t)u * kThreads;
                if (v < nv) ld8(body + v * 8, y[u]);
                else {
#pragma unroll
                    for (int q = 0; q < 8; ++q) y[u][q] = 0.f;
                }
            }
            float p2 = 0.f;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t v = v0 + (int64_t)u * kThreads;
                if (v >= nv) continue;
                if (!sb) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) p2 += y[u][q];
                } else {
                    const float4 a = reinterpret_cast<const float4*>(sb + v * 8)[0];
                    const float4 b = reinterpret_cast<const float4*>(sb + v * 8)[1];
                    p2 = fmaf(a.x, y[u][0], p2); p2 = fmaf(a.y, y[u][1], p2);
                    p2 = fmaf(a.z, y[u][2], p2); p2 = fmaf(a.w, y[u][3], p2);
                    p2 = fmaf(b.x, y[u][4], p2); p2 = fmaf(b.y, y[u][5], p2);
                    p2 = fmaf(b.z, y[u][6], p2); p2 = fmaf(b.w, y[u][7], p2);
                }
            }
            acc = ff_add(acc, p2);
        }
        const double tot = block_sum_ff(acc, red);
        if (threadIdx.x == 0) t[j] = tot * (double)scale_s;
    }
}

// Per pixel i: s_i = sum_j Y(i,j) t_j (t != nullptr), A_i = sum_j Y(i,j)^2 and
// B_i = sum_j Y(i,j) (stats != 0).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_row_pass(const T* __restrict__ Y, int64_t P, int64_t F, const float* __restrict__ t, double* __restrict__ s_out,
           double* __restrict__ a_out, double* __restrict__ b_out, int stats)
{
    __shared__ float ts[kTChunk];
    const int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x;
    const bool live = i < P;
    float2 sd = make_float2(0.f, 0.f), ad = sd, bd = sd;
    for (int64_t j0 = 0; j0 < F; j0 += kTChunk) {
        const int nj = (int)std::min<int64_t>(kTChunk, F - j0);
        if (t) {
            __syncthreads();
            for (int k = threadIdx.x; k < nj; k += kThreads) ts[k] = t[j0 + k];
            __syncthreads();
        }
        if (!live) continue;
        const T* yp = Y + i + j0 * P;
        for (int k0 = 0; k0 < nj; k0 += kSub) {
            const int kn = min(kSub, nj - k0);
            float sp = 0.f, ap = 0.f, bp = 0.f;
            if (kn == kSub) {
                float y[kSub];
#pragma unroll
                for (int k = 0; k < kSub; ++k) y[k] = ld(yp + (int64_t)(k0 + k) * P);
#pragma unroll
                for (int k = 0; k < kSub; ++k) {
                    if (t) sp = fmaf(y[k], ts[k0 + k], sp);
                    if (stats) {
                        ap = fmaf(y[k], y[k], ap);
                        bp += y[k];
                    }
                }
            } else {
                for (int k = 0; k < kn; ++k) {
                    const float y = ld(yp + (int64_t)(k0 + k) * P);
                    if (t) sp = fmaf(y, ts[k0 + k], sp);
                    if (stats) {
                        ap = fmaf(y, y, ap);
                        bp += y;
                    }
                }
            }
            if (t) sd = ff_add(sd, sp);
            if (stats) {
                ad = ff_add(ad, ap);
                bd = ff_add(bd, bp);
            }
        }
    }
    if (!live) return;
    if (s_out) s_out[i] = (double)sd.x + (double)sd.y;
    if (stats) {
        a_out[i] = (double)ad.x + (double)ad.y;
        b_out[i] = (double)bd.x + (double)bd.y;
    }
}

// sum of squares of x (n doubles) -> *out, and 1/sqrt of it -> *inv (one CTA)
__global__ void k_sumsq(const double* __restrict__ x, int64_t n, double* __restrict__ out, double* __restrict__ inv)
{
    __shared__ double red[kThreads / 32];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += kThreads) acc += x[i] * x[i];
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) {
        *out = acc;
        *inv = 1.0 / sqrt(acc);
    }
}

// partial sums of squares per CTA; the last CTA adds them (deterministic order)
__global__ void k_sumsq_big(const double* __restrict__ x, int64_t n, double* __restrict__ part,
                            unsigned int* __restrict__ done, double* __restrict__ out, double* __restrict__ inv)
{
    __shared__ double red[kThreads / 32];
    __shared__ bool last;
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads)
        acc += x[i] * x[i];
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = acc;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last CTA adds the partials, all its threads in a fixed order (a
    // single thread's chain of dependent FP64 adds is slow on GB300)
    __threadfence();
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kThreads) s += part[b];
    s = block_sum(s, red);
    if (threadIdx.x == 0) {
        *out = s;
        *inv = 1.0 / sqrt(s);
        *done = 0;
    }
}

// y = x * (*inv) (or x when inv == nullptr; inv = 1/sqrt of the sum of squares,
// formed once by the reduction, not per thread), FP64 -> FP32
__global__ void k_scale_out(const double* __restrict__ x, int64_t n, const double* __restrict__ inv,
                            float* __restrict__ y)
{
    const double v = inv ? *inv : 1.0;
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads)
        y[i] = (float)(x[i] * v);
}

// mean of y2 (F floats; y2 == nullptr: 0) -> *c (one CTA)
__global__ void k_mean(const float* __restrict__ y2, int64_t F, double* __restrict__ c)
{
    __shared__ double red[kThreads / 32];
    double acc = 0.0;
    if (y2)
        for (int64_t i = threadIdx.x; i < F; i += kThreads) acc += y2[i];
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) *c = acc / (double)F;
}

// std = sqrt((A - y1^2)/F - Bm^2 + 2 Bm y1 C - y1^2 C^2), Bm = B / F
// (compute_std_image.m:22-26); negative rounding residue -> 0.
__global__ void k_std(const double* __restrict__ A, const double* __restrict__ B, const float* __restrict__ y1,
                      const double* __restrict__ c, int64_t P, int64_t F, float* __restrict__ out)
{
    const double C = *c, invF = 1.0 / (double)F;
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < P; i += (int64_t)gridDim.x * kThreads) {
        const double a = y1 ? (double)y1[i] : 0.0;
        const double bm = B[i] * invF;
        const double v = (A[i] - a * a) * invF - bm * bm + 2.0 * bm * a * C - a * a * C * C;
        out[i] = (float)sqrt(v > 0.0 ? v : 0.0);
    }
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>(cdiv(n, kThreads), 152 * 16); }

template <typename T>
int background(sid_ctx* c, const T* Y, int64_t P, int64_t F, int maxIter, float* bg_s, float* bg_t, float* std_img,
               cudaStream_t st)
{
    SID_TRY(c->bg[0].alloc((size_t)P * sizeof(double)));                  // s (FP64)
    SID_TRY(c->bg[1].alloc((size_t)(F + 4096) * sizeof(double)));         // t, scalars, partials
    SID_TRY(c->bg[4].alloc(sizeof(unsigned int)));
    const int64_t ps = cdiv(P + 4, 4) * 4;  // pitch of the shifted weight copies
    if (maxIter > 1) SID_TRY(c->bg[5].alloc((size_t)(4 * ps) * sizeof(float)));
    float* s4 = maxIter > 1 ? c->bg[5].as<float>() : nullptr;
    double* sd = c->bg[0].as<double>();
    double* td = c->bg[1].as<double>();
    double* ss = td + F;       // sum of squares of t or s
    double* cm = td + F + 1;   // mean of t
    double* inv = td + F + 2;  // 1/sqrt(*ss)
    double* part = td + F + 8;
    unsigned int* done = c->bg[4].as<unsigned int>();
    SID_CUDA_TRY(cudaMemsetAsync(done, 0, sizeof(unsigned int), st));
    const bool stats = std_img != nullptr;
    if (stats) {
        SID_TRY(c->bg[2].alloc((size_t)P * sizeof(double)));
        SID_TRY(c->bg[3].alloc((size_t)P * sizeof(double)));
    }
    const unsigned gcol = (unsigned)std::min<int64_t>(F, 152 * 8), grow = (unsigned)cdiv(P, kThreads);
    const unsigned gred = std::min<unsigned>(grid_for(P), 4000);
    for (int it = 1; it <= maxIter; ++it) {
        // bg_temporal = bg_spatial' * Y, normalised (rank_1_factorization.m:33-34); the
        // first bg_spatial is ones / sqrt(P) (:30)
        if (it == 1) {
            k_col_pass<T><<<gcol, kThreads, 0, st>>>(Y, P, F, nullptr, nullptr, 0, (float)(1.0 / sqrt((double)P)), td);
        } else {
            k_shift4<<<grid_for(P), kThreads, 0, st>>>(bg_s, P, ps, s4);
            SID_CHECK_LAUNCH();
            k_col_pass<T><<<gcol, kThreads, 0, st>>>(Y, P, F, bg_s, s4, ps, 1.f, td);
        }
        SID_CHECK_LAUNCH();
        k_sumsq<<<1, kThreads, 0, st>>>(td, F, ss, inv);
        SID_CHECK_LAUNCH();
        k_scale_out<<<grid_for(F), kThreads, 0, st>>>(td, F, inv, bg_t);
        SID_CHECK_LAUNCH();
        // bg_spatial = Y * bg_temporal' (:35), normalised except after the last iteration (:36-38)
        const bool last = it == maxIter;
        k_row_pass<T><<<grow, kThreads, 0, st>>>(Y, P, F, bg_t, sd, stats && last ? c->bg[2].as<double>() : nullptr,
                                                 stats && last ? c->bg[3].as<double>() : nullptr,
                                                 stats && last ? 1 : 0);
        SID_CHECK_LAUNCH();
        if (!last) {
            k_sumsq_big<<<gred, kThreads, 0, st>>>(sd, P, part, done, ss, inv);
            SID_CHECK_LAUNCH();
        }
        k_scale_out<<<grid_for(P), kThreads, 0, st>>>(sd, P, last ? nullptr : inv, bg_s);
        SID_CHECK_LAUNCH();
    }
    if (stats) {
        k_mean<<<1, kThreads, 0, st>>>(bg_t, F, cm);
        SID_CHECK_LAUNCH();
        k_std<<<grid_for(P), kThreads, 0, st>>>(c->bg[2].as<double>(), c->bg[3].as<double>(), bg_s, cm, P, F,
                                                  std_img);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

template <typename T>
int std_image(sid_ctx* c, const T* Y, int64_t P, int64_t F, const float* y1, const float* y2, float* out,
              cudaStream_t st)
{
    SID_TRY(c->bg[1].alloc((size_t)(F + 4096) * sizeof(double)));
    SID_TRY(c->bg[2].alloc((size_t)P * sizeof(double)));
    SID_TRY(c->bg[3].alloc((size_t)P * sizeof(double)));
    double* cm = c->bg[1].as<double>() + F + 1;
    k_row_pass<T><<<(unsigned)cdiv(P, kThreads), kThreads, 0, st>>>(Y, P, F, nullptr, nullptr, c->bg[2].as<double>(),
                                                                    c->bg[3].as<double>(), 1);
    SID_CHECK_LAUNCH();
    k_mean<<<1, kThreads, 0, st>>>(y2, F, cm);
    SID_CHECK_LAUNCH();
    k_std<<<grid_for(P), kThreads, 0, st>>>(c->bg[2].as<double>(), c->bg[3].as<double>(), y1, cm, P, F, out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace

}  // namespace sid

using namespace sid;

extern "C" int sid_rank1_background(sid_ctx* c, const void* Y, int ydtype, int64_t P, int64_t F, int maxIter,
                                    float* bg_spatial, float* bg_temporal, float* std_img, void* stream)
{
    SID_REQUIRE(c && Y && bg_spatial && bg_temporal, "sid_rank1_background: NULL argument");
    SID_REQUIRE(P > 0 && F > 0, "sid_rank1_background: empty movie (P=%lld F=%lld)", (long long)P, (long long)F);
    SID_REQUIRE(maxIter >= 1, "sid_rank1_background: maxIter must be >= 1 (rank_1_factorization.m:31)");
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "sid_rank1_background: unknown dtype %d", ydtype);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (ydtype == SID_DTYPE_F16)
        return background(c, static_cast<const __half*>(Y), P, F, maxIter, bg_spatial, bg_temporal, std_img, st);
    return background(c, static_cast<const float*>(Y), P, F, maxIter, bg_spatial, bg_temporal, std_img, st);
}

extern "C" int sid_std_image(sid_ctx* c, const void* Y, int ydtype, int64_t P, int64_t F, const float* y1,
                             const float* y2, float* out, void* stream)
{
    SID_REQUIRE(c && Y && out, "sid_std_image: NULL argument");
    SID_REQUIRE(P > 0 && F > 0, "sid_std_image: empty movie (P=%lld F=%lld)", (long long)P, (long long)F);
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "sid_std_image: unknown dtype %d", ydtype);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (ydtype == SID_DTYPE_F16) return std_image(c, static_cast<const __half*>(Y), P, F, y1, y2, out, st);
    return std_image(c, static_cast<const float*>(Y), P, F, y1, y2, out, st);
}
