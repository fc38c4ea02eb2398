// gemm_simt.cu -- FP32 SIMT GEMM (the plain-precision path of the NNLS
// contractions) and the FP32 -> 16-bit operand split kernels for gemm_tc.cu.
//
// SGEMM, "TN" like the tensor-core kernel: C (m x n, col-major) = A^T B with
// A k x m and B k x n column-major (k contiguous).  128 x 128 CTA tile,
// 256 threads, 8 x 8 outputs per thread, BK = 16 staged through shared memory
// (transposed to [k][m] so the inner loop is an outer product of two float4
// pairs), register double buffering of the next K slice.
#include <cuda_bf16.h>

#include <algorithm>

#include "sid_internal.cuh"

namespace sid {

constexpr int SG_BM = 128, SG_BN = 128, SG_BK = 16;

__global__ void __launch_bounds__(256)
k_sgemm_tn(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C, int m, int n, int k,
           int64_t lda, int64_t ldb, int64_t ldc, int kb_per, int64_t split_stride)
{
    __shared__ __align__(16) float As[2][SG_BK][SG_BM + 4];
    __shared__ __align__(16) float Bs[2][SG_BK][SG_BN + 4];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * SG_BM, n0 = blockIdx.y * SG_BN;
    const int64_t kbeg = (int64_t)blockIdx.z * kb_per * SG_BK;
    const int64_t kend = min((int64_t)k, kbeg + (int64_t)kb_per * SG_BK);
    // loader mapping: 256 threads x 8 values = 128 rows x 16 k
    const int lr = tid >> 1;            // row (m or n) 0..127
    const int lk = (tid & 1) * 8;       // k offset 0 or 8
    const int tm = (tid & 15) * 4, tn = (tid >> 4) * 4;  // compute mapping: two 4-wide groups per dim

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    float ra[8], rb[8];
    auto gload = [&](int64_t k0) {
        const int gm = m0 + lr, gn = n0 + lr;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int64_t kk = k0 + lk + e;
            ra[e] = (gm < m && kk < kend) ? A[(int64_t)gm * lda + kk] : 0.f;
            rb[e] = (gn < n && kk < kend) ? B[(int64_t)gn * ldb + kk] : 0.f;
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            As[buf][lk + e][lr] = ra[e];
            Bs[buf][lk + e][lr] = rb[e];
        }
    };
    int buf = 0;
    if (kbeg < kend) {
        gload(kbeg);
        sstore(0);
    }
    __syncthreads();
    for (int64_t k0 = kbeg; k0 < kend; k0 += SG_BK) {
        const bool more = k0 + SG_BK < kend;
        if (more) gload(k0 + SG_BK);
#pragma unroll
        for (int kk = 0; kk < SG_BK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][tm]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][tm + 64]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tn]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tn + 64]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (more) {
            sstore(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
    float* out = C + (int64_t)blockIdx.z * split_stride;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = m0 + tm + (i < 4 ? i : 60 + i);
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = n0 + tn + (j < 4 ? j : 60 + j);
            if (c < n) out[(int64_t)r + ldc * c] = acc[i][j];
        }
    }
}

__global__ void k_splitk_reduce_simt(const float* __restrict__ part, int nsplit, int64_t split_stride, int m, int n,
                                     float* __restrict__ C, int64_t ldc, float alpha, float beta)
{
    const int64_t total = (int64_t)m * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % m);
        const int64_t c = i / m;
        float s = 0.f;
        for (int z = 0; z < nsplit; ++z) s += part[z * split_stride + r + (int64_t)m * c];
        float* d = C + r + ldc * c;
        *d = (beta != 0.f) ? alpha * s + beta * *d : alpha * s;
    }
}

// C = alpha * A^T B + beta * C (FP32).  ws >= splitk*m*n floats when splitk > 1
// or alpha/beta are not (1, 0).
int sgemm_tn(const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, float* C,
             int64_t ldc, float alpha, float beta, float* ws, int64_t ws_elems, cudaStream_t st)
{
    SID_REQUIRE(m > 0 && n > 0 && k > 0, "sgemm: empty problem");
    const int64_t tiles = cdiv(m, SG_BM) * cdiv(n, SG_BN);
    const int64_t nkb = cdiv(k, SG_BK);
    int splitk = 1;
    while (tiles * splitk < 4 * sm_count() && nkb / (splitk + 1) >= 16) ++splitk;
    const int kb_per = (int)cdiv(nkb, splitk);
    splitk = (int)cdiv(nkb, kb_per);
    const bool direct = splitk == 1 && alpha == 1.f && beta == 0.f;
    float* out = C;
    int64_t ldo = ldc, ss = 0;
    if (!direct) {
        ss = m * n;
        SID_REQUIRE(ws && ws_elems >= splitk * ss, "sgemm: workspace too small");
        out = ws;
        ldo = m;
    }
    dim3 grid((unsigned)cdiv(m, SG_BM), (unsigned)cdiv(n, SG_BN), (unsigned)splitk);
    k_sgemm_tn<<<grid, 256, 0, st>>>(A, B, out, (int)m, (int)n, (int)k, lda, ldb, ldo, kb_per, ss);
    SID_CHECK_LAUNCH();
    if (!direct) {
        k_splitk_reduce_simt<<<1024, 256, 0, st>>>(ws, splitk, ss, (int)m, (int)n, C, ldc, alpha, beta);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

int64_t sgemm_ws_elems(int64_t m, int64_t n, int64_t k)
{
    const int64_t tiles = cdiv(m, SG_BM) * cdiv(n, SG_BN);
    const int64_t nkb = cdiv(k, SG_BK);
    int splitk = 1;
    while (tiles * splitk < 4 * sm_count() && nkb / (splitk + 1) >= 16) ++splitk;
    return (int64_t)splitk * m * n;
}

// ------------------------------------------------ FP32 -> 16-bit splits ----
// Source: element (kk, r) of a k x rows matrix at src[kk + lds*r] (the
// reduction index contiguous).  Destination: the K-blocked layout of the
// tensor-core GEMM, element (kk, r) at ((kk/64)*rows + r)*64 + kk%64, with
// zeros past k.  hi = round(src*scale), lo = round(src*scale - hi).
// One thread per 4 consecutive elements of one row: 16-byte reads when the
// source allows them, 8-byte writes; a warp covers two 128-byte block rows.
template <bool BF16>
__global__ void k_split16_blk(const float* __restrict__ src, int64_t k, int64_t rows, int64_t lds,
                              uint16_t* __restrict__ hi, uint16_t* __restrict__ lo, float scale, int vec4,
                              const float* __restrict__ dscale)
{
    if (dscale) scale = *dscale;
    const int64_t nkb = (k + 63) / 64;
    const int64_t total = nkb * rows * 16;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(i & 15);
        const int64_t rr = i >> 4;
        const int64_t r = rr % rows, kb = rr / rows;
        const int64_t kk = kb * 64 + g * 4;
        float v[4];
        const float* sp = src + kk + lds * r;
        if (vec4 && kk + 3 < k) {
            const float4 q = *reinterpret_cast<const float4*>(sp);
            v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) v[e] = (kk + e < k) ? sp[e] : 0.f;
        }
        uint16_t h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float x = v[e] * scale;
            if (BF16) {
                const __nv_bfloat16 bh = __float2bfloat16_rn(x);
                h[e] = __bfloat16_as_ushort(bh);
                l[e] = __bfloat16_as_ushort(__float2bfloat16_rn(x - __bfloat162float(bh)));
            } else {
                const __half fh = __float2half_rn(x);
                h[e] = __half_as_ushort(fh);
                l[e] = __half_as_ushort(__float2half_rn(x - __half2float(fh)));
            }
        }
        const int64_t o = rr * 64 + g * 4;  // (kb*rows + r)*64 + 4g
        *reinterpret_cast<uint2*>(hi + o) = make_uint2(h[0] | ((uint32_t)h[1] << 16), h[2] | ((uint32_t)h[3] << 16));
        if (lo) *reinterpret_cast<uint2*>(lo + o) = make_uint2(l[0] | ((uint32_t)l[1] << 16), l[2] | ((uint32_t)l[3] << 16));
    }
}

// 16-bit copy of a k x rows matrix (src[kk + lds*r]) into the K-blocked
// layout.  One thread per 8 elements: 16-byte writes, 16-byte reads when aligned.
__global__ void k_copy16_blk(const uint16_t* __restrict__ src, int64_t k, int64_t rows, int64_t lds,
                             uint16_t* __restrict__ dst, int vec8)
{
    const int64_t nkb = (k + 63) / 64;
    const int64_t total = nkb * rows * 8;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(i & 7);
        const int64_t rr = i >> 3;
        const int64_t r = rr % rows, kb = rr / rows;
        const int64_t kk = kb * 64 + g * 8;
        const uint16_t* sp = src + kk + lds * r;
        uint4 out;
        if (vec8 && kk + 7 < k) {
            out = *reinterpret_cast<const uint4*>(sp);
        } else {
            uint16_t t[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) t[e] = (kk + e < k) ? sp[e] : (uint16_t)0;
            out = make_uint4(t[0] | ((uint32_t)t[1] << 16), t[2] | ((uint32_t)t[3] << 16),
                             t[4] | ((uint32_t)t[5] << 16), t[6] | ((uint32_t)t[7] << 16));
        }
        *reinterpret_cast<uint4*>(dst + rr * 64 + g * 8) = out;
    }
}

// The same K-blocked layouts from a row-contiguous source: element (kk, r) at
// src[r + ldr*kk] (a rows x k column-major matrix, e.g. a pixel-major P x R
// factor).  One CTA per 64 x 64 tile: coalesced reads along r into shared
// memory, then 128-byte block rows written along kk.  MODE 0: FP32 source,
// BF16 hi/lo; MODE 1: FP32 source, FP16 hi/lo of src*scale; MODE 2: 16-bit
// source copied (hi only).
template <int MODE>
__global__ void __launch_bounds__(256) k_blk16_t(const void* __restrict__ src_v, int64_t rows, int64_t k, int64_t ldr,
                                                 uint16_t* __restrict__ hi, uint16_t* __restrict__ lo, float scale,
                                                 const float* __restrict__ dscale)
{
    if (dscale) scale = *dscale;
    __shared__ float tile[64][65];
    __shared__ uint16_t tile16[64][66];
    const int64_t nrt = (rows + 63) / 64, nkt = (k + 63) / 64;
    for (int64_t t = blockIdx.x; t < nrt * nkt; t += gridDim.x) {
        const int64_t r0 = (t % nrt) * 64, kb = t / nrt, k0 = kb * 64;
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * 64; e += 256) {
            const int kk = e >> 6, r = e & 63;
            const bool in = r0 + r < rows && k0 + kk < k;
            if (MODE == 2) {
                const uint16_t* src = static_cast<const uint16_t*>(src_v);
                tile16[kk][r] = in ? src[(r0 + r) + ldr * (k0 + kk)] : (uint16_t)0;
            } else {
                const float* src = static_cast<const float*>(src_v);
                tile[kk][r] = in ? src[(r0 + r) + ldr * (k0 + kk)] : 0.f;
            }
        }
        __syncthreads();
        // 64 rows x 16 groups of 4 consecutive kk
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int r = e >> 4, g = e & 15;
            if (r0 + r >= rows) continue;
            uint16_t h[4], l[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int kk = g * 4 + q;
                if (MODE == 2) {
                    h[q] = tile16[kk][r];
                    l[q] = 0;
                } else if (MODE == 0) {
                    const float x = tile[kk][r];
                    const __nv_bfloat16 bh = __float2bfloat16_rn(x);
                    h[q] = __bfloat16_as_ushort(bh);
                    l[q] = __bfloat16_as_ushort(__float2bfloat16_rn(x - __bfloat162float(bh)));
                } else {
                    const float x = tile[kk][r] * scale;
                    const __half fh = __float2half_rn(x);
                    h[q] = __half_as_ushort(fh);
                    l[q] = __half_as_ushort(__float2half_rn(x - __half2float(fh)));
                }
            }
            const int64_t o = (kb * rows + r0 + r) * 64 + g * 4;
            *reinterpret_cast<uint2*>(hi + o) = make_uint2(h[0] | ((uint32_t)h[1] << 16), h[2] | ((uint32_t)h[3] << 16));
            if (lo && MODE != 2)
                *reinterpret_cast<uint2*>(lo + o) =
                    make_uint2(l[0] | ((uint32_t)l[1] << 16), l[2] | ((uint32_t)l[3] << 16));
        }
    }
}

// max |x| over n floats -> out (float bits, atomicMax; out must start at 0)
__global__ void k_absmax(const float* __restrict__ x, int64_t n, unsigned int* __restrict__ out)
{
    float m = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

int64_t blk16_elems(int64_t k, int64_t rows) { return cdiv(k, 64) * 64 * rows; }

// K-blocked 16-bit split of a k x rows FP32 matrix (see k_split16_blk).  An
// FP16 split multiplies by dscale[0] (device memory) when dscale is given,
// else by scale.
int split16_ds(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
               float scale, const float* dscale, cudaStream_t st)
{
    const int vec4 = ((lds & 3) == 0 && ((uintptr_t)src & 15) == 0) ? 1 : 0;
    const int64_t total = cdiv(k, 64) * rows * 16;
    const unsigned grid = (unsigned)std::min<int64_t>(cdiv(total, 256), 152 * 32);
    if (bf16) k_split16_blk<true><<<grid, 256, 0, st>>>(src, k, rows, lds, hi, lo, scale, vec4, nullptr);
    else k_split16_blk<false><<<grid, 256, 0, st>>>(src, k, rows, lds, hi, lo, scale, vec4, dscale);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int split16(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
            float scale, cudaStream_t st)
{
    return split16_ds(src, k, rows, lds, hi, lo, bf16, scale, nullptr, st);
}

int copy16_blk(const uint16_t* src, int64_t k, int64_t rows, int64_t lds, uint16_t* dst, cudaStream_t st)
{
    const int vec8 = ((lds & 7) == 0 && ((uintptr_t)src & 15) == 0) ? 1 : 0;
    const int64_t total = cdiv(k, 64) * rows * 8;
    const unsigned grid = (unsigned)std::min<int64_t>(cdiv(total, 256), 152 * 32);
    k_copy16_blk<<<grid, 256, 0, st>>>(src, k, rows, lds, dst, vec8);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// K-blocked 16-bit operand (reduction index k) of a rows x k matrix stored
// row-contiguous (src[r + ldr*kk]): FP32 split into BF16 hi/lo (bf16) or FP16
// hi/lo of src*scale, or a 16-bit source copied (src16).
int split16_t_ds(const float* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* hi, uint16_t* lo, bool bf16,
                 float scale, const float* dscale, cudaStream_t st)
{
    const int64_t tiles = cdiv(rows, 64) * cdiv(k, 64);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 152 * 8);
    if (bf16) k_blk16_t<0><<<grid, 256, 0, st>>>(src, rows, k, ldr, hi, lo, 1.f, nullptr);
    else k_blk16_t<1><<<grid, 256, 0, st>>>(src, rows, k, ldr, hi, lo, scale, dscale);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int split16_t(const float* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* hi, uint16_t* lo, bool bf16,
              float scale, cudaStream_t st)
{
    return split16_t_ds(src, rows, k, ldr, hi, lo, bf16, scale, nullptr, st);
}

int copy16_t(const uint16_t* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* dst, cudaStream_t st)
{
    const int64_t tiles = cdiv(rows, 64) * cdiv(k, 64);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 152 * 8);
    k_blk16_t<2><<<grid, 256, 0, st>>>(src, rows, k, ldr, dst, nullptr, 1.f, nullptr);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int absmax(const float* x, int64_t n, unsigned int* out, cudaStream_t st)
{
    SID_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(unsigned int), st));
    k_absmax<<<1024, 256, 0, st>>>(x, n, out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

__global__ void k_amax_pow2(const unsigned int* __restrict__ amax, float* __restrict__ scale)
{
    scale[0] = pow2_for(__uint_as_float(amax[0]));
}

__global__ void k_scale_ratio(const float* __restrict__ a, const float* __restrict__ b, float num,
                              float* __restrict__ out)
{
    out[0] = num / (a[0] * (b ? b[0] : 1.f));
}

// Device-resident power-of-two scale of x (n floats): dscale[0] brings max |x|
// into [2^13, 2^14) (1 for an all-zero or non-finite x); amax is scratch for
// one word.  Nothing is read back, so the stream never waits on the host.
int pow2_scale_dev(const float* x, int64_t n, unsigned int* amax, float* dscale, cudaStream_t st)
{
    SID_TRY(absmax(x, n, amax, st));
    k_amax_pow2<<<1, 1, 0, st>>>(amax, dscale);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// out[0] = num / (a[0] * b[0]) (b may be null), on the device: the alpha that
// undoes two power-of-two operand scales (exact).
int scale_ratio_dev(const float* a, const float* b, float num, float* out, cudaStream_t st)
{
    k_scale_ratio<<<1, 1, 0, st>>>(a, b, num, out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace sid
