// volconv.cu -- the neuron-kernel composition of the projector
// (reconstruct_S.m:126-127,188-189):
//   forwardFUN(X)  = P(convn(X, kernel, 'same'))
//   backwardFUN(y) = convn(P'(y), kernel, 'same')
// with one kernel both ways, as the reference composes them.  MATLAB's convn
// 'same' is the central part of the full convolution:
//   out(x, y, z) = sum_{i,j,l} V(x + ox - i, y + oy - j, z + oz - l) k(i, j, l),
//   (ox, oy, oz) = floor(size(k) / 2), V zero outside the volume.
// The solvers keep volumes in the polyphase layout, where x-neighbours lie in
// different lenslet-phase planes; the convolution therefore runs on the plain
// X x Y x Z layout between a polyphase -> volume and a volume -> polyphase
// conversion.  Kernel: one CTA per 64 x 16 output tile of one depth; for each
// kernel depth slice the input halo (64 + kx - 1) x (16 + ky - 1) is staged in
// shared memory.  Kernels up to 32 taps wide along x run a variant compiled for
// their (rounded) width: 4 x 4 outputs per thread, whole input windows in
// registers; wider ones slide a 4-output register window one tap at a time.
#include <algorithm>

#include "sid_internal.cuh"

namespace sid {

namespace {

constexpr int kTX = 64, kTY = 16, kOut = 4;   // tile, outputs per thread along x
constexpr int kConvThreads = (kTX / kOut) * kTY;  // 256

__global__ void __launch_bounds__(kConvThreads)
k_convn_same(const float* __restrict__ in, float* __restrict__ out, const float* __restrict__ ker, int X, int Y,
             int Z, int kx, int ky, int kz)
{
    extern __shared__ float cs[];
    const int SW = kTX + kx - 1, SH = kTY + ky - 1;
    float* tile = cs;             // [SH][SW]
    float* ks = cs + SW * SH;     // [ky][kx] of the current kernel depth
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z = blockIdx.z;
    const int ox = kx / 2, oy = ky / 2, oz = kz / 2;
    const int tx = threadIdx.x % (kTX / kOut), ty = threadIdx.x / (kTX / kOut);
    float acc[kOut] = {0.f, 0.f, 0.f, 0.f};
    // tile(r, c) = V(x0 + ox - (kx - 1) + c, y0 + oy - (ky - 1) + r, zin)
    const int xs = x0 + ox - (kx - 1), ys = y0 + oy - (ky - 1);
    for (int l = 0; l < kz; ++l) {
        const int zin = z + oz - l;
        if (zin < 0 || zin >= Z) continue;  // uniform over the CTA
        __syncthreads();
        const float* src = in + (int64_t)zin * X * Y;
        for (int e = threadIdx.x; e < SW * SH; e += kConvThreads) {
            const int r = e / SW, c = e - r * SW;
            const int x = xs + c, y = ys + r;
            tile[e] = (x >= 0 && x < X && y >= 0 && y < Y) ? src[(int64_t)y * X + x] : 0.f;
        }
        for (int e = threadIdx.x; e < kx * ky; e += kConvThreads) ks[e] = ker[(int64_t)l * kx * ky + e];
        __syncthreads();
        for (int j = 0; j < ky; ++j) {
            // output row ty at kernel row j reads tile row ty + ky - 1 - j
            const float* row = tile + (ty + ky - 1 - j) * SW + tx * kOut;
            const float* kr = ks + j * kx;
            // window w[q] = row[q + kx - 1 - i] for tap i, starting at i = 0
            float w[kOut];
#pragma unroll
            for (int q = 0; q < kOut; ++q) w[q] = row[q + kx - 1];
            for (int i = 0; i < kx; ++i) {
                const float kv = kr[i];
#pragma unroll
                for (int q = 0; q < kOut; ++q) acc[q] = fmaf(kv, w[q], acc[q]);
                if (i + 1 < kx) {
#pragma unroll
                    for (int q = kOut - 1; q > 0; --q) w[q] = w[q - 1];
                    w[0] = row[kx - 2 - i];
                }
            }
        }
    }
    const int y = y0 + ty;
    if (y >= Y) return;
    float* dst = out + (int64_t)z * X * Y + (int64_t)y * X;
#pragma unroll
    for (int q = 0; q < kOut; ++q) {
        const int x = x0 + tx * kOut + q;
        if (x < X) dst[x] = acc[q];
    }
}

// Tap extent along x known at compile time, rounded up to KXP (a multiple of 4;
// the extra taps are zero).  CTA: 64 x 64 outputs of one depth, each thread a
// 4 x 4 block.  Per kernel row j and output row r the thread loads its input
// window (4 + KXP - 1 values, as 16-byte vectors) once and applies all KXP taps
// from registers.
template <int KXP>
__global__ void __launch_bounds__(256)
k_convn_tiled(const float* __restrict__ in, float* __restrict__ out, const float* __restrict__ ker, int X, int Y,
              int Z, int kx, int ky, int kz)
{
    constexpr int TX = 64, TY = 64;
    constexpr int W = TX + KXP;   // tile pitch: 64 + KXP - 1 columns, padded to a multiple of 4
    constexpr int WIN = KXP + 4;  // window per output row
    extern __shared__ __align__(16) float cs[];
    const int H = TY + ky - 1;
    float* tile = cs;        // [H][W]
    float* ks = cs + H * W;  // [ky][KXP], zero beyond kx
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
    const int ox = kx / 2, oy = ky / 2, oz = kz / 2;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    // tile(r, c) = V(x0 + ox - (KXP - 1) + c, y0 + oy - (ky - 1) + r, zin)
    const int xs = x0 + ox - (KXP - 1), ys = y0 + oy - (ky - 1);
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = 0.f;
    for (int l = 0; l < kz; ++l) {
        const int zin = z + oz - l;
        if (zin < 0 || zin >= Z) continue;  // uniform over the CTA
        __syncthreads();
        const float* src = in + (int64_t)zin * X * Y;
        for (int e = threadIdx.x; e < H * W; e += 256) {
            const int r = e / W, c = e - r * W;
            const int x = xs + c, y = ys + r;
            tile[e] = (c < TX + KXP - 1 && x >= 0 && x < X && y >= 0 && y < Y) ? src[(int64_t)y * X + x] : 0.f;
        }
        for (int e = threadIdx.x; e < ky * KXP; e += 256) {
            const int j = e / KXP, i = e - j * KXP;
            ks[e] = i < kx ? ker[((int64_t)l * ky + j) * kx + i] : 0.f;
        }
        __syncthreads();
        for (int j = 0; j < ky; ++j) {
            float kv[KXP];
#pragma unroll
            for (int i = 0; i < KXP; i += 4) {
                const float4 k4 = *reinterpret_cast<const float4*>(ks + j * KXP + i);
                kv[i] = k4.x;
                kv[i + 1] = k4.y;
                kv[i + 2] = k4.z;
                kv[i + 3] = k4.w;
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float* row = tile + (ty * 4 + r + ky - 1 - j) * W + tx * 4;
                float w[WIN];
#pragma unroll
                for (int m = 0; m < WIN; m += 4) {
                    const float4 v = *reinterpret_cast<const float4*>(row + m);
                    w[m] = v.x;
                    w[m + 1] = v.y;
                    w[m + 2] = v.z;
                    w[m + 3] = v.w;
                }
#pragma unroll
                for (int i = 0; i < KXP; ++i)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[r][q] = fmaf(kv[i], w[q + KXP - 1 - i], acc[r][q]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int y = y0 + ty * 4 + r;
        if (y >= Y) continue;
        float* dst = out + (int64_t)z * X * Y + (int64_t)y * X;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int x = x0 + tx * 4 + q;
            if (x < X) dst[x] = acc[r][q];
        }
    }
}

template <int KXP>
int launch_tiled(const float* a, float* b, const float* ker, int X, int Y, int Z, int kx, int ky, int kz,
                 cudaStream_t st)
{
    const size_t sm = (size_t)((64 + ky - 1) * (64 + KXP) + ky * KXP) * sizeof(float);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_convn_tiled<KXP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 grid((unsigned)cdiv(X, 64), (unsigned)cdiv(Y, 64), (unsigned)Z);
    k_convn_tiled<KXP><<<grid, 256, sm, st>>>(a, b, ker, X, Y, Z, kx, ky, kz);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace

// out_vp = polyphase(convn(volume(in_vp), kernel, 'same')); in_vp and out_vp may alias.
int conv_poly(sid_plan* p, const float* in_vp, float* out_vp, cudaStream_t st)
{
    const int64_t nv = p->X * p->Y * p->Z;
    SID_TRY(p->kvol[0].alloc((size_t)nv * sizeof(float)));
    SID_TRY(p->kvol[1].alloc((size_t)nv * sizeof(float)));
    float* a = p->kvol[0].as<float>();
    float* b = p->kvol[1].as<float>();
    SID_TRY(vp_to_v(p, in_vp, a, p->Z, st));
    const int kx = (int)p->kdims[0], ky = (int)p->kdims[1], kz = (int)p->kdims[2];
    const int X = (int)p->X, Y = (int)p->Y, Z = (int)p->Z;
    const float* ker = p->kern.as<float>();
    int rc = SID_EINVAL;
    switch ((kx + 3) / 4) {
    case 1: rc = launch_tiled<4>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 2: rc = launch_tiled<8>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 3: rc = launch_tiled<12>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 4: rc = launch_tiled<16>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 5: rc = launch_tiled<20>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 6: rc = launch_tiled<24>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 7: rc = launch_tiled<28>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    case 8: rc = launch_tiled<32>(a, b, ker, X, Y, Z, kx, ky, kz, st); break;
    default: break;
    }
    if (kx <= 32) {
        SID_TRY(rc);
        return v_to_vp(p, b, out_vp, p->Z, st);
    }
    // wider kernels: the generic tile
    const size_t sm = (size_t)((kTX + kx - 1) * (kTY + ky - 1) + kx * ky) * sizeof(float);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_convn_same, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 grid((unsigned)cdiv(p->X, kTX), (unsigned)cdiv(p->Y, kTY), (unsigned)p->Z);
    k_convn_same<<<grid, kConvThreads, sm, st>>>(a, b, p->kern.as<float>(), (int)p->X, (int)p->Y, (int)p->Z, kx, ky,
                                                  kz);
    SID_CHECK_LAUNCH();
    return v_to_vp(p, b, out_vp, p->Z, st);
}

}  // namespace sid

using namespace sid;

extern "C" int sid_plan_set_kernel(sid_plan* p, const float* kernel, int64_t kx, int64_t ky, int64_t kz)
{
    SID_REQUIRE(p, "sid_plan_set_kernel: NULL plan");
    if (!kernel || kx <= 0 || ky <= 0 || kz <= 0) {
        p->kern.release();
        p->kvol[0].release();
        p->kvol[1].release();
        p->kvol[2].release();
        p->kdims[0] = p->kdims[1] = p->kdims[2] = 0;
        return SID_OK;
    }
    SID_REQUIRE(kx <= 64 && ky <= 64 && kz <= 64, "sid_plan_set_kernel: kernel %lld x %lld x %lld exceeds 64 per axis",
                (long long)kx, (long long)ky, (long long)kz);
    SID_TRY(p->kern.alloc((size_t)(kx * ky * kz) * sizeof(float)));
    SID_CUDA_TRY(cudaMemcpy(p->kern.p, kernel, (size_t)(kx * ky * kz) * sizeof(float), cudaMemcpyHostToDevice));
    p->kdims[0] = kx;
    p->kdims[1] = ky;
    p->kdims[2] = kz;
    return SID_OK;
}
