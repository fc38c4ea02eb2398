// spec_tc.cu -- the spectral projector's contraction on the tensor cores, for
// many volumes at once (reconstruct_S.m:162-212 reconstructs components side
// by side; forwardProjectGPU.m / backwardProjectGPU_new.m per component).
//
// Per lenslet-grid frequency f the projections are complex matrix products
// (spectral.cu):
//   forward  Ihat[b][o](f) = sum_k  K[f][o][k] Vhat[b][k](f)        n_out x n_in  times n_in  x nb
//   adjoint  Bhat[b][k](f) = sum_o  conj(K[f][o][k]) Ihat[b][o](f)   n_in  x n_out times n_out x nb
// With nb volumes they are GEMMs instead of matrix-vector products, and the
// tap spectra stream from HBM once per nb volumes.  Real form, the complex
// parts interleaved along the reduction index:
//   A, row r (o forward, k adjoint): (Re, Im) pairs of the 24-bit spectra --
//     the [f][o][k] planes for the forward, a transposed [f][k][o] copy for
//     the adjoint, so both are K-major;
//   B, columns 2b and 2b+1 of volume b: forward (Vr, -Vi) and (Vi, Vr),
//     adjoint (Yr, Yi) and (Yi, -Yr);
//   D[r][2b] = Re, D[r][2b+1] = Im.
// Precision.  A 24-bit float (sign, 8-bit exponent, 15 stored mantissa bits,
// spectral.cu f24_split) is exactly the sum of two BF16 numbers: its high 16
// bits, and the remainder below them (at most 8 significant bits).  B is split
// into three BF16 parts hi + mid + lo (24 significant bits, FP32's precision:
// with two parts, 16-17 bits, ISRA from background-clipped components -- which
// divides by near-zero back projections -- landed several times further from
// FP64 than the single-volume mixed form).  Five BF16 MMA passes
// (A_hi (B_hi + B_mid + B_lo) + A_lo (B_hi + B_mid); A_lo B_lo is below 2^-24)
// with FP32 accumulation in TMEM; the accumulator is drained into registers
// every 1024 reduction elements and added there with round-to-nearest (the
// tensor-core accumulator truncates, gemm_tc.cu).
//
// Kernel: persistent, one CTA per SM, over work items (128-row tile, f).  Warp
// 0 lane 0 drives a TMA ring (A high halves 128B-swizzled, A low bytes
// row-major, B hi/lo 128B-swizzled); warps 2-5 build the A remainders in
// shared memory from the high halves and low bytes (same swizzled positions,
// then fence.proxy.async so the tensor core sees them); warp 1 lane 0 issues
// tcgen05.mma (M = 128, N = BN, K = 16) into two TMEM accumulators; warps 6-13
// drain them and write D as complex values [f][b][r].  Every mbarrier wait is
// bounded; on a timeout the kernel stops issuing, waits for its MMAs, frees
// TMEM and reports through the plan's error word.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "ptx.cuh"
#include "sid_internal.cuh"
#include "tc.cuh"

namespace sid {

constexpr int TC_BM = 128;
constexpr int TC_BK = 64;      // 64 x 16-bit = one 128-byte swizzle row
constexpr int TC_KCHUNK = 16;  // K blocks per accumulation chunk (1024 reduction elements)
constexpr int TC_CONV_WARPS = 4;
constexpr int TC_DRAIN_WARPS = 8;
constexpr int TC_THREADS = (2 + TC_CONV_WARPS + TC_DRAIN_WARPS) * 32;
constexpr int kErrTimeoutSpecTc = 3;

struct SpecTcMaps {
    CUtensorMap ahi, alo, bhi, bmi, blo;
};

// NBP: B planes, 3 (hi, mid, lo) or 2 (hi, lo: 16-17 significant bits)
template <int BN, int STAGES, int NBP>
struct SpecTcSmem {
    static_assert(NBP == 2 || NBP == 3, "B is split into two or three BF16 planes");
    static constexpr int AHI = TC_BM * TC_BK * 2;  // 16 KB: high halves (BF16), swizzled
    static constexpr int ALO = AHI;                // remainders (BF16), same layout
    static constexpr int B = BN * TC_BK * 2;       // one B plane
    static constexpr int LO8 = TC_BM * TC_BK;      // 8 KB: low bytes, row-major
    static constexpr int OFF_ALO = AHI;
    static constexpr int OFF_BHI = AHI + ALO;
    static constexpr int OFF_BMI = OFF_BHI + B;    // (three planes)
    static constexpr int OFF_BLO = OFF_BHI + (NBP - 1) * B;
    static constexpr int OFF_LO8 = OFF_BLO + B;
    static constexpr int STAGE = OFF_LO8 + LO8;
    static constexpr int TMA_BYTES = AHI + NBP * B + LO8;
    static constexpr int TOTAL = STAGES * STAGE + 1024;
    static_assert(B % 1024 == 0 && STAGE % 1024 == 0, "stage tiles must stay 1024-byte aligned");
    static_assert(TOTAL <= 227 * 1024, "stages exceed the shared memory of one CTA");
};

// Remainders of one 8-element chunk: hi = 8 BF16 high halves, lo = their low bytes.
__device__ __forceinline__ uint4 f24_remainders(uint4 hi, uint2 lo)
{
    const uint32_t h[4] = {hi.x, hi.y, hi.z, hi.w};
    const uint32_t l[2] = {lo.x, lo.y};
    uint32_t out[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float r[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t h16 = (h[q] >> (16 * e)) & 0xFFFFu;
            const uint32_t l8 = (l[q >> 1] >> (8 * (2 * (q & 1) + e))) & 0xFFu;
            const float fh = __uint_as_float(h16 << 16);
            const float ff = __uint_as_float((h16 << 16) | (l8 << 8));
            r[e] = ff - fh;  // exact: at most 8 significant bits
        }
        const __nv_bfloat162 p = __floats2bfloat162_rn(r[0], r[1]);
        out[q] = *reinterpret_cast<const uint32_t*>(&p);
    }
    return make_uint4(out[0], out[1], out[2], out[3]);
}

// out[(f * nb + b) * rows + r] (float2) = (D[r][2b], D[r][2b+1]) for r < rows, b < nb.
// NBP = 3: five MMA passes A_hi (B_hi + B_mid + B_lo) + A_lo (B_hi + B_mid);
// NBP = 2: three, A_hi (B_hi + B_lo) + A_lo B_hi.
template <int BN, int STAGES, int NBP>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_spec_tc(const __grid_constant__ SpecTcMaps maps, int rows, int nkb, int akb0, int nmt, int64_t nitems, int nb,
          float2* __restrict__ out, int* __restrict__ err)
{
    using SM = SpecTcSmem<BN, STAGES, NBP>;
    constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators
    constexpr int HALF = BN / 2;            // columns per drain warp
    static_assert(HALF % 32 == 0, "BN must be a multiple of 64");
    extern __shared__ uint8_t tsm_raw[];
    uint8_t* tsm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tsm_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full[STAGES], conv[STAGES], empty[STAGES], tfull[2], tempty[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nci = (nkb + TC_KCHUNK - 1) / TC_KCHUNK;
    constexpr int PRODUCER = 0, ISSUER = 1, CONV0 = 2, DRAIN0 = 2 + TC_CONV_WARPS;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&conv[s], TC_CONV_WARPS);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], TC_DRAIN_WARPS * 32);
        }
        mbar_init(&done, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "n"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == PRODUCER) {
        if (lane == 0) {
            int it = 0;
            for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
                const int f = (int)(item / nmt), mt = (int)(item % nmt);
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = it % STAGES;
                    if (*(volatile int*)&abort_flag) break;
                    if (it >= STAGES && !mbar_wait(&empty[s], (uint32_t)(((it / STAGES) - 1) & 1), err)) {
                        atomicExch(&abort_flag, 1);
                        break;
                    }
                    uint8_t* st = tsm + s * SM::STAGE;
                    mbar_arrive_expect_tx(&full[s], SM::TMA_BYTES);
                    tma_load_3d(st, &maps.ahi, (akb0 + kb) * TC_BK, mt * TC_BM, f, &full[s]);
                    tma_load_3d(st + SM::OFF_LO8, &maps.alo, (akb0 + kb) * TC_BK, mt * TC_BM, f, &full[s]);
                    tma_load_3d(st + SM::OFF_BHI, &maps.bhi, kb * TC_BK, 0, f, &full[s]);
                    if (NBP == 3) tma_load_3d(st + SM::OFF_BMI, &maps.bmi, kb * TC_BK, 0, f, &full[s]);
                    tma_load_3d(st + SM::OFF_BLO, &maps.blo, kb * TC_BK, 0, f, &full[s]);
                }
                if (*(volatile int*)&abort_flag) break;
            }
        }
    } else if (warp == ISSUER) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc_m(TC_BM, BN, true);
            int it = 0, c = 0;
            bool ok = true;
            for (int64_t item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
                for (int ci = 0; ci < nci && ok; ++ci, ++c) {
                    const int b = c & 1;
                    if (*(volatile int*)&abort_flag) { ok = false; break; }
                    if (c >= 2 && !mbar_wait(&tempty[b], (uint32_t)(((c >> 1) - 1) & 1), err)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t acc = tmem + (uint32_t)(b * BN);
                    const int kb0 = ci * TC_KCHUNK, kb1 = min(nkb, kb0 + TC_KCHUNK);
                    bool first = true;
                    for (int kb = kb0; kb < kb1; ++kb, ++it) {
                        const int s = it % STAGES;
                        const uint32_t par = (uint32_t)((it / STAGES) & 1);
                        if (!mbar_wait(&full[s], par, err) || !mbar_wait(&conv[s], par, err)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t ahi = smem_u32(tsm + s * SM::STAGE);
                        const uint32_t alo = ahi + SM::OFF_ALO, bhi = ahi + SM::OFF_BHI;
                        const uint32_t bmi = ahi + SM::OFF_BMI, blo = ahi + SM::OFF_BLO;
#pragma unroll
                        for (int kk = 0; kk < TC_BK / 16; ++kk) {
                            const uint32_t o = kk * 32;  // 16 elements inside the 128-byte swizzle row
                            mma_bf16(acc, smem_desc_sw128(ahi + o), smem_desc_sw128(bhi + o), idesc, first ? 0 : 1);
                            first = false;
                            if (NBP == 3) mma_bf16(acc, smem_desc_sw128(ahi + o), smem_desc_sw128(bmi + o), idesc, 1);
                            mma_bf16(acc, smem_desc_sw128(ahi + o), smem_desc_sw128(blo + o), idesc, 1);
                            mma_bf16(acc, smem_desc_sw128(alo + o), smem_desc_sw128(bhi + o), idesc, 1);
                            if (NBP == 3) mma_bf16(acc, smem_desc_sw128(alo + o), smem_desc_sw128(bmi + o), idesc, 1);
                        }
                        mma_commit(&empty[s]);
                    }
                    if (!ok) break;
                    mma_commit(&tfull[b]);
                }
            }
            // every issued MMA has completed before TMEM is released
            mma_commit(&done);
            mbar_wait(&done, 0, err);
            if (!ok) atomicExch(&abort_flag, 1);
        }
    } else if (warp < DRAIN0) {
        // converters: remainders of the 24-bit floats into the A_lo tile
        const int ct = threadIdx.x - CONV0 * 32;
        int it = 0;
        for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
            bool ok = true;
            for (int kb = 0; kb < nkb; ++kb, ++it) {
                const int s = it % STAGES;
                if (*(volatile int*)&abort_flag) { ok = false; break; }
                ok = __all_sync(0xffffffffu, mbar_wait(&full[s], (uint32_t)((it / STAGES) & 1), err));
                if (!ok) {
                    if (lane == 0) atomicExch(&abort_flag, 1);
                    break;
                }
                uint8_t* st = tsm + s * SM::STAGE;
#pragma unroll 2
                for (int q = 0; q < (TC_BM * 8) / (TC_CONV_WARPS * 32); ++q) {
                    const int u = ct + q * TC_CONV_WARPS * 32;
                    const int r = u >> 3, j = u & 7;
                    const int sw = r * 128 + ((j ^ (r & 7)) << 4);  // 128-byte swizzle
                    const uint4 h = *reinterpret_cast<const uint4*>(st + sw);
                    const uint2 l = *reinterpret_cast<const uint2*>(st + SM::OFF_LO8 + r * 64 + j * 8);
                    *reinterpret_cast<uint4*>(st + SM::OFF_ALO + sw) = f24_remainders(h, l);
                }
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&conv[s]);
            }
            if (!ok) break;
        }
    } else {
        // drain warps: warp w reads TMEM lanes 32*(w%4).. and one half of the columns
        const int lg = warp & 3;
        const int ch0 = ((warp - DRAIN0) >> 2) * HALF;
        float accr[HALF];
        int c = 0;
        bool ok = true;
        for (int64_t item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
            const int f = (int)(item / nmt), mt = (int)(item % nmt);
#pragma unroll
            for (int j = 0; j < HALF; ++j) accr[j] = 0.f;
            for (int ci = 0; ci < nci; ++ci, ++c) {
                const int b = c & 1;
                ok = !*(volatile int*)&abort_flag;
                ok = __all_sync(0xffffffffu, ok && mbar_wait(&tfull[b], (uint32_t)((c >> 1) & 1), err));
                if (!ok) break;
                tc_fence_after();
#pragma unroll
                for (int c0 = 0; c0 < HALF; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * BN + ch0 + c0), v);
#pragma unroll
                    for (int j = 0; j < 32; ++j) accr[c0 + j] += v[j];
                }
                tc_fence_before();
                mbar_arrive(&tempty[b]);
            }
            if (!ok) break;
            const int row = mt * TC_BM + lg * 32 + lane;
            if (row < rows) {
#pragma unroll
                for (int j = 0; j < HALF; j += 2) {
                    const int vb = (ch0 + j) >> 1;
                    if (vb < nb) out[((int64_t)f * nb + vb) * rows + row] = make_float2(accr[j], accr[j + 1]);
                }
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TMEM_COLS) : "memory");
    }
    if (threadIdx.x == 0 && abort_flag && err) atomicExch(err, kErrTimeoutSpecTc);
}

// ------------------------------------------------------------ data motion --
// 24-bit spectra transposed per frequency: [f][o][k] -> [f][k][o_pad] (zeros for o >= n_out).
__global__ void k_f24_transpose(const ushort2* __restrict__ h, const uchar2* __restrict__ l, ushort2* __restrict__ th,
                                uchar2* __restrict__ tl, int n_out, int64_t n_in_pad, int o_pad)
{
    __shared__ ushort2 sh[32][33];
    __shared__ uchar2 sl[32][33];
    const int64_t f = blockIdx.z;
    const int64_t k0 = (int64_t)blockIdx.x * 32;
    const int o0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int o = o0 + i;
        const int64_t k = k0 + threadIdx.x;
        const bool in = o < n_out && k < n_in_pad;
        const int64_t src = (f * n_out + o) * n_in_pad + k;
        sh[i][threadIdx.x] = in ? h[src] : make_ushort2(0, 0);
        sl[i][threadIdx.x] = in ? l[src] : make_uchar2(0, 0);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t k = k0 + i;
        const int o = o0 + threadIdx.x;
        if (k < n_in_pad && o < o_pad) {
            const int64_t dst = (f * n_in_pad + k) * o_pad + o;
            th[dst] = sh[threadIdx.x][i];
            tl[dst] = sl[threadIdx.x][i];
        }
    }
}

// B operand planes [f][BN][2 * nch_pad] (BF16 hi, mid and lo) from nb channel
// spectra src[b][c][f] (c < nch); columns of volumes b >= nb and channels
// c >= nch are zero.  ADJ selects the adjoint's column pattern.
template <bool ADJ>
__global__ void k_tc_pack(const float2* __restrict__ src, int nb, int nch, int nch_pad, int nf, int BN,
                          uint32_t* __restrict__ bhi, uint32_t* __restrict__ bmi, uint32_t* __restrict__ blo)
{
    __shared__ float2 t[32][33];
    const int b = blockIdx.z;  // volume, < BN / 2
    const int c0 = blockIdx.x * 32, f0 = blockIdx.y * 32;
    const int tid = threadIdx.x;
    for (int i = tid; i < 32 * 32; i += blockDim.x) {
        const int cc = i >> 5, ff = i & 31;
        const int c = c0 + cc, f = f0 + ff;
        t[cc][ff] = (b < nb && c < nch && f < nf) ? src[((int64_t)b * nch + c) * nf + f] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int64_t kp2 = nch_pad;  // 32-bit words (pairs) per B row
    for (int i = tid; i < 32 * 2 * 32; i += blockDim.x) {
        const int cc = i & 31, col = (i >> 5) & 1, ff = i >> 6;
        const int c = c0 + cc, f = f0 + ff;
        if (c >= nch_pad || f >= nf) continue;
        const float2 v = t[cc][ff];
        float x0, x1;
        if (!ADJ) {
            x0 = col ? v.y : v.x;
            x1 = col ? v.x : -v.y;
        } else {
            x0 = col ? v.y : v.x;
            x1 = col ? -v.x : v.y;
        }
        // x = hi + mid + lo: each remainder is exact in FP32
        const __nv_bfloat162 hi = __floats2bfloat162_rn(x0, x1);
        const float2 hf = __bfloat1622float2(hi);
        const float r0 = x0 - hf.x, r1 = x1 - hf.y;
        const __nv_bfloat162 mi = __floats2bfloat162_rn(r0, r1);
        const float2 mf = __bfloat1622float2(mi);
        const __nv_bfloat162 lo = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
        const int64_t o = ((int64_t)f * BN + 2 * b + col) * kp2 + c;
        bhi[o] = *reinterpret_cast<const uint32_t*>(&hi);
        bmi[o] = *reinterpret_cast<const uint32_t*>(&mi);
        blo[o] = *reinterpret_cast<const uint32_t*>(&lo);
    }
}

// dst[b][c][f] = src[f][b][c] for c < nch (src rows of length rows >= nch)
__global__ void k_tc_unpack(const float2* __restrict__ src, int nb, int rows, int nch, int nf,
                            float2* __restrict__ dst)
{
    __shared__ float2 t[32][33];
    const int b = blockIdx.z;
    const int c0 = blockIdx.x * 32, f0 = blockIdx.y * 32;
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ff = i >> 5, cc = i & 31;
        const int f = f0 + ff, c = c0 + cc;
        t[ff][cc] = (f < nf && c < nch) ? src[((int64_t)f * nb + b) * rows + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int cc = i >> 5, ff = i & 31;
        const int f = f0 + ff, c = c0 + cc;
        if (f < nf && c < nch) dst[((int64_t)b * nch + c) * nf + f] = t[ff][cc];
    }
}

// ---------------------------------------------------------------- host ----
static int64_t tc_o_pad(const sid_plan* p) { return cdiv(p->N * p->N, 8) * 8; }

int build_spectra_tc(sid_plan* p)
{
    SID_REQUIRE(p->spec_f24, "tensor-core spectra: the plan needs SID_PLAN_SPECTRAL_F24");
    const int64_t n_out = p->N * p->N, n_in_pad = cdiv(p->N * p->N * p->Z, 8) * 8, o_pad = tc_o_pad(p);
    const size_t nent = (size_t)(p->nf * n_in_pad * o_pad);
    SID_TRY(p->khat_f24th.alloc(nent * sizeof(ushort2)));
    SID_TRY(p->khat_f24tl.alloc(nent * sizeof(uchar2)));
    dim3 grid((unsigned)cdiv(n_in_pad, 32), (unsigned)cdiv(o_pad, 32), (unsigned)p->nf);
    k_f24_transpose<<<grid, dim3(32, 8)>>>(p->khat_f24h.as<ushort2>(), p->khat_f24l.as<uchar2>(),
                                           p->khat_f24th.as<ushort2>(), p->khat_f24tl.as<uchar2>(), (int)n_out,
                                           n_in_pad, (int)o_pad);
    SID_CHECK_LAUNCH();
    SID_CUDA_TRY(cudaDeviceSynchronize());
    p->spec_tc = true;
    return SID_OK;
}

constexpr int kTcMaxVolumes = 64;

int spectral_tc_max_volumes() { return kTcMaxVolumes; }

// Device bytes a group of g volumes needs beyond the plan's operator data: the
// solver's polyphase volumes (iterate, Htf, back projection) and images, the
// channel spectra, the B operand planes and the contraction output.
static int64_t tc_group_bytes(const sid_plan* p, int64_t g)
{
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = cdiv(n_in, 8) * 8;
    const int64_t nv = n_out * p->Lx * p->Ly * p->Z, ni = n_out * p->Lx * p->Ly;
    const int64_t bn = g <= 32 ? 64 : 128;
    const int64_t per_vol = (3 * nv + ni) * 4 + (n_in + n_out) * p->nf * 8;
    const int64_t bplanes = 3 * p->nf * bn * 2 * n_in_pad * 2;
    const int64_t out = p->nf * g * n_in_pad * 8;
    return g * per_vol + bplanes + out;
}

// Volumes per tensor-core pass: 64 where the free device memory (plus what
// the plan's workspaces already hold) fits that group with a 10 % margin,
// else 32, 16 or 8.
int spectral_tc_group(const sid_plan* p, int64_t nb)
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return 32;
    }
    int64_t held = 0;
    const sid::DBuf* bufs[] = {&p->ws[0], &p->ws[1], &p->ws[4], &p->ws[5], &p->vhat, &p->ihat, &p->tcb, &p->tco};
    for (const sid::DBuf* b : bufs) held += (int64_t)b->bytes;
    const int64_t avail = (int64_t)fr + held;
    for (int64_t g : {64, 32, 16, 8})
        if (g <= 32 || nb > 32)
            if (tc_group_bytes(p, g) * 11 / 10 <= avail) return (int)g;
    return 8;
}

// A maps: 24-bit planes (high halves as BF16, low bytes) of rows x kp elements
// per frequency; B maps: BN x kpb BF16 per frequency.
static int tc_maps(SpecTcMaps* m, const void* ah, const void* al, const void* bh, const void* bm, const void* bl,
                   int64_t rows, int64_t kp, int64_t kpb, int64_t nf, int bn)
{
    std::memset(m, 0, sizeof(*m));
    const uint64_t da[3] = {(uint64_t)kp, (uint64_t)rows, (uint64_t)nf};
    const uint64_t sa16[2] = {(uint64_t)(kp * 2), (uint64_t)(rows * kp * 2)};
    const uint64_t sa8[2] = {(uint64_t)kp, (uint64_t)(rows * kp)};
    const uint32_t boxa[3] = {TC_BK, TC_BM, 1};
    SID_TRY(encode_tmap_3d(&m->ahi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, ah, da, sa16, boxa, CU_TENSOR_MAP_SWIZZLE_128B));
    SID_TRY(encode_tmap_3d(&m->alo, CU_TENSOR_MAP_DATA_TYPE_UINT8, al, da, sa8, boxa, CU_TENSOR_MAP_SWIZZLE_NONE));
    const uint64_t db[3] = {(uint64_t)kpb, (uint64_t)bn, (uint64_t)nf};
    const uint64_t sb[2] = {(uint64_t)(kpb * 2), (uint64_t)(bn * kpb * 2)};
    const uint32_t boxb[3] = {TC_BK, (uint32_t)bn, 1};
    SID_TRY(encode_tmap_3d(&m->bhi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, bh, db, sb, boxb, CU_TENSOR_MAP_SWIZZLE_128B));
    SID_TRY(encode_tmap_3d(&m->bmi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, bm, db, sb, boxb, CU_TENSOR_MAP_SWIZZLE_128B));
    SID_TRY(encode_tmap_3d(&m->blo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, bl, db, sb, boxb, CU_TENSOR_MAP_SWIZZLE_128B));
    return SID_OK;
}

template <int BN, int STAGES, int NBP>
static int launch_spec_tc(const SpecTcMaps& maps, int rows, int nkb, int akb0, int64_t nf, int nb, float2* out,
                          int* err, cudaStream_t st)
{
    using SM = SpecTcSmem<BN, STAGES, NBP>;
    SID_TRY(smem_attr((const void*)k_spec_tc<BN, STAGES, NBP>, SM::TOTAL));
    const int nmt = (int)cdiv(rows, TC_BM);
    const int64_t nitems = (int64_t)nmt * nf;
    const unsigned grid = (unsigned)std::min<int64_t>(nitems, sm_count());
    k_spec_tc<BN, STAGES, NBP><<<grid, TC_THREADS, SM::TOTAL, st>>>(maps, rows, nkb, akb0, nmt, nitems, nb, out,
                                                                     err);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// stages of the 227 KB of shared memory: three B planes 3 x 64 KB (BN = 64) or
// 2 x 88 KB (BN = 128); two B planes 4 x 56 KB or 3 x 72 KB
static int spec_tc_run(const SpecTcMaps& maps, int bn, int nbp, int rows, int nkb, int akb0, int64_t nf, int nb,
                       float2* out, int* err, cudaStream_t st)
{
    if (nbp == 2)
        return bn == 64 ? launch_spec_tc<64, 4, 2>(maps, rows, nkb, akb0, nf, nb, out, err, st)
                        : launch_spec_tc<128, 3, 2>(maps, rows, nkb, akb0, nf, nb, out, err, st);
    return bn == 64 ? launch_spec_tc<64, 3, 3>(maps, rows, nkb, akb0, nf, nb, out, err, st)
                    : launch_spec_tc<128, 2, 3>(maps, rows, nkb, akb0, nf, nb, out, err, st);
}

int spec_tc_forward_raw(const void* ah, const void* al, int64_t rows, int64_t kp, int akb0, const uint16_t* bplanes,
                        int nbp, int64_t kpb, int64_t nf, int nb, float2* out, int* err, cudaStream_t st)
{
    SID_REQUIRE(nbp == 2 || nbp == 3, "tensor-core projection: B in %d planes", nbp);
    SID_REQUIRE(nb >= 1 && nb <= kTcMaxVolumes, "tensor-core projection: %d volumes outside [1, %d]", nb,
                kTcMaxVolumes);
    SID_REQUIRE(kpb % TC_BK == 0 && akb0 >= 0 && (int64_t)akb0 * TC_BK + kpb <= cdiv(kp, TC_BK) * TC_BK,
                "tensor-core projection: reduction range outside the operator");
    const int bn = nb <= 32 ? 64 : 128;
    const size_t plane = (size_t)(nf * bn * kpb);
    SpecTcMaps maps;
    SID_TRY(tc_maps(&maps, ah, al, bplanes, bplanes + plane, bplanes + (nbp - 1) * plane, rows, kp, kpb, nf, bn));
    return spec_tc_run(maps, bn, nbp, (int)rows, (int)(kpb / TC_BK), akb0, nf, nb, out, err, st);
}

// One contraction: A (rows x kp per frequency), B from nb channel spectra
// src[b][nch][nf], result dst[b][nch_out][nf] (rows >= nch_out).
static int tc_contract(sid_plan* p, bool adj, const float2* src, int nb, int64_t nch, int64_t nch_pad,
                       const void* ah, const void* al, int64_t rows, int64_t nch_out, float2* dst, cudaStream_t st)
{
    SID_REQUIRE(nb >= 1 && nb <= kTcMaxVolumes, "tensor-core projection: %d volumes outside [1, %d]", nb,
                kTcMaxVolumes);
    const int bn = nb <= 32 ? 64 : 128;
    const int64_t kp = 2 * nch_pad, nf = p->nf;
    const size_t plane = (size_t)(nf * bn * kp);  // BF16 elements of one B plane
    SID_TRY(p->tcb.alloc(3 * plane * sizeof(uint16_t)));
    SID_TRY(p->tco.alloc((size_t)(nf * nb * rows) * sizeof(float2)));
    uint16_t* bh = p->tcb.as<uint16_t>();
    uint16_t* bm = bh + plane;
    uint16_t* bl = bm + plane;
    {
        dim3 grid((unsigned)cdiv(nch_pad, 32), (unsigned)cdiv(nf, 32), (unsigned)(bn / 2));
        uint32_t *h = reinterpret_cast<uint32_t*>(bh), *m = reinterpret_cast<uint32_t*>(bm),
                 *l = reinterpret_cast<uint32_t*>(bl);
        if (adj) k_tc_pack<true><<<grid, 256, 0, st>>>(src, nb, (int)nch, (int)nch_pad, (int)nf, bn, h, m, l);
        else k_tc_pack<false><<<grid, 256, 0, st>>>(src, nb, (int)nch, (int)nch_pad, (int)nf, bn, h, m, l);
        SID_CHECK_LAUNCH();
    }
    SpecTcMaps maps;
    SID_TRY(tc_maps(&maps, ah, al, bh, bm, bl, rows, kp, kp, nf, bn));
    const int nkb = (int)cdiv(kp, TC_BK);
    p->timer.begin(st);
    int rc = spec_tc_run(maps, bn, 3, (int)rows, nkb, 0, nf, nb, p->tco.as<float2>(), p->errflag.as<int>(), st);
    p->timer.finish(st);
    SID_TRY(rc);
    return spec_tc_unpack(p->tco.as<float2>(), nb, (int)rows, (int)nch_out, nf, dst, st);
}

int spec_tc_unpack(const float2* src, int nb, int rows, int nch, int64_t nf, float2* dst, cudaStream_t st)
{
    dim3 grid((unsigned)cdiv(nch, 32), (unsigned)cdiv(nf, 32), (unsigned)nb);
    k_tc_unpack<<<grid, 256, 0, st>>>(src, nb, rows, nch, (int)nf, dst);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_forward_tc(sid_plan* p, const float* vp, float* ip, int nb, cudaStream_t st)
{
    SID_REQUIRE(p->spec_tc, "tensor-core projection: the plan was built without SID_PLAN_SPECTRAL_TC");
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = cdiv(n_in, 8) * 8;
    SID_TRY(p->vhat.alloc((size_t)(nb * n_in * p->nf) * sizeof(float2)));
    SID_TRY(p->ihat.alloc((size_t)(nb * n_out * p->nf) * sizeof(float2)));
    SID_TRY(spec_r2c(p, vp, p->vhat.as<float2>(), nb * n_in, st));
    SID_TRY(tc_contract(p, false, p->vhat.as<float2>(), nb, n_in, n_in_pad, p->khat_f24h.p, p->khat_f24l.p, n_out,
                        n_out, p->ihat.as<float2>(), st));
    return spec_c2r(p, p->ihat.as<float2>(), ip, nb * n_out, st);
}

int spectral_adjoint_tc(sid_plan* p, const float* ip, float* bp, int nb, cudaStream_t st)
{
    SID_REQUIRE(p->spec_tc, "tensor-core projection: the plan was built without SID_PLAN_SPECTRAL_TC");
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = cdiv(n_in, 8) * 8;
    SID_TRY(p->vhat.alloc((size_t)(nb * n_in * p->nf) * sizeof(float2)));
    SID_TRY(p->ihat.alloc((size_t)(nb * n_out * p->nf) * sizeof(float2)));
    SID_TRY(spec_r2c(p, ip, p->ihat.as<float2>(), nb * n_out, st));
    SID_TRY(tc_contract(p, true, p->ihat.as<float2>(), nb, n_out, tc_o_pad(p), p->khat_f24th.p, p->khat_f24tl.p,
                        n_in_pad, n_in, p->vhat.as<float2>(), st));
    return spec_c2r(p, p->vhat.as<float2>(), bp, nb * n_in, st);
}

}  // namespace sid
