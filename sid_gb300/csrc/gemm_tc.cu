// gemm_tc.cu -- tcgen05 tensor-core GEMM for the NNLS Gram and cross products.
//
//   C (m x n, column-major, ldc) = sum_{p < npass} A_p^T B_p
//   A_p (k x m) and B_p (k x n): 16-bit operands, both BF16 or both FP16, in
//   the K-BLOCKED layout [k/64][row][64] (element (kk, r) at
//   ((kk/64)*rows + r)*64 + kk%64), zero-padded to whole 64-element blocks;
//   FP32 accumulation.
// The blocked layout makes every 64 x BN TMA box one contiguous run of memory:
// with a plain column-major operand the rows of a box are a whole column apart
// (2 MB for a 1M-pixel movie), so each box touched BN pages and the GEMM ran
// at a third of its speed on full-size problems.
// This is the "TN" form every contraction of the path takes: S'S and S'Y with
// the library and the movie stored pixel-major (LS_nnls.m:76,82,
// fast_nnls.m:54-57, T_update.m:24-25), and G*x in the NNLS iterations.
// Passing (hi, lo) splits of FP32 operands as extra passes gives the split
// precision products (hi*hi + hi*lo + lo*hi) with FP32 accumulation in TMEM.
//
// Kernel: one 128 x BN output tile per CTA (optionally a K range of it, for
// split-K), 10 warps.  One thread drives a STAGES-deep TMA ring (128B-swizzled
// 64-element K blocks, completion on "full" mbarriers); one thread issues
// tcgen05.mma (cta_group::1, M=128, N=BN, K=16 per instruction) into one of two
// TMEM accumulators and releases each stage through tcgen05.commit on its
// "empty" mbarrier; eight warps read finished accumulators back with tcgen05.ld
// and sum them in registers, writing the tile once.
// Every mbarrier wait is bounded (ptx.cuh); on a timeout the CTA records the
// error, stops issuing, waits (bounded) for issued MMAs, frees TMEM and exits.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ptx.cuh"
#include "sid_internal.cuh"
#include "tc.cuh"

namespace sid {

constexpr int GEMM_BM = 128;
constexpr int GEMM_BK = 64;  // 64 x 16-bit = 128 bytes: one swizzle row
constexpr int GEMM_MAXPASS = 3;
constexpr int kErrTimeoutGemm = 2;

struct GemmMaps {
    CUtensorMap a[GEMM_MAXPASS];
    CUtensorMap b[GEMM_MAXPASS];
};

__device__ __forceinline__ uint32_t instr_desc(int n, bool bf16) { return instr_desc_m(GEMM_BM, n, bf16); }

template <int BN, int STAGES>
struct GemmSmem {
    static constexpr int A_BYTES = GEMM_BM * GEMM_BK * 2;  // 16 KB
    static constexpr int B_BYTES = BN * GEMM_BK * 2;
    static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /* alignment slack */;
};

// grid: (ceil(m/128), ceil(n/BN), splitk).  out + z*split_stride receives the
// partial sum of K blocks [z*kb_per, (z+1)*kb_per) of every pass.
//
// Warp roles (320 threads): warps 0-7 drain the accumulator -- warp w reads
// TMEM lanes 32*(w%4)..+31 (tile rows) and columns [(w/4)*BN/2, (w/4+1)*BN/2)
// -- warp 8 lane 0 is the TMA producer, warp 9 lane 0 issues the MMAs.  The
// tensor-core FP32 accumulator does not round to nearest, so long K chains
// drift (a 70000-deep chain lost 9e-5): the K range is cut into chunks of
// GEMM_KCHUNK blocks, each accumulated in one of two TMEM buffers while the
// previous chunk is drained and added, round-to-nearest, into registers; the
// tile is written once at the end.
constexpr int GEMM_KCHUNK = 16;  // 16 x 64 = 1024 reduction elements per chain
constexpr int GEMM_DRAIN_WARPS = 8;
constexpr int GEMM_THREADS = (GEMM_DRAIN_WARPS + 2) * 32;

template <int BN, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
k_gemm_tc(const __grid_constant__ GemmMaps maps, int npass, int m, int n, int nkb, int kb_per, int bf16,
          float* __restrict__ out, int64_t ldc, int64_t split_stride, float alpha, int* __restrict__ err, int sym,
          const float* __restrict__ dalpha)
{
    // symmetric product (A'A): tiles wholly below the diagonal are mirrored afterwards
    if (sym && (int)blockIdx.x * GEMM_BM >= (int)blockIdx.y * BN + BN) return;
    using SM = GemmSmem<BN, STAGES>;
    constexpr uint32_t ACC_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;  // two accumulators
    constexpr int HALF = BN / 2;                  // columns per drain thread
    static_assert(HALF % 32 == 0, "BN must be a multiple of 64");
    extern __shared__ uint8_t gsm_raw[];
    uint8_t* gsm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(gsm_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], tfull[2], tempty[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * GEMM_BM, n0 = blockIdx.y * BN;
    const int kb0 = blockIdx.z * kb_per;
    const int kb1 = min(nkb, kb0 + kb_per);
    const int nloc = kb1 > kb0 ? (kb1 - kb0) : 0;
    const int nchunk = (nloc + GEMM_KCHUNK - 1) / GEMM_KCHUNK;
    constexpr int PRODUCER = GEMM_DRAIN_WARPS, ISSUER = GEMM_DRAIN_WARPS + 1;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], GEMM_DRAIN_WARPS * 32);
        }
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
    float* dst = out + (int64_t)blockIdx.z * split_stride;

    if (warp == PRODUCER) {
        if (lane == 0) {
            // TMA producer: chunk -> pass -> k block
            int it = 0;
            for (int c = 0; c < nchunk && !abort_flag; ++c) {
                const int cb0 = kb0 + c * GEMM_KCHUNK, cb1 = min(kb1, cb0 + GEMM_KCHUNK);
                for (int pass = 0; pass < npass; ++pass) {
                    for (int kb = cb0; kb < cb1; ++kb, ++it) {
                        const int s = it % STAGES;
                        if (it >= STAGES && !mbar_wait(&empty[s], (uint32_t)(((it / STAGES) - 1) & 1), err)) {
                            atomicExch(&abort_flag, 1);
                            break;
                        }
                        if (*(volatile int*)&abort_flag) break;
                        uint8_t* sa = gsm + s * SM::STAGE_BYTES;
                        uint8_t* sb = sa + SM::A_BYTES;
                        mbar_arrive_expect_tx(&full[s], SM::STAGE_BYTES);
                        tma_load_3d(sa, &maps.a[pass], 0, m0, kb, &full[s]);
                        tma_load_3d(sb, &maps.b[pass], 0, n0, kb, &full[s]);
                    }
                    if (*(volatile int*)&abort_flag) break;
                }
            }
        }
    } else if (warp == ISSUER) {
        if (lane == 0) {
            // MMA issuer: chunk c accumulates into TMEM buffer c & 1
            const uint32_t idesc = instr_desc(BN, bf16 != 0);
            int it = 0;
            bool ok = true;
            for (int c = 0; c < nchunk && ok; ++c) {
                const int b = c & 1;
                if (c >= 2 && !mbar_wait(&tempty[b], (uint32_t)(((c >> 1) - 1) & 1), err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
                const int cb0 = kb0 + c * GEMM_KCHUNK, cb1 = min(kb1, cb0 + GEMM_KCHUNK);
                bool first = true;
                for (int pass = 0; pass < npass && ok; ++pass) {
                    for (int kb = cb0; kb < cb1; ++kb, ++it) {
                        const int s = it % STAGES;
                        if (!mbar_wait(&full[s], (uint32_t)((it / STAGES) & 1), err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t sa = smem_u32(gsm + s * SM::STAGE_BYTES);
                        const uint32_t sb = sa + SM::A_BYTES;
#pragma unroll
                        for (int kk = 0; kk < GEMM_BK / 16; ++kk) {
                            // advance 16 elements = 32 bytes inside the 128-byte swizzle row
                            mma_bf16(acc, smem_desc_sw128(sa + kk * 32), smem_desc_sw128(sb + kk * 32), idesc,
                                     first ? 0 : 1);
                            first = false;
                        }
                        mma_commit(&empty[s]);
                    }
                }
                mma_commit(&tfull[b]);  // arrives when this chunk's MMAs have completed
            }
            if (!ok) atomicExch(&abort_flag, 1);
        }
    } else {
        // drain warps: add each finished chunk into registers
        const int lg = warp & 3;           // TMEM lane group = tile rows 32*lg..
        const int ch0 = (warp >> 2) * HALF;  // first column of this warp
        const int row = m0 + lg * 32 + lane;
        float accr[HALF];
#pragma unroll
        for (int j = 0; j < HALF; ++j) accr[j] = 0.f;
        bool ok = true;
        for (int c = 0; c < nchunk; ++c) {
            const int b = c & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(&tfull[b], (uint32_t)((c >> 1) & 1), err));
            if (!ok) break;
            tc_fence_after();
#pragma unroll
            for (int c0 = 0; c0 < HALF; c0 += 32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * ACC_COLS + ch0 + c0), v);
#pragma unroll
                for (int j = 0; j < 32; ++j) accr[c0 + j] += v[j];
            }
            tc_fence_before();
            mbar_arrive(&tempty[b]);
        }
        if (ok && row < m) {
            const float al = dalpha ? alpha * *dalpha : alpha;
#pragma unroll
            for (int j = 0; j < HALF; ++j) {
                const int col = n0 + ch0 + j;
                if (col < n) dst[(int64_t)row + ldc * col] = accr[j] * al;
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TMEM_COLS) : "memory");
    }
    if (threadIdx.x == 0 && abort_flag && err) atomicExch(err, kErrTimeoutGemm);
}

// Sum split-K partials: C = alpha * sum_z P[z] + beta * C (beta == 0 ignores C).
__global__ void k_splitk_reduce(const float* __restrict__ part, int nsplit, int64_t split_stride, int m, int n,
                                int64_t ldp, float* __restrict__ C, int64_t ldc, float alpha, float beta,
                                const float* __restrict__ dalpha)
{
    if (dalpha) alpha *= *dalpha;
    const int64_t total = (int64_t)m * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % m);
        const int64_t c = i / m;
        float s = 0.f;
        for (int z = 0; z < nsplit; ++z) s += part[z * split_stride + r + ldp * c];
        float* d = C + r + ldc * c;
        *d = (beta != 0.f) ? alpha * s + beta * *d : alpha * s;
    }
}

// ----------------------------------------------------------- host side ----
int encode_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, const void* base, const uint64_t dims[3],
                   const uint64_t strides[2], const uint32_t box[3], CUtensorMapSwizzle swizzle)
{
    SID_REQUIRE(((uintptr_t)base & 15) == 0, "tensor map: base address not 16-byte aligned");
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return SID_ECUDA;
        }
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    cuuint64_t d[3] = {dims[0], dims[1], dims[2]};
    cuuint64_t str[2] = {strides[0], strides[1]};
    cuuint32_t bx[3] = {box[0], box[1], box[2]};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode(map, dtype, 3, const_cast<void*>(base), d, str, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
        return SID_ECUDA;
    }
    return SID_OK;
}

static int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t nkb, int box_rows, bool bf16)
{
    // K-blocked operand: dims {64, rows, nkb}, byte strides {128, rows*128}
    const uint64_t dims[3] = {(uint64_t)GEMM_BK, (uint64_t)rows, (uint64_t)nkb};
    const uint64_t strides[2] = {(uint64_t)(GEMM_BK * 2), (uint64_t)(rows * GEMM_BK * 2)};
    const uint32_t box[3] = {GEMM_BK, (uint32_t)box_rows, 1};
    return encode_tmap_3d(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, base, dims,
                          strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
}

template <int BN, int STAGES>
static int launch_gemm(const GemmMaps& maps, int npass, int m, int n, int nkb, int splitk, bool bf16, float* out,
                       int64_t ldc, int64_t split_stride, float alpha, const float* dalpha, int* err, bool sym,
                       cudaStream_t st)
{
    using SM = GemmSmem<BN, STAGES>;
    SID_TRY(smem_attr((const void*)k_gemm_tc<BN, STAGES>, SM::TOTAL));
    const int kb_per = (int)cdiv(nkb, splitk);
    dim3 grid((unsigned)cdiv(m, GEMM_BM), (unsigned)cdiv(n, BN), (unsigned)splitk);
    k_gemm_tc<BN, STAGES><<<grid, GEMM_THREADS, SM::TOTAL, st>>>(maps, npass, m, n, nkb, kb_per, bf16 ? 1 : 0, out, ldc,
                                                         split_stride, alpha, err, sym ? 1 : 0, dalpha);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Output tiles a launch computes: all of them, or for a symmetric product
// (A'A, m == n) those reaching the diagonal or above it.
static int64_t gemm_tiles(int m, int n, int bn, bool sym)
{
    const int64_t tm = cdiv(m, GEMM_BM), tn = cdiv(n, bn);
    if (!sym) return tm * tn;
    int64_t t = 0;
    for (int64_t j = 0; j < tn; ++j) t += std::min<int64_t>(tm, cdiv(j * bn + bn, GEMM_BM));
    return t;
}

// Tile width and split-K choice (the project's autotuner for this kernel).
// For each tile width BN in {256, 192, 128, 64} and each split of K into s
// parts of >= 8 K blocks (s <= 64), estimate the time in units of one 64-deep
// K block of one 128 x 256 tile (~0.75 us for three passes) as
//   waves x (K blocks per CTA x BN / efficiency(BN) + 1024)    (+ s m n / 4096 if s > 1)
// with waves = ceil(tiles x s / SMs), 1024 the fixed cost of a CTA (TMEM
// allocation, pipeline fill, the drain of its tile; ~3 us) and the last term
// the split-K sum's traffic, and keep the fastest: the split that fills the
// last wave best, not merely the first that gives four waves.  The
// efficiencies model tcgen05's shared-memory operand traffic per MMA:
// A (128 x 16) plus B (BN x 16) must be read for 128*BN*16 MACs, so BN = 64
// is limited by shared-memory bandwidth (measured) and BN = 256 amortises A
// best.  A symmetric product counts only the tiles it computes (the 800-wide
// Gram: 19 tiles of 256 columns hold 1.95x the triangle's outputs, 28 of 128
// columns 1.43x).
static void gemm_autotune_sms(int m, int n, int nkb, bool sym, int sms, int* bn, int* splitk)
{
    const int cands[4] = {256, 192, 128, 64};
    // measured on the 800-wide Gram at P = 1,010,025 (of the MMA work each width computes):
    // 256 at 99 % of the BF16 peak, 192 at 77 %, 128 at 53 %
    const double eff[4] = {1.0, 0.78, 0.55, 0.45};
    double best = 1e300;
    int bbn = 256, bs = 1;
    for (int i = 0; i < 4; ++i) {
        const int c = cands[i];
        const int64_t tiles = gemm_tiles(m, n, c, sym);
        for (int s0 = 1; s0 <= 64; ++s0) {
            if (s0 > 1 && nkb / s0 < 8) break;
            const int64_t kb_per = cdiv(nkb, s0);
            const int s = (int)cdiv(nkb, kb_per);
            const int64_t waves = cdiv(tiles * s, sms);
            const double t = (double)waves * ((double)kb_per * (double)c / eff[i] + 1024.0) +
                             (s > 1 ? (double)s * (double)m * (double)n / 4096.0 : 0.0);
            if (t < best * (1.0 - 1e-9)) {
                best = t;
                bbn = c;
                bs = s;
            }
        }
    }
    *bn = bbn;
    *splitk = bs;
}

static void gemm_autotune_impl(int m, int n, int nkb, bool sym, int* bn, int* splitk)
{
    gemm_autotune_sms(m, n, nkb, sym, sm_count(), bn, splitk);
}

void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk) { gemm_autotune_impl(m, n, nkb, false, bn, splitk); }
void gemm_autotune_sym(int m, int nkb, int* bn, int* splitk) { gemm_autotune_impl(m, m, nkb, true, bn, splitk); }

// C(r, c) = C(c, r) for r > c: completes a symmetric product computed on and above the diagonal
__global__ void k_mirror_lower(float* __restrict__ C, int m, int64_t ldc)
{
    const int64_t total = (int64_t)m * m;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % m), c = (int)(i / m);
        if (r > c) C[r + ldc * c] = C[c + ldc * r];
    }
}

// out (m x n, ldc) = sum_p A_p^T B_p; A_p: k x m, B_p: k x n, 16-bit K-blocked.
// ws: >= splitk * m * n floats when splitk > 1 or beta != 0 (alpha alone is
// applied as the tiles are stored).
static int gemm_tn_impl(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k,
                        bool bf16, float* C, int64_t ldc, float alpha, const float* dalpha, float beta, int bn,
                        int splitk, float* ws, int64_t ws_elems, int* err, bool sym, cudaStream_t st)
{
    SID_REQUIRE(npass >= 1 && npass <= GEMM_MAXPASS, "gemm: npass %d outside [1,3]", npass);
    SID_REQUIRE(m > 0 && n > 0 && k > 0, "gemm: empty problem");
    SID_REQUIRE(!sym || m == n, "gemm: a symmetric product needs m == n");
    const int nkb = (int)cdiv(k, GEMM_BK);
    if (bn <= 0 || splitk <= 0) gemm_autotune_impl((int)m, (int)n, nkb, sym, &bn, &splitk);
    splitk = std::max(1, std::min(splitk, nkb));
    GemmMaps maps;
    std::memset(&maps, 0, sizeof(maps));
    for (int p = 0; p < npass; ++p) {
        SID_TRY(make_map(&maps.a[p], A[p], m, nkb, GEMM_BM, bf16));
        SID_TRY(make_map(&maps.b[p], B[p], n, nkb, bn, bf16));
    }
    const bool direct = (splitk == 1 && beta == 0.f);
    float* out = C;
    int64_t ldo = ldc, sstride = 0;
    if (!direct) {
        ldo = m;
        sstride = m * n;
        SID_REQUIRE(ws && ws_elems >= splitk * sstride, "gemm: split-K workspace too small");
        out = ws;
    }
    int rc;
    switch (bn) {
    case 256: rc = launch_gemm<256, 4>(maps, npass, (int)m, (int)n, nkb, splitk, bf16, out, ldo, sstride, direct ? alpha : 1.f, direct ? dalpha : nullptr, err, sym, st); break;
    case 192: rc = launch_gemm<192, 5>(maps, npass, (int)m, (int)n, nkb, splitk, bf16, out, ldo, sstride, direct ? alpha : 1.f, direct ? dalpha : nullptr, err, sym, st); break;
    case 128: rc = launch_gemm<128, 6>(maps, npass, (int)m, (int)n, nkb, splitk, bf16, out, ldo, sstride, direct ? alpha : 1.f, direct ? dalpha : nullptr, err, sym, st); break;
    case 64: rc = launch_gemm<64, 8>(maps, npass, (int)m, (int)n, nkb, splitk, bf16, out, ldo, sstride, direct ? alpha : 1.f, direct ? dalpha : nullptr, err, sym, st); break;
    default: set_error("gemm: unsupported tile width %d", bn); return SID_EINVAL;
    }
    SID_TRY(rc);
    if (!direct) {
        k_splitk_reduce<<<1024, 256, 0, st>>>(ws, splitk, sstride, (int)m, (int)n, m, C, ldc, alpha, beta, dalpha);
        SID_CHECK_LAUNCH();
    }
    if (sym) {
        k_mirror_lower<<<1024, 256, 0, st>>>(C, (int)m, ldc);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
            float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws, int64_t ws_elems, int* err,
            cudaStream_t st)
{
    return gemm_tn_impl(A, B, npass, m, n, k, bf16, C, ldc, alpha, nullptr, beta, bn, splitk, ws, ws_elems, err, false,
                        st);
}

int gemm_tn_ds(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
               float* C, int64_t ldc, float alpha, const float* dalpha, float beta, int bn, int splitk, float* ws,
               int64_t ws_elems, int* err, cudaStream_t st)
{
    return gemm_tn_impl(A, B, npass, m, n, k, bf16, C, ldc, alpha, dalpha, beta, bn, splitk, ws, ws_elems, err, false,
                        st);
}

// Symmetric product C = sum_p A_p^T B_p with A_p^T B_p + A_q^T B_q symmetric
// over the passes (A'A, or the split hi/lo passes of A'A): only the tiles on
// and above the diagonal are computed, the rest mirrored (an exactly symmetric
// result).  beta must be 0.
int gemm_tn_sym(const void* const* A, const void* const* B, int npass, int64_t m, int64_t k, bool bf16, float* C,
                int64_t ldc, float alpha, int bn, int splitk, float* ws, int64_t ws_elems, int* err, cudaStream_t st)
{
    return gemm_tn_impl(A, B, npass, m, m, k, bf16, C, ldc, alpha, nullptr, 0.f, bn, splitk, ws, ws_elems, err, true,
                        st);
}

}  // namespace sid

extern "C" int sid_gemm_tile_plan(int64_t m, int64_t n, int64_t k, int symmetric, int sms, int* bn, int* splitk)
{
    SID_REQUIRE(bn && splitk, "sid_gemm_tile_plan: NULL output");
    SID_REQUIRE(m > 0 && n > 0 && k > 0 && sms > 0 && m <= INT32_MAX && n <= INT32_MAX,
                "sid_gemm_tile_plan: bad sizes");
    SID_REQUIRE(!symmetric || m == n, "sid_gemm_tile_plan: a symmetric product needs m == n");
    sid::gemm_autotune_sms((int)m, (int)n, (int)sid::cdiv(k, sid::GEMM_BK), symmetric != 0, sms, bn, splitk);
    return SID_OK;
}
