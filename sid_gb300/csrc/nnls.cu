// nnls.cu -- batched multi-right-hand-side NNLS (LS_nnls.m, fast_nnls.m).
//
// All F columns iterate in lock step on the GPU.  Both solvers are projected
// gradient with an exact line search; one iteration is
//   mask:   passive = (x > 0) | (df < 0), d = df .* passive, s1 = sum d^2
//   G d     (contraction: tcgen05 split precision, or FP32 SIMT)
//   step:   alpha = s1 / sum(d .* G d), x_new = max(x - alpha d, 0),
//           step = x_new - x, convergence statistic of the step, and
//           G step = -alpha (G d) + G (clamp corrections), formed in place
//           from the contraction's G d (the clamps touch few entries); the
//           next iteration's mask kernel applies df = df + G step before it
//           reads df.  (With use_std a second contraction forms G step.)
//   retire: the reference's log-linear extrapolation test
// The iterate x and the gradient df are double-float (about 44 significant
// bits, FP32 arithmetic) and the gradient is updated incrementally
// (fast_nnls.m:153 does exactly this; LS_nnls.m:119 recomputes df = -h + G x,
// which is the same quantity): the contraction's rounding then shrinks with
// the steps, so the step statistics keep falling as they do in the
// reference's FP64 arithmetic and its convergence test can fire.  With a
// gradient recomputed from a 16- or 32-bit product every iteration the steps
// stall at the product's noise floor and no column ever retires early.
// What the incremental gradient does carry is the drift of every increment's
// rounding, so the increments are formed close to FP32 accuracy: on the tensor
// cores the Gram (|G| <= 1 after normalisation, scaled by 2^14) and each
// column of d (scaled by its own power of two 2^e_j, found by the mask kernel)
// enter as FP16 hi/lo pairs (22 significant bits each; hi*hi + hi*lo + lo*hi
// with FP32 accumulation), and the step kernel multiplies G d by 2^-e_j.
// BF16 hi/lo pairs (16 bits) let the gradient drift by about 1e-5 of |x|,
// enough to move converged columns visibly away from the FP64 result.
//
// Every kernel reads the iteration number from device memory, so a chunk of
// iterations is captured once in a CUDA graph and replayed.  A retired column
// is frozen (never written again), which is what removing it from x does in
// the reference (LS_nnls.m:158-168, fast_nnls.m:165-179).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "sid_internal.cuh"

namespace sid {
int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st);
int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
            float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws, int64_t ws_elems, int* err,
            cudaStream_t st);
void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk);
int sgemm_tn(const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, float* C,
             int64_t ldc, float alpha, float beta, float* ws, int64_t ws_elems, cudaStream_t st);
int64_t sgemm_ws_elems(int64_t m, int64_t n, int64_t k);
int split16(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
            float scale, cudaStream_t st);
int64_t blk16_elems(int64_t k, int64_t rows);
int ctx_sync(sid_ctx* c, cudaStream_t st);
int absmax(const float* x, int64_t n, unsigned int* out, cudaStream_t st);

struct NnlsCounters {
    int iter;    // LS_nnls: iteration number; fast_nnls: the reference's s
    int active;  // columns still iterating
    int first;   // index of the first active column (LS_nnls k(1) rule)
    int pad;
};

enum { SOLVER_LS = 0, SOLVER_FAST = 1 };

// Double-float numbers: value = hi + lo with |lo| <= ulp(hi)/2 (about 44
// significant bits), updated with error-free FP32 transformations (TwoSum,
// then a Fast2Sum renormalisation).  The NNLS iterate and gradient need more
// than FP32 (the reference's log-linear retirement test resolves steps far
// below FP32 resolution of the gradient), and GB300's FP64 pipe runs at a
// small fraction of its FP32 rate.
__device__ __forceinline__ float2 dd_add(float2 a, float b)
{
    const float s = a.x + b;
    const float bb = s - a.x;
    const float e = ((a.x - (s - bb)) + (b - bb)) + a.y;
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
__device__ __forceinline__ float2 dd_from(double v)
{
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}
__device__ __forceinline__ double dd_to(float2 a) { return (double)a.x + (double)a.y; }

struct ColBufs {
    float2 *x, *df;      // K x F double-float iterate and gradient
    float* v;            // K x F FP32 operand of the next contraction (SIMT path)
    uint16_t *vhi, *vlo; // K x F BF16 split operand, K-blocked (tensor-core path)
    float* g;            // K x F contraction result
    double* test;        // sample x F window of step statistics
    float2* s1;          // per column: sum d.^2, plain and scaled by 2^100
    double* fit;         // 3 x F window-fit results
    float *anyp, *xmax;  // per column: passive count, max x
    double* xi;          // 2 x sample fit matrix
    float *u, *gu;       // use_std: column-sum vector and G * it
    const float* Gf;     // K x K FP32 (normalised) Gram: the clamp corrections of G * step
    int sparse;          // G * step formed in the step kernel (no second contraction)
    int f16s;            // tensor-core operand as FP16 hi/lo of d * 2^e_j (per-column power of two)
    float* dsc;          // per column: 2^-e_j, applied to the contraction result
    int* active;
    NnlsCounters* cnt;
    int F;
};

// write the next contraction operand: FP32 copy or BF16 hi/lo split
__device__ __forceinline__ void put_operand(const ColBufs& b, int64_t o, int j, int k, float val)
{
    if (b.vhi) {
        // K-blocked layout of the tensor-core GEMM: ((k/64)*F + j)*64 + k%64
        const int64_t i = (((int64_t)(k >> 6) * b.F + j) << 6) + (k & 63);
        const float f = val;
        const __nv_bfloat16 h = __float2bfloat16_rn(f);
        b.vhi[i] = __bfloat16_as_ushort(h);
        b.vlo[i] = __bfloat16_as_ushort(__float2bfloat16_rn(f - __bfloat162float(h)));
    } else {
        b.v[o + k] = val;
    }
}

// FP16 hi/lo of v (|v| <= 2^14, a scaled operand), K-blocked like put_operand
__device__ __forceinline__ void put_operand_f16(const ColBufs& b, int j, int k, float v)
{
    const int64_t i = (((int64_t)(k >> 6) * b.F + j) << 6) + (k & 63);
    const __half h = __float2half_rn(v);
    b.vhi[i] = __half_as_ushort(h);
    b.vlo[i] = __half_as_ushort(__float2half_rn(v - __half2float(h)));
}

// (pow2_for, sid_internal.cuh: FP16 hi/lo of values scaled into [2^13, 2^14)
// keep 22 significant bits of each entry relative to its column's largest, in
// FP16's normal range.)

// Reductions on the FP32 and integer pipes.  A sum is carried as an
// unevaluated pair hi + lo (an error-free two-sum at every addition), so the
// partials add up as accurately as an FP64 sum would.  The column kernels issue
// no FP64 instruction at all: GB300's FP64 rate is about 1/64 of its FP32
// rate, an FP64 warp instruction holds its SM sub-partition for tens of cycles
// whatever number of lanes it has active, and a few of them per warp cost as
// much as the column pass itself.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    const float l = (a.y + b.y) + e;
    const float hi = s + l;
    return make_float2(hi, l - (hi - s));
}

__device__ __forceinline__ float2 warp_sum_ff(float v)
{
    float2 a = make_float2(v, 0.f);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, a.x, off), __shfl_xor_sync(0xffffffffu, a.y, off));
        a = ff_add(a, o);
    }
    return a;
}

__device__ __forceinline__ float warp_max_f(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// Column kernels: four warps per frame column (two columns per 256-thread
// CTA), lanes stride over the K components; warp-shuffle reductions, then one
// shared-memory exchange across the column's warps.  Inactive columns skip
// the work but still reach the barriers.
constexpr int kWarpsPerCol = 4;
constexpr int kColsPerCta = 2;
constexpr int kColThreads = 32 * kWarpsPerCol;

struct ColIdx {
    int cl, wc, lane, j;
};

__device__ __forceinline__ ColIdx col_idx()
{
    ColIdx c;
    c.cl = threadIdx.x / kColThreads;
    c.wc = (threadIdx.x >> 5) % kWarpsPerCol;
    c.lane = threadIdx.x & 31;
    c.j = blockIdx.x * kColsPerCta + c.cl;
    return c;
}

// Column sums of products for the line search, s1 = sum d.^2 and
// den = sum d .* (G d) (LS_nnls.m:122, fast_nnls.m:119).  A converging column's
// masked gradient shrinks geometrically, and below |d| ~ 1e-19 its FP32
// products underflow: den reaches 0 while s1 is still a denormal, which would
// make alpha infinite.  Each thread therefore keeps a second partial of the same
// products with both factors scaled by 2^50 (exact).  alpha is the ratio of
// the two scaled sums when both are finite (they overflow only for products
// above ~1e8, where the plain sums are exact to FP32 rounding), else of the
// two plain sums.
constexpr float kWideUp = 0x1p50f;

__device__ __forceinline__ void wide_fma(float a, float b, float& plain, float& wide)
{
    plain = fmaf(a, b, plain);
    wide = fmaf(a * kWideUp, b * kWideUp, wide);
}

// num, den: {plain, scaled} column sums
__device__ __forceinline__ float wide_ratio(float2 num, float2 den)
{
    return (isfinite(num.y) && isfinite(den.y)) ? num.y / den.y : num.x / den.x;
}

// The pending gradient update df += G step of the previous iteration
// (fast_nnls.m:153; the incremental form of LS_nnls.m:119), then the passive
// set and masked gradient (LS_nnls.m:120-121, fast_nnls.m:100,163).  g holds
// G step (zero before the first iteration).
// (inc_iter: the first thread also advances the iteration counter, which no
// thread of this kernel reads and the step kernel after it does.)  ROWS > 0:
// every row of the column is one of this thread's ROWS register rows (K <=
// ROWS * kColThreads), loaded together before any is used (more loads in
// flight), and the masked gradient stays in registers for the FP16 operand
// pass; ROWS = 0: any K, rows streamed.
template <int ROWS>
__global__ void __launch_bounds__(256) k_nn_mask(ColBufs b, int K, int F, int use_std, int inc_iter)
{
    if (inc_iter && blockIdx.x == 0 && threadIdx.x == 0) b.cnt->iter += 1;
    __shared__ float2 red[kColsPerCta][kWarpsPerCol][2];
    __shared__ float redm[kColsPerCta][kWarpsPerCol];
    __shared__ int redn[kColsPerCta][kWarpsPerCol];
    __shared__ float reda[kColsPerCta][kWarpsPerCol];
    const ColIdx c = col_idx();
    const bool act = c.j < F && b.active[c.j];
    float acc_f = 0.f, accw_f = 0.f, mx_f = -INFINITY, am_f = 0.f;
    int np_i = 0;
    constexpr int RR = ROWS > 0 ? ROWS : 1;
    float dmr[RR];
    // one row: pending gradient update, passive set, operand, statistics
    auto row = [&](int64_t o, int k, float g, float2 xv, float2 dold) -> float {
        if (use_std) g -= b.gu[k];
        const float2 dv = dd_add(dold, g);
        b.df[o + k] = dv;
        const bool p = xv.x > 0.f || dv.x < 0.f;
        const float dm = p ? dv.x + dv.y : 0.f;
        if (b.f16s) am_f = fmaxf(am_f, fabsf(dm));
        else put_operand(b, o, c.j, k, dm);
        wide_fma(dm, dm, acc_f, accw_f);
        np_i += p ? 1 : 0;
        mx_f = fmaxf(mx_f, xv.x);
        return dm;
    };
    if (act) {
        const int64_t o = (int64_t)c.j * K;
        if (ROWS > 0) {
            float gv[RR];
            float2 xr[RR], dr[RR];
#pragma unroll
            for (int t = 0; t < RR; ++t) {
                const int k = c.wc * 32 + c.lane + t * kColThreads;
                if (k < K) {
                    gv[t] = b.g[o + k];
                    xr[t] = b.x[o + k];
                    dr[t] = b.df[o + k];
                }
            }
#pragma unroll
            for (int t = 0; t < RR; ++t) {
                const int k = c.wc * 32 + c.lane + t * kColThreads;
                dmr[t] = k < K ? row(o, k, gv[t], xr[t], dr[t]) : 0.f;
            }
        } else {
#pragma unroll 2
            for (int k = c.wc * 32 + c.lane; k < K; k += kColThreads) row(o, k, b.g[o + k], b.x[o + k], b.df[o + k]);
        }
    }
    const float2 acc = warp_sum_ff(acc_f);
    const float2 accw = warp_sum_ff(accw_f);
    const int np = __reduce_add_sync(0xffffffffu, np_i);
    const float mx = warp_max_f(mx_f);
    const float am = warp_max_f(am_f);
    if (c.lane == 0) {
        red[c.cl][c.wc][0] = acc;
        red[c.cl][c.wc][1] = accw;
        redn[c.cl][c.wc] = np;
        redm[c.cl][c.wc] = mx;
        reda[c.cl][c.wc] = am;
    }
    __syncthreads();
    if (b.f16s && act) {
        // second pass: the scaled FP16 hi/lo operand (d read back from the updated df)
        float amax = reda[c.cl][0];
        for (int w = 1; w < kWarpsPerCol; ++w) amax = fmaxf(amax, reda[c.cl][w]);
        const float sc = pow2_for(amax);
        if (ROWS > 0) {
#pragma unroll
            for (int t = 0; t < RR; ++t) {
                const int k = c.wc * 32 + c.lane + t * kColThreads;
                if (k < K) put_operand_f16(b, c.j, k, dmr[t] * sc);
            }
        } else {
            const int64_t o = (int64_t)c.j * K;
            for (int k = c.wc * 32 + c.lane; k < K; k += kColThreads) {
                const float2 xv = b.x[o + k], dv = b.df[o + k];
                const float dm = (xv.x > 0.f || dv.x < 0.f) ? dv.x + dv.y : 0.f;
                put_operand_f16(b, c.j, k, dm * sc);
            }
        }
        if (c.wc == 0 && c.lane == 0) b.dsc[c.j] = 1.f / sc;
    }
    if (act && c.wc == 0 && c.lane == 0) {
        float2 s = red[c.cl][0][0], sw = red[c.cl][0][1];
        int n = redn[c.cl][0];
        float m = redm[c.cl][0];
        for (int w = 1; w < kWarpsPerCol; ++w) {
            s = ff_add(s, red[c.cl][w][0]);
            sw = ff_add(sw, red[c.cl][w][1]);
            n += redn[c.cl][w];
            m = fmaxf(m, redm[c.cl][w]);
        }
        b.s1[c.j] = make_float2(s.x, sw.x);
        b.anyp[c.j] = (float)n;
        b.xmax[c.j] = m;
    }
}

// G step without a second contraction (sparse mode).  step = -alpha d + c with
// d the masked gradient whose product G d the first contraction left in b.g,
// and c nonzero only where the bound clamps (a small fraction of the entries),
// so G step = -alpha (G d) + sum over the clamped k of G(:, k) c_k.  The clamped
// entries of a column are compacted in thread order (deterministic), in rounds
// of kClampList, and b.g is overwritten with G step for the next iteration's
// mask kernel (fast_nnls.m:153).
constexpr int kStepRows = 16;   // most rows per thread: K <= 16 * 128 in sparse mode
constexpr int kClampList = 256;

template <int ROWS>
__device__ __forceinline__ void gstep_sparse(const ColBufs& b, int K, const ColIdx& c, bool act, int64_t o,
                                             float alpha_f, const float (&cc)[ROWS], unsigned cmask)
{
    __shared__ int lk[kColsPerCta][kClampList];
    __shared__ float lc[kColsPerCta][kClampList];
    __shared__ int wtot[kColsPerCta][kWarpsPerCol];
    __shared__ int rounds_s;
    const int cnt = __popc(cmask);
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (c.lane >= d) incl += v;
    }
    if (threadIdx.x == 0) rounds_s = 0;
    __syncthreads();
    if (c.lane == 31) wtot[c.cl][c.wc] = incl;
    __syncthreads();
    int base = 0, ntot = 0;
    for (int w = 0; w < kWarpsPerCol; ++w) {
        if (w < c.wc) base += wtot[c.cl][w];
        ntot += wtot[c.cl][w];
    }
    if (c.wc == 0 && c.lane == 0) atomicMax(&rounds_s, (ntot + kClampList - 1) / kClampList);
    __syncthreads();
    const int rounds = rounds_s;
    float corr[ROWS];
#pragma unroll
    for (int t = 0; t < ROWS; ++t) corr[t] = 0.f;
    for (int r = 0; r < rounds; ++r) {
        const int lo = r * kClampList;
        int pos = base + incl - cnt;
#pragma unroll
        for (int t = 0; t < ROWS; ++t)
            if (cmask & (1u << t)) {
                if (pos >= lo && pos < lo + kClampList) {
                    lk[c.cl][pos - lo] = c.wc * 32 + c.lane + t * kColThreads;
                    lc[c.cl][pos - lo] = cc[t];
                }
                ++pos;
            }
        __syncthreads();
        const int n = min(kClampList, ntot - lo);
        if (act) {
            // four clamped columns of G per pass keep four L2 reads in flight per row
            for (int m = 0; m < n; m += 4) {
                const float* gc[4];
                float cv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool ok = m + u < n;
                    gc[u] = b.Gf + (int64_t)(ok ? lk[c.cl][m + u] : 0) * K;
                    cv[u] = ok ? lc[c.cl][m + u] : 0.f;
                }
#pragma unroll
                for (int t = 0; t < ROWS; ++t) {
                    const int k = c.wc * 32 + c.lane + t * kColThreads;
                    if (k < K) {
                        float a = corr[t];
#pragma unroll
                        for (int u = 0; u < 4; ++u) a = fmaf(__ldg(gc[u] + k), cv[u], a);
                        corr[t] = a;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!act) return;
#pragma unroll
    for (int t = 0; t < ROWS; ++t) {
        const int k = c.wc * 32 + c.lane + t * kColThreads;
        if (k < K) b.g[o + k] = fmaf(-alpha_f, b.g[o + k], corr[t]);
    }
}

// exact line search, clamp, step statistic (LS_nnls.m:122-142, fast_nnls.m:119-145).
// `gu` (use_std) holds G * (column sum of d) / F, subtracted from G d.
template <int ROWS>
__global__ void __launch_bounds__(256) k_nn_step(ColBufs b, int K, int F, int solver, int sample, int tol_p,
                                                 int use_std)
{
    __shared__ float2 red[kColsPerCta][kWarpsPerCol][2];
    const ColIdx c = col_idx();
    const bool act = c.j < F && b.active[c.j];
    const int64_t o = (int64_t)c.j * K;
    const float gsc = (b.f16s && act) ? b.dsc[c.j] : 1.f;  // undoes the operand's power-of-two scale
    float s2_f = 0.f, s2w_f = 0.f;
    // when the ROWS register rows cover the column, the iterate and the masked
    // gradient are loaded once (all rows together) and kept for the update
    const bool regs = K <= ROWS * kColThreads;
    float2 xr[ROWS];
    float dmr[ROWS];
    if (act && regs) {
        float2 dr[ROWS];
        float gr[ROWS];
#pragma unroll
        for (int t = 0; t < ROWS; ++t) {
            const int k = c.wc * 32 + c.lane + t * kColThreads;
            if (k < K) {
                xr[t] = b.x[o + k];
                dr[t] = b.df[o + k];
                gr[t] = b.g[o + k];
            }
        }
#pragma unroll
        for (int t = 0; t < ROWS; ++t) {
            const int k = c.wc * 32 + c.lane + t * kColThreads;
            dmr[t] = 0.f;
            if (k < K) {
                dmr[t] = (xr[t].x > 0.f || dr[t].x < 0.f) ? dr[t].x + dr[t].y : 0.f;
                float g = gr[t] * gsc;
                if (use_std) g -= b.gu[k];
                wide_fma(dmr[t], g, s2_f, s2w_f);
            }
        }
    } else if (act) {
#pragma unroll 2
        for (int k = c.wc * 32 + c.lane; k < K; k += kColThreads) {
            const float2 xv = b.x[o + k], dv = b.df[o + k];
            const float dm = (xv.x > 0.f || dv.x < 0.f) ? dv.x + dv.y : 0.f;
            float g = b.g[o + k] * gsc;
            if (use_std) g -= b.gu[k];
            wide_fma(dm, g, s2_f, s2w_f);
        }
    }
    const float2 s2 = warp_sum_ff(s2_f);
    const float2 s2w = warp_sum_ff(s2w_f);
    if (c.lane == 0) {
        red[c.cl][c.wc][0] = s2;
        red[c.cl][c.wc][1] = s2w;
    }
    __syncthreads();
    // one thread per column forms alpha and shares it
    __shared__ float alpha_s[kColsPerCta];
    if (c.wc == 0 && c.lane == 0) {
        float2 den = red[c.cl][0][0], denw = red[c.cl][0][1];
        for (int w = 1; w < kWarpsPerCol; ++w) {
            den = ff_add(den, red[c.cl][w][0]);
            denw = ff_add(denw, red[c.cl][w][1]);
        }
        // NaN (no passive entry) gives no step (LS_nnls.m:123, fast_nnls.m:120);
        // so does a step beyond the FP32 range, which only sums below the
        // range of the products above can produce
        float af = act ? wide_ratio(b.s1[c.j], make_float2(den.x, denw.x)) : 0.f;
        if (!isfinite(af)) af = 0.f;
        alpha_s[c.cl] = af;
    }
    __syncthreads();
    float a1_f = 0.f, a2_f = 0.f;
    const float alpha_f = alpha_s[c.cl];
    // sparse mode: this thread's clamp corrections c = step - (-alpha d), rows
    // k = wc*32 + lane + 128 t (t < ROWS)
    float cc[ROWS];
    unsigned cmask = 0;
    // one row: clamp, store, operand (dense mode), statistic; returns the clamp
    // correction (0 where the bound does not clamp)
    auto row_with = [&](int k, float2 xv, float dm) -> float {
        const float pstep = dm * alpha_f;
        float2 xn = dd_add(xv, -pstep);
        // the step x_new - x exactly: -alpha d, or -x where the bound clamps
        float stp = -pstep, corr = 0.f;
        if (xn.x < 0.f) {
            xn = make_float2(0.f, 0.f);
            stp = -(xv.x + xv.y);
            corr = stp + pstep;
        }
        b.x[o + k] = xn;
        if (!b.sparse) put_operand(b, o, c.j, k, stp);
        // the convergence statistic takes the difference of the stored
        // iterates, as the reference does: it reaches 0 once the step falls
        // below the iterate's rounding, where the FP64 reference's does too
        const float dx = (xn.x - xv.x) + (xn.y - xv.y);
        if (solver == SOLVER_LS) {
            a1_f += dx;                      // sum(x - x_)
            a2_f = fmaf(xv.x, xv.x, a2_f);   // sum(x_.^2)
        } else {
            a1_f += (tol_p == 2) ? dx * dx : fabsf(dx);
        }
        return corr;
    };
    auto row = [&](int k) -> float {
        const float2 xv = b.x[o + k], dv = b.df[o + k];
        return row_with(k, xv, (xv.x > 0.f || dv.x < 0.f) ? dv.x + dv.y : 0.f);
    };
    if (act) {
#pragma unroll
        for (int t = 0; t < ROWS; ++t) {
            const int k = c.wc * 32 + c.lane + t * kColThreads;
            cc[t] = 0.f;
            if (k >= K) continue;
            cc[t] = regs ? row_with(k, xr[t], dmr[t]) : row(k);
            if (cc[t] != 0.f) cmask |= 1u << t;
        }
        // rows past ROWS * 128 (dense mode only: sparse mode needs K <= ROWS * 128)
        for (int k = c.wc * 32 + c.lane + ROWS * kColThreads; k < K; k += kColThreads) row(k);
    }
    const float2 a1p = warp_sum_ff(a1_f);
    const float2 a2p = warp_sum_ff(a2_f);
    __syncthreads();  // everyone has read the first exchange
    if (c.lane == 0) {
        red[c.cl][c.wc][0] = a1p;
        red[c.cl][c.wc][1] = a2p;
    }
    __syncthreads();
    const int it = b.cnt->iter;
    if (act && c.wc == 0 && c.lane == 0 && (it & 1)) {
        float2 t1 = red[c.cl][0][0], t2 = red[c.cl][0][1];
        for (int w = 1; w < kWarpsPerCol; ++w) {
            t1 = ff_add(t1, red[c.cl][w][0]);
            t2 = ff_add(t2, red[c.cl][w][1]);
        }
        // FP32 logarithms: the statistic feeds a linear fit with absolute
        // tolerances (tol_ * sample), far above FP32 rounding of a logarithm
        float t;
        int e;
        if (solver == SOLVER_LS) {
            t = logf(fabsf(t1.x)) - 0.5f * logf(t2.x);  // log(t1^2 / t2) / 2, LS_nnls.m:136
            e = (it - 1) / 2;
        } else {
            t = (tol_p == 2) ? 0.5f * logf(t1.x) : logf(t1.x);  // fast_nnls.m:138-141
            e = (it - 3) / 2;
        }
        if (e >= 0) b.test[(int64_t)(e % sample) * F + c.j] = (double)t;
    }
    if (b.sparse) gstep_sparse(b, K, c, act, o, alpha_f * gsc, cc, cmask);
}

// df = df + G x0 for a warm start with use_std (G x0 minus its column-sum term)
__global__ void k_nn_update(ColBufs b, int K, int F, int use_std)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = i / K;
        if (!b.active[j]) continue;
        float g = b.g[i];
        if (use_std) g -= b.gu[i - j * K];
        b.df[i] = dd_add(b.df[i], g);
    }
}

// k = Xi * window (Xi = inv(X'X) X' for X = [1 3 5 ...; 1 ...]), residual sum |X k - window|
__device__ void window_fit(const double* test, int sample, int F, int j, int e_last, const double* xi, double* k1,
                           double* resid, double* tend)
{
    double a = 0.0, c = 0.0;
    for (int t = 0; t < sample; ++t) {
        const double v = test[(int64_t)((e_last - sample + 1 + t) % sample) * F + j];
        a += xi[t] * v;
        c += xi[sample + t] * v;
    }
    double r = 0.0;
    for (int t = 0; t < sample; ++t) {
        const double v = test[(int64_t)((e_last - sample + 1 + t) % sample) * F + j];
        r += fabs((double)(2 * t + 1) * a + c - v);
    }
    *k1 = a;
    *resid = r;
    *tend = test[(int64_t)(e_last % sample) * F + j];
}

__global__ void k_nn_fit(ColBufs b, int F, int solver, int sample, int max_iter, int use_std)
{
    const int it = b.cnt->iter;
    if (it > max_iter || use_std || !(it & 1) || it <= 2 * sample) return;
    const int e_last = solver == SOLVER_LS ? (it - 1) / 2 : (it - 3) / 2;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!b.active[j]) continue;
        double k1, r, te;
        window_fit(b.test, sample, F, j, e_last, b.xi, &k1, &r, &te);
        b.fit[j] = k1;
        b.fit[F + j] = r;
        b.fit[2 * F + j] = te;
    }
}

__global__ void k_first_active(const int* __restrict__ active, NnlsCounters* cnt, int F)
{
    __shared__ int best;
    if (threadIdx.x == 0) best = F;
    __syncthreads();
    for (int j = threadIdx.x; j < F; j += blockDim.x)
        if (active[j]) atomicMin(&best, j);
    __syncthreads();
    if (threadIdx.x == 0) cnt->first = best;
}

// Retirement.
// LS_nnls.m:132-152: all columns after max_iter; on odd iterations past
//   2*sample: exp(t_end)/(1 - exp(k1 of the FIRST active column)) < tol
//   & sum|fit residual| < tol_*sample & exp(k1) < 1, or t_end == -inf.
// fast_nnls.m:146-158: all columns once s > max_iter; on odd s past 2*sample:
//   no passive entry, or h_max*exp(t_end)/(1-exp(k1)) < tol*K*max(x_old)
//   & sum|fit residual| < tol_*sample & exp(k1) < 1.
__global__ void k_nn_retire(ColBufs b, int32_t* __restrict__ iters, int K, int F, int solver, int sample, double tol,
                            double tol_, int max_iter, int use_std, double hmax)
{
    const int it = b.cnt->iter;
    const bool all = it > max_iter;
    if (!all && (use_std || !(it & 1) || it <= 2 * sample)) return;
    const double k1first = (b.cnt->first < F) ? b.fit[b.cnt->first] : 0.0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!b.active[j]) continue;
        bool ids = all;
        if (!all) {
            const double k1 = b.fit[j], r = b.fit[F + j], te = b.fit[2 * F + j];
            const bool c2 = r < tol_ * (double)sample;
            const bool c3 = exp(k1) < 1.0;
            if (solver == SOLVER_LS) {
                const bool c1 = exp(te) / (1.0 - exp(k1first)) < tol;
                ids = (c1 && c2 && c3) || (te == -INFINITY);
            } else {
                const bool c1 = hmax * exp(te) / (1.0 - exp(k1)) < tol * (double)K * (double)b.xmax[j];
                ids = (b.anyp[j] == 0.f) || (c1 && c2 && c3);
            }
        }
        if (ids) {
            b.active[j] = 0;
            if (iters) iters[j] = it;
            atomicSub(&b.cnt->active, 1);
        }
    }
}

// fast_nnls's test and retirement in one pass: its retirement reads only the
// column's own fit (unlike LS_nnls, which reads the first active column's).
__global__ void k_nn_fit_retire_fast(ColBufs b, int32_t* __restrict__ iters, int K, int F, int sample, double tol,
                                     double tol_, int max_iter, double hmax)
{
    const int it = b.cnt->iter;
    const bool all = it > max_iter;
    if (!all && (!(it & 1) || it <= 2 * sample)) return;
    const int e_last = (it - 3) / 2;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!b.active[j]) continue;
        bool ids = all;
        if (!all) {
            double k1, r, te;
            window_fit(b.test, sample, F, j, e_last, b.xi, &k1, &r, &te);
            b.fit[j] = k1;
            b.fit[F + j] = r;
            b.fit[2 * F + j] = te;
            const bool c1 = hmax * exp(te) / (1.0 - exp(k1)) < tol * (double)K * (double)b.xmax[j];
            ids = (b.anyp[j] == 0.f) || (c1 && r < tol_ * (double)sample && exp(k1) < 1.0);
        }
        if (ids) {
            b.active[j] = 0;
            if (iters) iters[j] = it;
            atomicSub(&b.cnt->active, 1);
        }
    }
}

// ------------------------------------------------------------ set-up kernels --
// df = -(h - lambda) for LS_nnls (h = A'Y), df = hs .* (-h + lambda) for fast_nnls
__global__ void k_df_init(const float* __restrict__ h, const float* __restrict__ hs, float2* __restrict__ df, int K,
                          int64_t n, double lambda, int solver)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double hv = (double)h[i];
        df[i] = dd_from((solver == SOLVER_LS) ? -(hv - lambda) : (double)hs[i % K] * (-hv + lambda));
    }
}

// df += g (FP32 contraction of the start point), x given in FP32
__global__ void k_add_g(float2* __restrict__ df, const float* __restrict__ g, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        df[i] = dd_add(df[i], g[i]);
}

__global__ void k_x_from(float2* __restrict__ x, const float* __restrict__ src, const float* __restrict__ hs, int K,
                         int64_t n)
{
    // x = src (LS_nnls start point) or diag(1./hs) * W (fast_nnls.m:72)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = dd_from(hs ? (double)src[i] / (double)hs[i % K] : (double)src[i]);
}

__global__ void k_x_out(float* __restrict__ X, const float2* __restrict__ x, const float* __restrict__ hs, int K,
                        int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        X[i] = hs ? (float)((double)hs[i % K] * dd_to(x[i])) : (float)dd_to(x[i]);
}

// use_std (LS_nnls.m:107): u = sum over active columns of the operand / F
__global__ void k_colsum_operand(ColBufs b, int K, int F)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < F; ++j) {
            if (!b.active[j]) continue;
            if (b.vhi) {
                const int64_t i = (((int64_t)(k >> 6) * b.F + j) << 6) + (k & 63);
                s += (double)__bfloat162float(__ushort_as_bfloat16(b.vhi[i])) +
                     (double)__bfloat162float(__ushort_as_bfloat16(b.vlo[i]));
            } else {
                s += (double)b.v[(int64_t)j * K + k];
            }
        }
        b.u[k] = (float)(s / (double)F);
    }
}

__global__ void k_movie_rowsum(const void* __restrict__ Y, int f16, int64_t P, int64_t F, float* __restrict__ out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int64_t f = 0; f < F; ++f)
            s += f16 ? (double)__half2float(static_cast<const __half*>(Y)[p + P * f])
                     : (double)static_cast<const float*>(Y)[p + P * f];
        out[p] = (float)s;
    }
}

// h(:, j) -= w / F
__global__ void k_sub_colvec(float* __restrict__ h, const float* __restrict__ w, int K, int F, float invF)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        h[i] -= w[i % K] * invF;
}

// Q = G ./ sqrt(diag G diag G'), hs = 1 ./ sqrt(diag G)   (fast_nnls.m:54-56)
__global__ void k_diag_rsqrt(const float* __restrict__ G, float* __restrict__ hs, int K)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
        hs[k] = (float)(1.0 / sqrt((double)G[(int64_t)k * K + k]));
}

__global__ void k_normalise_gram(float* __restrict__ G, const float* __restrict__ hs, int K)
{
    const int64_t n = (int64_t)K * K;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % K), c = (int)(i / K);
        G[i] = (float)((double)G[i] * (double)hs[r] * (double)hs[c]);
    }
}

__global__ void k_fill_int(int* __restrict__ a, int n, int v)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

// --------------------------------------------- warm_start == 1 (fast_nnls.m:66-69) --
// x = inv(Q) (-df) by Gauss-Jordan elimination with partial pivoting on the
// augmented FP64 matrix M = [Q | -df] (K x (K + F), column-major): after
// step j column j is e_j, and at the end the right block holds inv(Q) (-df)
// (MATLAB forms inv(Q) and multiplies; the solve is the same product without
// the explicit inverse).  A zero pivot sets *err (MATLAB warns that Q is
// singular and returns Inf/NaN).
__global__ void __launch_bounds__(1024) k_gj_pivot(double* __restrict__ M, int K, int64_t ncols, int j,
                                                   int* __restrict__ err)
{
    __shared__ double bv[32];
    __shared__ int bi[32];
    __shared__ int piv;
    double best = -1.0;
    int arg = j;
    for (int i = j + threadIdx.x; i < K; i += blockDim.x) {
        const double v = fabs(M[i + (int64_t)K * j]);
        if (v > best) { best = v; arg = i; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, arg, off);
        if (ov > best || (ov == best && oi < arg)) { best = ov; arg = oi; }
    }
    if ((threadIdx.x & 31) == 0) { bv[threadIdx.x >> 5] = best; bi[threadIdx.x >> 5] = arg; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = -1.0;
        int a = j;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            if (bv[w] > b || (bv[w] == b && bi[w] < a)) { b = bv[w]; a = bi[w]; }
        piv = a;
        if (!(b > 0.0)) atomicExch(err, 1);
    }
    __syncthreads();
    const int p = piv;
    // swap rows j and p, then scale row j by the pivot (columns j.., column j becomes 1)
    for (int64_t c = j + threadIdx.x; c < ncols; c += blockDim.x) {
        const double a = M[j + (int64_t)K * c], b = M[p + (int64_t)K * c];
        M[j + (int64_t)K * c] = b;
        M[p + (int64_t)K * c] = a;
    }
    __syncthreads();
    const double inv = 1.0 / M[j + (int64_t)K * j];
    __syncthreads();
    for (int64_t c = j + threadIdx.x; c < ncols; c += blockDim.x) M[j + (int64_t)K * c] *= inv;
}

__global__ void k_gj_elim(double* __restrict__ M, int K, int64_t ncols, int j)
{
    const int64_t w = ncols - j - 1;  // columns after j
    const int64_t n = (int64_t)K * w;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % K);
        const int64_t c = j + 1 + e / K;
        if (i == j) continue;
        M[i + (int64_t)K * c] -= M[i + (int64_t)K * j] * M[j + (int64_t)K * c];
    }
}

// M = [Q | -df] in FP64
__global__ void k_gj_load(const float* __restrict__ G, const float2* __restrict__ df, int K, int64_t F,
                          double* __restrict__ M)
{
    const int64_t n = (int64_t)K * (K + F);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / K;
        M[e] = c < K ? (double)G[e] : -dd_to(df[e - (int64_t)K * K]);
    }
}

// x = max(inv(Q)(-df), 0) as the double-float iterate and its FP32 copy
__global__ void k_gj_store(const double* __restrict__ M, int K, int64_t F, float2* __restrict__ x,
                           float* __restrict__ xf)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double v = M[(int64_t)K * K + e];
        if (v < 0.0) v = 0.0;  // x(x<0) = 0
        x[e] = dd_from(v);
        xf[e] = (float)v;
    }
}

// -------------------------------------------- opts.total (fast_nnls.m:101-117) --
// One step length for all columns: alpha = sum(df_.^2) / sum(df_ .* (Q df_))
// over the whole K x F block.  Per-block partial sums (FP32 two-sum pairs)
// are reduced by one block into the device scalar alpha.
__global__ void __launch_bounds__(256) k_tot_mask(ColBufs b, int64_t n, float2* __restrict__ part)
{
    float2 acc = make_float2(0.f, 0.f);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 xv = b.x[e], dv = b.df[e];
        const float dm = (xv.x > 0.f || dv.x < 0.f) ? dv.x + dv.y : 0.f;  // df .* passive
        b.v[e] = dm;
        acc = ff_add(acc, make_float2(dm * dm, fmaf(dm, dm, -dm * dm)));
    }
    __shared__ float2 red[8];
    for (int off = 16; off > 0; off >>= 1)
        acc = ff_add(acc, make_float2(__shfl_xor_sync(0xffffffffu, acc.x, off), __shfl_xor_sync(0xffffffffu, acc.y, off)));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 s = red[0];
        for (int w = 1; w < 8; ++w) s = ff_add(s, red[w]);
        part[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) k_tot_den(const float* __restrict__ v, const float* __restrict__ g, int64_t n,
                                                 float2* __restrict__ part)
{
    float2 acc = make_float2(0.f, 0.f);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float a = v[e], c = g[e];
        acc = ff_add(acc, make_float2(a * c, fmaf(a, c, -a * c)));
    }
    __shared__ float2 red[8];
    for (int off = 16; off > 0; off >>= 1)
        acc = ff_add(acc, make_float2(__shfl_xor_sync(0xffffffffu, acc.x, off), __shfl_xor_sync(0xffffffffu, acc.y, off)));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 s = red[0];
        for (int w = 1; w < 8; ++w) s = ff_add(s, red[w]);
        part[blockIdx.x] = s;
    }
}

// alpha = sum(num parts) / sum(den parts); NaN -> 0 (fast_nnls.m:103)
__global__ void k_tot_alpha(const float2* __restrict__ num, const float2* __restrict__ den, int nb,
                            float* __restrict__ alpha)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, c = 0.0;
    for (int i = 0; i < nb; ++i) {
        a += (double)num[i].x + (double)num[i].y;
        c += (double)den[i].x + (double)den[i].y;
    }
    double al = a / c;
    if (al != al) al = 0.0;
    *alpha = (float)al;
}

// x_ = max(x - alpha df_, 0); v = x_ - x (the operand of Q (x_ - x)); x = x_
__global__ void k_tot_step(ColBufs b, int64_t n, const float* __restrict__ alpha)
{
    const float al = *alpha;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 xv = b.x[e];
        const float pstep = b.v[e] * al;
        float2 xn = dd_add(xv, -pstep);
        float stp = -pstep;
        if (xn.x < 0.f) {
            xn = make_float2(0.f, 0.f);
            stp = -(xv.x + xv.y);
        }
        b.x[e] = xn;
        b.v[e] = stp;
    }
}

// X = diag(h) * ones: the reference leaves xx at its initial ones in total
// mode (fast_nnls.m:87 and the break at :113-115 never assigns it)
__global__ void k_fill_h(float* __restrict__ X, const float* __restrict__ hs, int K, int64_t n)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        X[e] = hs[e % K];
}

__global__ void k_df_out(const float2* __restrict__ df, int64_t n, float* __restrict__ out)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = (float)dd_to(df[e]);
}

__global__ void k_df_from(const float* __restrict__ src, int64_t n, float2* __restrict__ df)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        df[e] = make_float2(src[e], 0.f);
}

// ------------------------------------------------------------ host driver --
static std::vector<double> fit_matrix(int sample)
{
    double s11 = 0, s12 = 0, s22 = sample;
    for (int t = 0; t < sample; ++t) {
        const double a = 2.0 * t + 1.0;
        s11 += a * a;
        s12 += a;
    }
    const double det = s11 * s22 - s12 * s12;
    const double i11 = s22 / det, i12 = -s12 / det, i22 = s11 / det;
    std::vector<double> xi(2 * sample);
    for (int t = 0; t < sample; ++t) {
        const double a = 2.0 * t + 1.0;
        xi[t] = i11 * a + i12;
        xi[sample + t] = i12 * a + i22;
    }
    return xi;
}

struct NnlsWork {
    ColBufs b;
    float* h;      // K x F FP32 (A'Y)
    float* G;      // K x K Gram (or normalised Gram)
    float* hs;     // K scaling (fast_nnls)
    uint16_t *Ghi, *Glo;
    bool split;
    bool f16s;      // Gram and iteration operands as scaled FP16 hi/lo (else BF16 hi/lo)
    float gscale;   // power of two applied to the Gram before its FP16 split (max|G| * gscale in [2^13, 2^14))
};

static int alloc_work(sid_ctx* c, int64_t K, int64_t F, int sample, bool split, NnlsWork* w, cudaStream_t st)
{
    const int64_t KF = K * F;
    DBuf* nn = c->nn;
    SID_TRY(nn[0].alloc(KF * 8));  // x
    SID_TRY(nn[1].alloc(KF * 8));  // df
    SID_TRY(nn[2].alloc(KF * 4));  // v / h
    SID_TRY(nn[3].alloc(KF * 4));  // g
    SID_TRY(nn[4].alloc((size_t)sample * F * 8));
    SID_TRY(nn[5].alloc((size_t)(7 * F + 2 * sample + 8) * 8));
    SID_TRY(nn[6].alloc((size_t)F * 4 + 64));
    SID_TRY(nn[7].alloc((size_t)(K * K + 3 * K + 16) * 4));
    SID_TRY(nn[10].alloc(KF * 4));  // h
    if (split) {
        SID_TRY(nn[8].alloc((size_t)blk16_elems(K, F) * 2));
        SID_TRY(nn[9].alloc((size_t)blk16_elems(K, F) * 2));
        SID_TRY(nn[11].alloc((size_t)blk16_elems(K, K) * 2));
        SID_TRY(nn[12].alloc((size_t)blk16_elems(K, K) * 2));
        // zero the K-blocked operands once: entries past K in the last block stay zero
        SID_CUDA_TRY(cudaMemsetAsync(nn[8].p, 0, (size_t)blk16_elems(K, F) * 2, st));
        SID_CUDA_TRY(cudaMemsetAsync(nn[9].p, 0, (size_t)blk16_elems(K, F) * 2, st));
    }
    ColBufs& b = w->b;
    b.x = nn[0].as<float2>();
    b.df = nn[1].as<float2>();
    b.v = nn[2].as<float>();
    b.g = nn[3].as<float>();
    b.test = nn[4].as<double>();
    double* sc = nn[5].as<double>();
    b.s1 = reinterpret_cast<float2*>(sc);
    b.fit = sc + F;  // 3F
    b.anyp = reinterpret_cast<float*>(sc + 4 * F);
    b.xmax = reinterpret_cast<float*>(sc + 5 * F);
    b.xi = sc + 6 * F;
    b.dsc = reinterpret_cast<float*>(sc + 6 * F + 2 * sample + 8);
    b.active = nn[6].as<int>();
    b.cnt = reinterpret_cast<NnlsCounters*>(nn[6].as<uint8_t>() + cdiv(F * 4, 16) * 16);
    float* fs = nn[7].as<float>();
    w->G = fs;
    w->hs = fs + K * K;
    b.u = w->hs + K;
    b.gu = b.u + K;
    w->h = nn[10].as<float>();
    b.F = (int)F;
    b.vhi = split ? nn[8].as<uint16_t>() : nullptr;
    b.vlo = split ? nn[9].as<uint16_t>() : nullptr;
    w->Ghi = split ? nn[11].as<uint16_t>() : nullptr;
    w->Glo = split ? nn[12].as<uint16_t>() : nullptr;
    w->split = split;
    w->f16s = false;
    w->gscale = 1.f;
    b.f16s = 0;
    return SID_OK;
}

// Operand format of the iterations: scaled FP16 hi/lo in sparse mode (one
// contraction per iteration; the operand is d, whose column scale the mask
// kernel finds), BF16 hi/lo otherwise (use_std's column sums and the dense
// mode's second operand read BF16).
static bool f16_operands(const NnlsWork& w, int64_t K, bool use_std)
{
    return w.split && !use_std && K <= (int64_t)kStepRows * kColThreads;
}

// 16-bit split of the (normalised) Gram in the format the iterations use.  The
// FP16 split scales the Gram by the power of two that puts its largest entry
// in [2^13, 2^14) (2^14 for fast_nnls's normalised Gram, whose diagonal is 1).
static int split_gram(sid_ctx* c, NnlsWork& w, int64_t K, bool f16s, cudaStream_t st)
{
    w.f16s = f16s;
    w.b.f16s = f16s ? 1 : 0;
    w.gscale = 1.f;
    if (!w.split) return SID_OK;
    if (f16s) {
        SID_TRY(c->scal.alloc(64));
        SID_TRY(absmax(w.G, K * K, c->scal.as<unsigned int>(), st));
        unsigned int bits = 0;
        SID_CUDA_TRY(cudaMemcpyAsync(&bits, c->scal.p, sizeof(bits), cudaMemcpyDeviceToHost, st));
        SID_CUDA_TRY(cudaStreamSynchronize(st));
        float mx;
        std::memcpy(&mx, &bits, sizeof(mx));
        if (mx > 0.f && std::isfinite(mx)) {
            int ex;
            std::frexp(mx, &ex);
            w.gscale = std::ldexp(1.f, std::max(-126, std::min(126, 14 - ex)));
        }
    }
    return split16(w.G, K, K, K, w.Ghi, w.Glo, !f16s, w.gscale, st);
}

// g = G * operand (operand = b.v or its BF16 split)
static int gmul(sid_ctx* c, const NnlsWork& w, int64_t K, int64_t F, cudaStream_t st)
{
    if (!w.split)
        return sgemm_tn(w.G, w.b.v, K, F, K, K, K, w.b.g, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4),
                        st);
    const void* As[3] = {w.Ghi, w.Ghi, w.Glo};
    const void* Bs[3] = {w.b.vhi, w.b.vlo, w.b.vhi};
    int bn = 0, sk = 0;
    gemm_autotune((int)K, (int)F, (int)cdiv(K, 64), &bn, &sk);
    return gemm_tn(As, Bs, 3, K, F, K, !w.f16s, w.b.g, K, 1.f / w.gscale, 0.f, bn, sk,
                   c->ws.as<float>(), (int64_t)(c->ws.bytes / 4),
                   c->errflag.as<int>(), st);
}

static int ensure_gemm_ws(sid_ctx* c, int64_t K, int64_t F, bool split)
{
    int64_t need = std::max<int64_t>(sgemm_ws_elems(K, F, K), sgemm_ws_elems(K, 1, K));
    if (split) {
        int bn = 0, sk = 0;
        gemm_autotune((int)K, (int)F, (int)cdiv(K, 64), &bn, &sk);
        need = std::max<int64_t>(need, (int64_t)sk * K * F);
    }
    return c->ws.alloc((size_t)need * 4);
}

static const int kChunk = 16;  // iterations per captured graph

template <class Body>
static int run_iterations(sid_ctx* c, const ColBufs& b, int max_iter, Body body, cudaStream_t st)
{
    cudaStream_t cap = st;
    bool own = false;
    if (st == nullptr) {
        SID_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        own = true;
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = SID_OK;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        set_error("NNLS: stream capture failed to start");
        rc = SID_ECUDA;
    }
    if (rc == SID_OK) {
        for (int i = 0; i < kChunk && rc == SID_OK; ++i) rc = body(cap);
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        if (rc == SID_OK && e != cudaSuccess) {
            set_error("NNLS: stream capture failed: %s", cudaGetErrorString(e));
            rc = SID_ECUDA;
        }
    }
    if (rc == SID_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        set_error("NNLS: graph instantiation failed");
        rc = SID_ECUDA;
    }
    const int max_chunks = (max_iter + 2) / kChunk + 2;
    for (int ch = 0; ch < max_chunks && rc == SID_OK; ++ch) {
        if (cudaGraphLaunch(exec, cap) != cudaSuccess) {
            set_error("NNLS: graph launch failed");
            rc = SID_ECUDA;
            break;
        }
        NnlsCounters h;
        cudaError_t e = cudaMemcpyAsync(&h, b.cnt, sizeof(h), cudaMemcpyDeviceToHost, cap);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cap);
        if (e != cudaSuccess) {
            set_error("NNLS: %s", cudaGetErrorString(e));
            rc = SID_ECUDA;
            break;
        }
        if (h.active == 0) break;
        if (ch == max_chunks - 1) {
            set_error("NNLS: columns still active after the iteration cap");
            rc = SID_ENOCONV;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (own) cudaStreamDestroy(cap);
    if (rc == SID_OK) rc = ctx_sync(c, st);
    return rc;
}

static int nnls_common_checks(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                              const sid_nnls_opts* o, int prec)
{
    SID_REQUIRE(c && A && Y && o, "NNLS: NULL argument");
    SID_REQUIRE(P > 0 && K > 0 && F > 0, "NNLS: empty problem (P=%lld K=%lld F=%lld)", (long long)P, (long long)K,
                (long long)F);
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "NNLS: unknown Y dtype %d", ydtype);
    SID_REQUIRE(prec == SID_PREC_FP32 || prec == SID_PREC_SPLIT, "NNLS: precision must be FP32 or SPLIT");
    SID_REQUIRE(o->sample >= 1 && o->max_iter >= 0, "NNLS: sample must be >= 1 and max_iter >= 0");
    return SID_OK;
}

// Shared iteration loop of both solvers.
static int iterate(sid_ctx* c, NnlsWork& w, int64_t K, int64_t F, int solver, const sid_nnls_opts* o, double hmax,
                   int32_t* iters, cudaStream_t st)
{
    ColBufs& b = w.b;
    const int sample = (int)o->sample;
    const std::vector<double> xi = fit_matrix(sample);
    SID_CUDA_TRY(cudaMemcpyAsync(b.xi, xi.data(), xi.size() * 8, cudaMemcpyHostToDevice, st));
    k_fill_int<<<64, 256, 0, st>>>(b.active, (int)F, 1);
    SID_CHECK_LAUNCH();
    NnlsCounters h0{solver == SOLVER_FAST ? 1 : 0, (int)F, 0, 0};  // fast_nnls starts at s = 1
    SID_CUDA_TRY(cudaMemcpyAsync(b.cnt, &h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    SID_TRY(ensure_gemm_ws(c, K, F, w.split));
    // one contraction outside the capture configures the kernels
    SID_TRY(gmul(c, w, K, F, st));
    // the mask kernel applies the previous iteration's df += G step from g:
    // nothing is pending before the first iteration
    SID_CUDA_TRY(cudaMemsetAsync(b.g, 0, (size_t)(K * F) * sizeof(float), st));
    SID_CUDA_TRY(cudaMemsetAsync(b.gu, 0, (size_t)K * sizeof(float), st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    const int use_std = (solver == SOLVER_LS && o->use_std) ? 1 : 0;
    const int max_iter = (int)o->max_iter;
    // G step from G d and the clamp corrections (one contraction per iteration),
    // except with use_std, whose operand carries a column-mean term
    b.sparse = (!use_std && K <= (int64_t)kStepRows * kColThreads) ? 1 : 0;
    b.Gf = w.G;
    auto gmul_std = [&](cudaStream_t s) -> int {
        SID_TRY(gmul(c, w, K, F, s));
        if (use_std) {
            // G(v) = G v - G (sum over active columns of v) / F   (LS_nnls.m:107)
            k_colsum_operand<<<cdiv(K, 256), 256, 0, s>>>(b, (int)K, (int)F);
            SID_CHECK_LAUNCH();
            SID_TRY(sgemm_tn(w.G, b.u, K, 1, K, K, K, b.gu, K, 1.f, 0.f, c->ws.as<float>(),
                             (int64_t)(c->ws.bytes / 4), s));
        }
        return SID_OK;
    };
    const bool fast_fused = solver == SOLVER_FAST && !use_std;
    auto body = [&](cudaStream_t s) -> int {
        // the mask kernel advances the iteration counter (one launch fewer per iteration)
        if (K <= 8 * kColThreads)
            k_nn_mask<8><<<(unsigned)cdiv(F, kColsPerCta), kColsPerCta * kColThreads, 0, s>>>(b, (int)K, (int)F,
                                                                                             use_std, 1);
        else
            k_nn_mask<0><<<(unsigned)cdiv(F, kColsPerCta), kColsPerCta * kColThreads, 0, s>>>(b, (int)K, (int)F,
                                                                                             use_std, 1);
        SID_CHECK_LAUNCH();
        SID_TRY(gmul_std(s));
        if (K <= 8 * kColThreads)
            k_nn_step<8><<<(unsigned)cdiv(F, kColsPerCta), kColsPerCta * kColThreads, 0, s>>>(
                b, (int)K, (int)F, solver, sample, (int)o->tol_p, use_std);
        else
            k_nn_step<kStepRows><<<(unsigned)cdiv(F, kColsPerCta), kColsPerCta * kColThreads, 0, s>>>(
                b, (int)K, (int)F, solver, sample, (int)o->tol_p, use_std);
        SID_CHECK_LAUNCH();
        if (!b.sparse) SID_TRY(gmul_std(s));  // G step: applied by the next iteration's mask kernel
        if (fast_fused) {
            k_nn_fit_retire_fast<<<cdiv(F, 256), 256, 0, s>>>(b, iters, (int)K, (int)F, sample, o->tol, o->tol_,
                                                              max_iter, hmax);
            SID_CHECK_LAUNCH();
            return SID_OK;
        }
        k_nn_fit<<<cdiv(F, 256), 256, 0, s>>>(b, (int)F, solver, sample, max_iter, use_std);
        SID_CHECK_LAUNCH();
        if (solver == SOLVER_LS) {
            k_first_active<<<1, 1024, 0, s>>>(b.active, b.cnt, (int)F);
            SID_CHECK_LAUNCH();
        }
        k_nn_retire<<<cdiv(F, 256), 256, 0, s>>>(b, iters, (int)K, (int)F, solver, sample, o->tol, o->tol_, max_iter,
                                                  use_std, hmax);
        SID_CHECK_LAUNCH();
        return SID_OK;
    };
    return run_iterations(c, b, max_iter, body, st);
}

}  // namespace sid

using namespace sid;

extern "C" void sid_ls_nnls_defaults(sid_nnls_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->lambda = 0.0;
    o->sample = 300;
    o->tol = 1e-7;
    o->tol_ = 1e-2;
    o->max_iter = 2000;
    o->use_std = 0;
    o->tol_p = 1;
}

extern "C" void sid_fast_nnls_defaults(sid_nnls_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->lambda = 0.0;
    o->sample = 30;
    o->tol = 1e-6;
    o->tol_ = 1e-1;
    o->max_iter = 2000;
    o->use_std = 0;
    o->tol_p = 1;
}

extern "C" int sid_ls_nnls(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                           const sid_nnls_opts* o, float* G, int g_given, float* X, int x_given, int prec,
                           int32_t* iters, void* stream)
{
    SID_TRY(nnls_common_checks(c, A, Y, ydtype, P, K, F, o, prec));
    SID_REQUIRE(X, "LS_nnls: X is NULL");
    SID_REQUIRE(!g_given || G, "LS_nnls: g_given without G");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool split = prec == SID_PREC_SPLIT;
    NnlsWork w;
    SID_TRY(alloc_work(c, K, F, (int)o->sample, split, &w, st));
    ColBufs& b = w.b;
    const bool f16 = ydtype == SID_DTYPE_F16;
    // h = A'Y   (LS_nnls.m:76)
    SID_TRY(contract(c, A, Y, f16, K, F, P, P, P, w.h, K, 1.f, 0.f, f16 ? SID_PREC_SPLIT : prec, st));
    // G = A'A   (LS_nnls.m:82), or the caller's G
    if (g_given) SID_CUDA_TRY(cudaMemcpyAsync(w.G, G, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
    else SID_TRY(contract(c, A, A, false, K, K, P, P, P, w.G, K, 1.f, 0.f, prec, st));
    if (o->use_std) {
        // h = h - A' sum(Y,2) / F   (LS_nnls.m:104)
        DBuf ys;
        SID_TRY(ys.alloc((size_t)P * 4));
        k_movie_rowsum<<<1024, 256, 0, st>>>(Y, f16 ? 1 : 0, P, F, ys.as<float>());
        SID_CHECK_LAUNCH();
        SID_TRY(c->ws.alloc((size_t)std::max<int64_t>(sgemm_ws_elems(K, 1, P), 1) * 4));
        SID_TRY(sgemm_tn(A, ys.as<float>(), K, 1, P, P, P, b.u, K, 1.f, 0.f, c->ws.as<float>(),
                         (int64_t)(c->ws.bytes / 4), st));
        k_sub_colvec<<<1024, 256, 0, st>>>(w.h, b.u, (int)K, (int)F, 1.f / (float)F);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaStreamSynchronize(st));
        ys.release();
    }
    SID_TRY(split_gram(c, w, K, f16_operands(w, K, o->use_std != 0), st));
    // df = -h + G x0  (x0 = 0 unless given)
    k_df_init<<<1024, 256, 0, st>>>(w.h, nullptr, b.df, (int)K, K * F, o->lambda, SOLVER_LS);
    SID_CHECK_LAUNCH();
    if (x_given) {
        k_x_from<<<1024, 256, 0, st>>>(b.x, X, nullptr, (int)K, K * F);
        SID_CHECK_LAUNCH();
        SID_TRY(ensure_gemm_ws(c, K, F, split));
        if (o->use_std) {
            // G x0 through the iterations' own operand (the column-sum kernel reads it)
            if (split) SID_TRY(split16(X, K, F, K, b.vhi, b.vlo, true, 1.f, st));
            else SID_CUDA_TRY(cudaMemcpyAsync(b.v, X, (size_t)(K * F) * 4, cudaMemcpyDeviceToDevice, st));
            SID_TRY(gmul(c, w, K, F, st));
        } else {
            // G x0 once, FP32
            SID_TRY(sgemm_tn(w.G, X, K, F, K, K, K, b.g, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4),
                             st));
        }
        if (o->use_std) {
            // the start gradient needs G(x0) - G sum(x0,2)/F
            k_fill_int<<<64, 256, 0, st>>>(b.active, (int)F, 1);
            SID_CHECK_LAUNCH();
            k_colsum_operand<<<cdiv(K, 256), 256, 0, st>>>(b, (int)K, (int)F);
            SID_CHECK_LAUNCH();
            SID_TRY(sgemm_tn(w.G, b.u, K, 1, K, K, K, b.gu, K, 1.f, 0.f, c->ws.as<float>(),
                             (int64_t)(c->ws.bytes / 4), st));
            k_fill_int<<<64, 256, 0, st>>>(b.active, (int)F, 1);
            SID_CHECK_LAUNCH();
            k_nn_update<<<2048, 256, 0, st>>>(b, (int)K, (int)F, 1);
        } else {
            k_add_g<<<1024, 256, 0, st>>>(b.df, b.g, K * F);
        }
        SID_CHECK_LAUNCH();
    } else {
        SID_CUDA_TRY(cudaMemsetAsync(b.x, 0, (size_t)(K * F) * 8, st));
    }
    SID_TRY(iterate(c, w, K, F, SOLVER_LS, o, 0.0, iters, st));
    k_x_out<<<1024, 256, 0, st>>>(X, b.x, nullptr, (int)K, K * F);
    SID_CHECK_LAUNCH();
    if (G && !g_given) SID_CUDA_TRY(cudaMemcpyAsync(G, w.G, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
    return ctx_sync(c, st);
}

// x = inv(Q)(-df), clamped, as the start (fast_nnls.m:66-69); xf: FP32 copy
static int warm_inverse(sid_ctx* c, NnlsWork& w, int64_t K, int64_t F, cudaStream_t st)
{
    DBuf& m = c->nn[15];
    SID_TRY(m.alloc((size_t)(K * (K + F)) * 8 + 16));
    double* M = m.as<double>();
    int* err = reinterpret_cast<int*>(m.as<uint8_t>() + (size_t)(K * (K + F)) * 8);
    SID_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    k_gj_load<<<2048, 256, 0, st>>>(w.G, w.b.df, (int)K, F, M);
    SID_CHECK_LAUNCH();
    const int64_t ncols = K + F;
    for (int j = 0; j < (int)K; ++j) {
        k_gj_pivot<<<1, 1024, 0, st>>>(M, (int)K, ncols, j, err);
        const int64_t n = K * (ncols - j - 1);
        if (n > 0) k_gj_elim<<<(unsigned)std::min<int64_t>(cdiv(n, 256), 4096), 256, 0, st>>>(M, (int)K, ncols, j);
    }
    SID_CHECK_LAUNCH();
    int he = 0;
    SID_CUDA_TRY(cudaMemcpyAsync(&he, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    SID_REQUIRE(!he, "fast_nnls: warm_start == 1 needs inv(Q), and Q is singular");
    k_gj_store<<<1024, 256, 0, st>>>(M, (int)K, F, w.b.x, w.b.v);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// opts.total: max_iter iterations with one step length for all columns
static int total_iterations(sid_ctx* c, NnlsWork& w, int64_t K, int64_t F, int max_iter, cudaStream_t st)
{
    ColBufs& b = w.b;
    const int64_t n = K * F;
    const int nb = 512;
    DBuf& pb = c->nn[13];
    SID_TRY(pb.alloc((size_t)(2 * nb) * sizeof(float2) + 16));
    float2* pnum = pb.as<float2>();
    float2* pden = pnum + nb;
    float* alpha = reinterpret_cast<float*>(pden + nb);
    SID_TRY(c->ws.alloc((size_t)std::max<int64_t>(sgemm_ws_elems(K, F, K), 1) * 4));
    // the loop breaks once s > max_iter after an iteration (fast_nnls.m:112-116): max(max_iter, 1) iterations
    for (int it = 0; it < std::max(max_iter, 1); ++it) {
        k_tot_mask<<<nb, 256, 0, st>>>(b, n, pnum);
        SID_TRY(sgemm_tn(w.G, b.v, K, F, K, K, K, b.g, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4),
                         st));
        k_tot_den<<<nb, 256, 0, st>>>(b.v, b.g, n, pden);
        k_tot_alpha<<<1, 32, 0, st>>>(pnum, pden, nb, alpha);
        k_tot_step<<<1024, 256, 0, st>>>(b, n, alpha);
        SID_CHECK_LAUNCH();
        // df = df + Q (x_ - x)   fast_nnls.m:106
        SID_TRY(sgemm_tn(w.G, b.v, K, F, K, K, K, b.g, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4),
                         st));
        k_add_g<<<1024, 256, 0, st>>>(b.df, b.g, n);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

extern "C" int sid_fast_nnls_ex(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                                const sid_nnls_opts* o, int total, int warm_mode, const float* W, const float* Q_in,
                                const float* df_in, const float* h_in, float* X, float* Q_out, float* df_out,
                                float* h_out, int prec, int32_t* iters, void* stream)
{
    SID_REQUIRE(c && o && X, "fast_nnls: NULL argument");
    SID_REQUIRE(K > 0 && F > 0, "fast_nnls: empty problem (K=%lld F=%lld)", (long long)K, (long long)F);
    SID_REQUIRE(prec == SID_PREC_FP32 || prec == SID_PREC_SPLIT, "NNLS: precision must be FP32 or SPLIT");
    SID_REQUIRE(o->sample >= 1 && o->max_iter >= 0, "NNLS: sample must be >= 1 and max_iter >= 0");
    SID_REQUIRE(o->tol_p == 1 || o->tol_p == 2, "fast_nnls: tol_p must be 1 or 2");
    SID_REQUIRE(warm_mode >= 0 && warm_mode <= 2, "fast_nnls: warm_mode must be 0, 1 or 2");
    SID_REQUIRE(warm_mode != 2 || W, "fast_nnls: warm_mode 2 needs the warm-start matrix");
    SID_REQUIRE(!Q_in == !h_in, "fast_nnls: Q and h are given together (fast_nnls.m:58-62)");
    const bool need_a = !Q_in || !df_in;
    if (need_a) {
        SID_REQUIRE(A && Y && P > 0, "fast_nnls: A and Y are needed to form %s", !Q_in ? "Q" : "df");
        SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "NNLS: unknown Y dtype %d", ydtype);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool split = prec == SID_PREC_SPLIT;
    NnlsWork w;
    SID_TRY(alloc_work(c, K, F, (int)o->sample, split, &w, st));
    ColBufs& b = w.b;
    const bool f16 = ydtype == SID_DTYPE_F16;
    if (Q_in) {
        // the caller's normalised Gram and scaling (fast_nnls.m:58-62)
        SID_CUDA_TRY(cudaMemcpyAsync(w.G, Q_in, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
        SID_CUDA_TRY(cudaMemcpyAsync(w.hs, h_in, (size_t)K * 4, cudaMemcpyDeviceToDevice, st));
    } else {
        // Q = A'A normalised, hs = 1./sqrt(diag)   (fast_nnls.m:53-56)
        SID_TRY(contract(c, A, A, false, K, K, P, P, P, w.G, K, 1.f, 0.f, prec, st));
        k_diag_rsqrt<<<cdiv(K, 256), 256, 0, st>>>(w.G, w.hs, (int)K);
        SID_CHECK_LAUNCH();
        k_normalise_gram<<<1024, 256, 0, st>>>(w.G, w.hs, (int)K);
        SID_CHECK_LAUNCH();
    }
    if (df_in) {
        k_df_from<<<1024, 256, 0, st>>>(df_in, K * F, b.df);
        SID_CHECK_LAUNCH();
    } else {
        // df = diag(hs)(-A'Y + lambda)   (fast_nnls.m:57,60)
        SID_TRY(contract(c, A, Y, f16, K, F, P, P, P, w.h, K, 1.f, 0.f, f16 ? SID_PREC_SPLIT : prec, st));
        k_df_init<<<1024, 256, 0, st>>>(w.h, w.hs, b.df, (int)K, K * F, o->lambda, SOLVER_FAST);
        SID_CHECK_LAUNCH();
    }
    SID_TRY(split_gram(c, w, K, f16_operands(w, K, false), st));
    SID_TRY(ensure_gemm_ws(c, K, F, split));
    if (warm_mode == 2) {
        // x = diag(1./hs) W   (fast_nnls.m:72)
        k_x_from<<<1024, 256, 0, st>>>(b.x, W, w.hs, (int)K, K * F);
        SID_CHECK_LAUNCH();
        k_x_out<<<1024, 256, 0, st>>>(b.v, b.x, nullptr, (int)K, K * F);
        SID_CHECK_LAUNCH();
    } else if (warm_mode == 1) {
        SID_TRY(warm_inverse(c, w, K, F, st));
    } else {
        SID_CUDA_TRY(cudaMemsetAsync(b.x, 0, (size_t)(K * F) * 8, st));
    }
    if (warm_mode) {
        // df = df + Q x   (fast_nnls.m:69,73), once in FP32
        SID_TRY(sgemm_tn(w.G, b.v, K, F, K, K, K, b.g, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4), st));
        k_add_g<<<1024, 256, 0, st>>>(b.df, b.g, K * F);
        SID_CHECK_LAUNCH();
    }
    if (total) {
        SID_TRY(total_iterations(c, w, K, F, (int)o->max_iter, st));
        k_fill_h<<<1024, 256, 0, st>>>(X, w.hs, (int)K, K * F);
        SID_CHECK_LAUNCH();
        if (df_out) {
            k_df_out<<<1024, 256, 0, st>>>(b.df, K * F, df_out);
            SID_CHECK_LAUNCH();
        }
        if (iters) {
            k_fill_int<<<64, 256, 0, st>>>(iters, (int)F, (int)o->max_iter + 1);
            SID_CHECK_LAUNCH();
        }
    } else {
        std::vector<float> hs(K);
        SID_CUDA_TRY(cudaMemcpyAsync(hs.data(), w.hs, (size_t)K * 4, cudaMemcpyDeviceToHost, st));
        SID_CUDA_TRY(cudaStreamSynchronize(st));
        double hmax = -INFINITY;
        for (float v : hs) hmax = std::max(hmax, (double)v);
        SID_TRY(iterate(c, w, K, F, SOLVER_FAST, o, hmax, iters, st));
        k_x_out<<<1024, 256, 0, st>>>(X, b.x, w.hs, (int)K, K * F);
        SID_CHECK_LAUNCH();
    }
    if (Q_out) SID_CUDA_TRY(cudaMemcpyAsync(Q_out, w.G, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
    if (h_out) SID_CUDA_TRY(cudaMemcpyAsync(h_out, w.hs, (size_t)K * 4, cudaMemcpyDeviceToDevice, st));
    return ctx_sync(c, st);
}

extern "C" int sid_fast_nnls(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                             const sid_nnls_opts* o, const float* warm_start, float* X, float* Q_out, int prec,
                             int32_t* iters, void* stream)
{
    SID_TRY(nnls_common_checks(c, A, Y, ydtype, P, K, F, o, prec));
    return sid_fast_nnls_ex(c, A, Y, ydtype, P, K, F, o, 0, warm_start ? 2 : 0, warm_start, nullptr, nullptr,
                            nullptr, X, Q_out, nullptr, nullptr, prec, iters, stream);
}
