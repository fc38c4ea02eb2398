// nnls.cu -- batched multi-right-hand-side NNLS (LS_nnls.m, fast_nnls.m).
//
// All F columns iterate in lock step on the GPU.  An iteration is
//   two K x K by K x F contractions (gemm_tc.cu split precision, or FP32 SIMT)
//   + two column kernels (one CTA per column: projected gradient, exact line
//     search, clamp, convergence statistic) + the retirement kernels,
// all reading the iteration number from device memory so that a chunk of
// iterations is captured once in a CUDA graph and replayed.  A retired column
// is frozen (its x is never written again), which is what removing it from x
// does in the reference (LS_nnls.m:158-168, fast_nnls.m:165-179); the host
// polls the number of active columns between graph replays.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "sid_internal.cuh"

namespace sid {
int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st);
int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, int64_t lda,
            int64_t ldb, bool bf16, float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws,
            int64_t ws_elems, int* err, cudaStream_t st);
void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk);
int sgemm_tn(const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, float* C,
             int64_t ldc, float alpha, float beta, float* ws, int64_t ws_elems, cudaStream_t st);
int64_t sgemm_ws_elems(int64_t m, int64_t n, int64_t k);
int split16(const float* src, int64_t rows, int64_t cols, int64_t lds, uint16_t* hi, uint16_t* lo, int64_t ld,
            bool bf16, float scale, cudaStream_t st);
int ctx_sync(sid_ctx* c, cudaStream_t st);

// device counters
struct NnlsCounters {
    int iter;      // LS_nnls: iteration number; fast_nnls: the reference's s
    int active;    // columns still iterating
    int first;     // index of the first active column (LS_nnls k(1) rule)
    int pad;
};

__device__ __forceinline__ float block_sum(float v, float* red)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x < 32) {
        s = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (l == 0) red[0] = s;
    }
    __syncthreads();
    return red[0];
}

__device__ __forceinline__ float block_max(float v, float* red)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    float s = -INFINITY;
    if (threadIdx.x < 32) {
        s = (l < (int)(blockDim.x >> 5)) ? red[l] : -INFINITY;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, off));
        if (l == 0) red[0] = s;
    }
    __syncthreads();
    return red[0];
}

__device__ __forceinline__ void split_bf16(float v, uint16_t* hi, uint16_t* lo)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    *hi = __bfloat16_as_ushort(h);
    *lo = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(h)));
}

__global__ void k_iter_inc(NnlsCounters* c) { c->iter += 1; }

// ---------------------------------------------------------------- LS_nnls --
// d_ = passive .* (-h + G x [- G u / F]), s1 = sum d_^2 (LS_nnls.m:119-122)
__global__ void k_ls_grad_col(const float* __restrict__ gx, const float* __restrict__ h,
                              const float* __restrict__ x, const float* __restrict__ gu, float invF,
                              float* __restrict__ d, uint16_t* __restrict__ dhi, uint16_t* __restrict__ dlo,
                              int64_t ld16, float* __restrict__ s1, const int* __restrict__ active, int K)
{
    __shared__ float red[32];
    const int j = blockIdx.x;
    if (!active[j]) return;
    const int64_t o = (int64_t)j * K;
    float acc = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        float df = gx[o + k] - h[o + k];
        if (gu) df -= gu[k] * invF;
        const float dm = (x[o + k] > 0.f || df < 0.f) ? df : 0.f;
        d[o + k] = dm;
        if (dhi) split_bf16(dm, dhi + (int64_t)j * ld16 + k, dlo + (int64_t)j * ld16 + k);
        acc += dm * dm;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) s1[j] = acc;
}

// alpha = s1 / sum(d_ .* G d_) (NaN -> 0); x <- max(x - alpha d_, 0); on odd
// iterations append log((sum(x - x_old))^2 / sum(x_old^2)) / 2 to the window
// (LS_nnls.m:122-142).
__global__ void k_ls_step_col(float* __restrict__ x, const float* __restrict__ d, const float* __restrict__ gd,
                              const float* __restrict__ gu, float invF, const float* __restrict__ s1,
                              uint16_t* __restrict__ xhi, uint16_t* __restrict__ xlo, int64_t ld16,
                              float* __restrict__ test, int sample, const int* __restrict__ active,
                              const NnlsCounters* __restrict__ cnt, int K, int F)
{
    __shared__ float red[32];
    const int j = blockIdx.x;
    if (!active[j]) return;
    const int64_t o = (int64_t)j * K;
    float s2 = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        float g = gd[o + k];
        if (gu) g -= gu[k] * invF;
        s2 += d[o + k] * g;
    }
    s2 = block_sum(s2, red);
    float alpha = s1[j] / s2;
    if (isnan(alpha)) alpha = 0.f;
    float dsum = 0.f, x2 = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const float xo = x[o + k];
        float xn = xo - d[o + k] * alpha;
        if (xn < 0.f) xn = 0.f;
        x[o + k] = xn;
        if (xhi) split_bf16(xn, xhi + (int64_t)j * ld16 + k, xlo + (int64_t)j * ld16 + k);
        dsum += xn - xo;
        x2 += xo * xo;
    }
    dsum = block_sum(dsum, red);
    x2 = block_sum(x2, red);
    const int it = cnt->iter;
    if (threadIdx.x == 0 && (it & 1)) {
        const int e = (it - 1) / 2;  // window entry number
        test[(int64_t)(e % sample) * F + j] = logf(dsum * dsum / x2) * 0.5f;
    }
}

// Linear fit of the last `sample` window entries against [1 3 5 ...; 1 1 1]:
// k = Xi * test (Xi = inv(X'X) X', LS_nnls.m:116-117), residual sum |X k - test|.
__device__ void window_fit(const float* test, int sample, int F, int j, int e_last, const float* xi, float* k1,
                           float* k2, float* resid, float* tend)
{
    // entries e_last-sample+1 .. e_last in chronological order
    float a = 0.f, b = 0.f;
    for (int t = 0; t < sample; ++t) {
        const int e = e_last - sample + 1 + t;
        const float v = test[(int64_t)(e % sample) * F + j];
        a += xi[t] * v;
        b += xi[sample + t] * v;
    }
    float r = 0.f;
    for (int t = 0; t < sample; ++t) {
        const int e = e_last - sample + 1 + t;
        const float v = test[(int64_t)(e % sample) * F + j];
        r += fabsf((float)(2 * t + 1) * a + b - v);
    }
    *k1 = a;
    *k2 = b;
    *resid = r;
    *tend = test[(int64_t)(e_last % sample) * F + j];
}

// per-column fit, then the first active column (single block)
__global__ void k_ls_fit(const float* __restrict__ test, int sample, const float* __restrict__ xi,
                         const int* __restrict__ active, float* __restrict__ fit, const NnlsCounters* __restrict__ cnt,
                         int F, int max_iter, int use_std)
{
    const int it = cnt->iter;
    if (it > max_iter || use_std || !(it & 1) || it <= 2 * sample) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!active[j]) continue;
        float k1, k2, r, te;
        window_fit(test, sample, F, j, (it - 1) / 2, xi, &k1, &k2, &r, &te);
        fit[j] = k1;
        fit[F + j] = r;
        fit[2 * F + j] = te;
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

// Retirement (LS_nnls.m:132-152): all columns after max_iter; otherwise, on odd
// iterations past 2*sample, columns with
//   exp(t_end)/(1 - exp(k1 of the first active column)) < tol
//   & sum|fit residual| < tol_*sample & exp(k1) < 1,  or t_end == -inf.
__global__ void k_ls_retire(int* __restrict__ active, const float* __restrict__ fit, NnlsCounters* cnt,
                            int32_t* __restrict__ iters, int F, int sample, float tol, float tol_, int max_iter,
                            int use_std)
{
    const int it = cnt->iter;
    const bool all = it > max_iter;
    if (!all && (use_std || !(it & 1) || it <= 2 * sample)) return;
    const float k1first = (cnt->first < F) ? fit[cnt->first] : 0.f;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!active[j]) continue;
        bool ids = all;
        if (!all) {
            const float k1 = fit[j], r = fit[F + j], te = fit[2 * F + j];
            const bool c1 = expf(te) / (1.f - expf(k1first)) < tol;
            const bool c2 = r < tol_ * (float)sample;
            const bool c3 = expf(k1) < 1.f;
            ids = (c1 && c2 && c3) || (te == -INFINITY);
        }
        if (ids) {
            active[j] = 0;
            if (iters) iters[j] = it;
            atomicSub(&cnt->active, 1);
        }
    }
}

// h = A'Y - lambda (in place on h)
__global__ void k_add_scalar(float* __restrict__ h, int64_t n, float v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        h[i] += v;
}

// u = sum over active columns of v (K-vector)
__global__ void k_rowsum_active(const float* __restrict__ v, const int* __restrict__ active, int K, int F,
                                float* __restrict__ u)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int j = 0; j < F; ++j)
            if (active[j]) s += v[(int64_t)j * K + k];
        u[k] = s;
    }
}

// y(p) = sum over frames of Y(p, f) (FP32 or FP16 movie)
__global__ void k_movie_rowsum(const void* __restrict__ Y, int f16, int64_t P, int64_t F, float* __restrict__ out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int64_t f = 0; f < F; ++f)
            s += f16 ? __half2float(static_cast<const __half*>(Y)[p + P * f]) : static_cast<const float*>(Y)[p + P * f];
        out[p] = s;
    }
}

// h(:, j) -= w / F for every column
__global__ void k_sub_colvec(float* __restrict__ h, const float* __restrict__ w, int K, int F, float invF)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        h[i] -= w[i % K] * invF;
}

__global__ void k_split_cols(const float* __restrict__ x, int K, int F, uint16_t* __restrict__ hi,
                             uint16_t* __restrict__ lo, int64_t ld16)
{
    const int64_t n = (int64_t)ld16 * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = i % ld16, j = i / ld16;
        const float v = (k < K) ? x[j * K + k] : 0.f;
        split_bf16(v, hi + i, lo + i);
    }
}

// ------------------------------------------------------------ fast_nnls ---
// Q = G ./ sqrt(diag G diag G'), hs = 1 ./ sqrt(diag G)   (fast_nnls.m:54-56)
__global__ void k_normalise_gram(float* __restrict__ G, float* __restrict__ hs, int K)
{
    const int64_t n = (int64_t)K * K;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % K), c = (int)(i / K);
        const float dr = G[(int64_t)r * K + r], dc = G[(int64_t)c * K + c];
        G[i] = G[i] / sqrtf(dr * dc);
    }
}

__global__ void k_diag_rsqrt(const float* __restrict__ G, float* __restrict__ hs, int K)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
        hs[k] = 1.f / sqrtf(G[(int64_t)k * K + k]);
}

// df = diag(hs) * (-A'Y + lambda)  (fast_nnls.m:57) applied in place to h = A'Y
__global__ void k_fast_df0(float* __restrict__ df, const float* __restrict__ hs, int K, int F, float lambda)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        df[i] = hs[i % K] * (-df[i] + lambda);
}

// x = diag(1 ./ hs) * W (fast_nnls.m:72)
__global__ void k_fast_warm(float* __restrict__ x, const float* __restrict__ W, const float* __restrict__ hs, int K,
                            int F)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = W[i] / hs[i % K];
}

__global__ void k_axpy(float* __restrict__ y, const float* __restrict__ x, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] += x[i];
}

// passive = (x > 0) | (df < 0); d_ = df .* passive; s1 = sum d_^2; anyp = any(passive)
__global__ void k_fast_mask_col(const float* __restrict__ x, const float* __restrict__ df, float* __restrict__ d,
                                uint16_t* __restrict__ dhi, uint16_t* __restrict__ dlo, int64_t ld16,
                                float* __restrict__ s1, float* __restrict__ anyp, float* __restrict__ xmax,
                                const int* __restrict__ active, int K)
{
    __shared__ float red[32];
    const int j = blockIdx.x;
    if (!active[j]) return;
    const int64_t o = (int64_t)j * K;
    float acc = 0.f, np = 0.f, mx = -INFINITY;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const float xv = x[o + k], dv = df[o + k];
        const bool p = xv > 0.f || dv < 0.f;
        const float dm = p ? dv : 0.f;
        d[o + k] = dm;
        if (dhi) split_bf16(dm, dhi + (int64_t)j * ld16 + k, dlo + (int64_t)j * ld16 + k);
        acc += dm * dm;
        np += p ? 1.f : 0.f;
        mx = fmaxf(mx, xv);
    }
    acc = block_sum(acc, red);
    np = block_sum(np, red);
    mx = block_max(mx, red);
    if (threadIdx.x == 0) {
        s1[j] = acc;
        anyp[j] = np;
        xmax[j] = mx;
    }
}

// alpha = s1 / sum(d_ .* Q d_); x_ = max(x - alpha d_, 0); step = x_ - x (kept in
// d for the next contraction); on odd s the log-l1 (tol_p 1) or log-l2 (tol_p 2)
// step norm is appended to the window (fast_nnls.m:119-145).
__global__ void k_fast_step_col(float* __restrict__ x, float* __restrict__ d, const float* __restrict__ qd,
                                const float* __restrict__ s1, uint16_t* __restrict__ shi, uint16_t* __restrict__ slo,
                                int64_t ld16, float* __restrict__ test, int sample, int tol_p,
                                const int* __restrict__ active, const NnlsCounters* __restrict__ cnt, int K, int F)
{
    __shared__ float red[32];
    const int j = blockIdx.x;
    if (!active[j]) return;
    const int64_t o = (int64_t)j * K;
    float s2 = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) s2 += d[o + k] * qd[o + k];
    s2 = block_sum(s2, red);
    float alpha = s1[j] / s2;
    if (isnan(alpha)) alpha = 0.f;
    float nrm = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const float xo = x[o + k];
        float xn = xo - d[o + k] * alpha;
        if (xn < 0.f) xn = 0.f;
        const float stp = xn - xo;
        x[o + k] = xn;
        d[o + k] = stp;
        if (shi) split_bf16(stp, shi + (int64_t)j * ld16 + k, slo + (int64_t)j * ld16 + k);
        nrm += (tol_p == 2) ? stp * stp : fabsf(stp);
    }
    nrm = block_sum(nrm, red);
    const int s = cnt->iter;
    if (threadIdx.x == 0 && (s & 1)) {
        const int e = (s - 3) / 2;  // s = 3, 5, 7, ... -> entries 0, 1, 2, ...
        test[(int64_t)(e % sample) * F + j] = (tol_p == 2) ? logf(sqrtf(nrm)) : logf(nrm);
    }
}

// Retirement (fast_nnls.m:146-179): on odd s past 2*sample, columns with no
// passive entry, or  h_max*exp(t_end)/(1-exp(k1)) < tol*K*max(x)
//   & sum|fit residual| < tol_*sample & exp(k1) < 1;  every column once s > max_iter.
__global__ void k_fast_retire(int* __restrict__ active, const float* __restrict__ test, int sample,
                              const float* __restrict__ xi, const float* __restrict__ anyp,
                              const float* __restrict__ xmax, float hmax, NnlsCounters* cnt,
                              int32_t* __restrict__ iters, int K, int F, float tol, float tol_, int max_iter)
{
    const int s = cnt->iter;
    const bool all = s > max_iter;
    const bool check = (s & 1) && s > 2 * sample;
    if (!all && !check) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < F; j += gridDim.x * blockDim.x) {
        if (!active[j]) continue;
        bool ids = all;
        if (!all) {
            float k1, k2, r, te;
            window_fit(test, sample, F, j, (s - 3) / 2, xi, &k1, &k2, &r, &te);
            const bool nop = anyp[j] == 0.f;
            const bool c1 = hmax * expf(te) / (1.f - expf(k1)) < tol * (float)K * xmax[j];
            const bool c2 = r < tol_ * (float)sample;
            const bool c3 = expf(k1) < 1.f;
            ids = nop || (c1 && c2 && c3);
        }
        if (ids) {
            active[j] = 0;
            if (iters) iters[j] = s;
            atomicSub(&cnt->active, 1);
        }
    }
}

// xx = diag(hs) * x
__global__ void k_scale_rows(float* __restrict__ X, const float* __restrict__ x, const float* __restrict__ hs, int K,
                             int F)
{
    const int64_t n = (int64_t)K * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        X[i] = hs[i % K] * x[i];
}

__global__ void k_fill_int(int* __restrict__ a, int n, int v)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

// ------------------------------------------------------------ host driver --
struct NnlsBufs {
    float *h, *x, *d, *g, *test, *s1, *fit, *xi, *gu, *u, *anyp, *xmax, *hs, *Gw;
    int* active;
    NnlsCounters* cnt;
    uint16_t *Ghi, *Glo, *xhi, *xlo, *dhi, *dlo;
    int64_t ld16;
};

static std::vector<float> fit_matrix(int sample)
{
    // Xi = inv(X'X) X' for X = [1 3 5 ... (2*sample-1); 1 ... 1]' (2 x sample, row-major)
    double s11 = 0, s12 = 0, s22 = sample;
    for (int t = 0; t < sample; ++t) {
        const double a = 2.0 * t + 1.0;
        s11 += a * a;
        s12 += a;
    }
    const double det = s11 * s22 - s12 * s12;
    const double i11 = s22 / det, i12 = -s12 / det, i22 = s11 / det;
    std::vector<float> xi(2 * sample);
    for (int t = 0; t < sample; ++t) {
        const double a = 2.0 * t + 1.0;
        xi[t] = (float)(i11 * a + i12);
        xi[sample + t] = (float)(i12 * a + i22);
    }
    return xi;
}

static int alloc_nnls(sid_ctx* c, int64_t K, int64_t F, int sample, bool split, NnlsBufs* b)
{
    const int64_t KF = K * F;
    const int64_t ld16 = cdiv(K, 8) * 8;
    DBuf* nn = c->nn;
    SID_TRY(nn[0].alloc(KF * 4));   // h / df
    SID_TRY(nn[1].alloc(KF * 4));   // x
    SID_TRY(nn[2].alloc(KF * 4));   // d
    SID_TRY(nn[3].alloc(KF * 4));   // G*x / G*d
    SID_TRY(nn[4].alloc((size_t)sample * F * 4));
    SID_TRY(nn[5].alloc((size_t)(8 * F + 4 * K + 2 * sample + 64) * 4));
    SID_TRY(nn[6].alloc((size_t)F * 4 + sizeof(NnlsCounters)));
    SID_TRY(nn[7].alloc((size_t)K * K * 4));  // G workspace
    if (split) {
        SID_TRY(nn[8].alloc((size_t)ld16 * K * 2));
        SID_TRY(nn[9].alloc((size_t)ld16 * K * 2));
        SID_TRY(nn[10].alloc((size_t)ld16 * F * 2));
        SID_TRY(nn[11].alloc((size_t)ld16 * F * 2));
        SID_TRY(nn[12].alloc((size_t)ld16 * F * 2));
        SID_TRY(nn[13].alloc((size_t)ld16 * F * 2));
    }
    b->h = nn[0].as<float>();
    b->x = nn[1].as<float>();
    b->d = nn[2].as<float>();
    b->g = nn[3].as<float>();
    b->test = nn[4].as<float>();
    float* sc = nn[5].as<float>();
    b->s1 = sc;
    b->fit = sc + F;          // 3F
    b->anyp = sc + 4 * F;
    b->xmax = sc + 5 * F;
    b->xi = sc + 8 * F;       // 2*sample
    b->gu = b->xi + 2 * sample;  // K
    b->u = b->gu + K;            // K
    b->hs = b->u + K;            // K
    b->active = reinterpret_cast<int*>(nn[6].p);
    b->cnt = reinterpret_cast<NnlsCounters*>(nn[6].as<uint8_t>() + cdiv(F * 4, 16) * 16);
    b->Gw = nn[7].as<float>();
    b->ld16 = ld16;
    b->Ghi = split ? nn[8].as<uint16_t>() : nullptr;
    b->Glo = split ? nn[9].as<uint16_t>() : nullptr;
    b->xhi = split ? nn[10].as<uint16_t>() : nullptr;
    b->xlo = split ? nn[11].as<uint16_t>() : nullptr;
    b->dhi = split ? nn[12].as<uint16_t>() : nullptr;
    b->dlo = split ? nn[13].as<uint16_t>() : nullptr;
    return SID_OK;
}

// out (K x F) = G * v, with G symmetric, at the solver precision.
static int gmul(sid_ctx* c, const NnlsBufs& b, const float* G, const float* v, const uint16_t* vhi,
                const uint16_t* vlo, int64_t K, int64_t F, float* out, bool split, cudaStream_t st)
{
    if (!split) {
        return sgemm_tn(G, v, K, F, K, K, K, out, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4), st);
    }
    const void* As[3] = {b.Ghi, b.Ghi, b.Glo};
    const void* Bs[3] = {vhi, vlo, vhi};
    int bn = 0, sk = 0;
    gemm_autotune((int)K, (int)F, (int)cdiv(K, 64), &bn, &sk);
    return gemm_tn(As, Bs, 3, K, F, K, b.ld16, b.ld16, true, out, K, 1.f, 0.f, bn, sk, c->ws.as<float>(),
                   (int64_t)(c->ws.bytes / 4), c->errflag.as<int>(), st);
}

static int ensure_gemm_ws(sid_ctx* c, int64_t K, int64_t F, bool split)
{
    int64_t need = sgemm_ws_elems(K, F, K);
    if (split) {
        int bn = 0, sk = 0;
        gemm_autotune((int)K, (int)F, (int)cdiv(K, 64), &bn, &sk);
        need = std::max<int64_t>(need, (int64_t)sk * K * F);
    }
    return c->ws.alloc((size_t)need * 4);
}

static const int kChunk = 16;  // iterations per captured graph

template <class Body>
static int run_iterations(sid_ctx* c, const NnlsBufs& b, int max_iter, Body body, cudaStream_t st)
{
    // Capture kChunk iterations into a graph, replay until no column is active.
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
    const int sample = (int)o->sample;
    NnlsBufs b;
    SID_TRY(alloc_nnls(c, K, F, sample, split, &b));
    const bool f16 = ydtype == SID_DTYPE_F16;
    // h = A'Y - lambda   (LS_nnls.m:76)
    SID_TRY(contract(c, A, Y, f16, K, F, P, P, P, b.h, K, 1.f, 0.f, f16 ? SID_PREC_SPLIT : prec, st));
    if (o->lambda != 0.0) {
        k_add_scalar<<<1024, 256, 0, st>>>(b.h, K * F, (float)-o->lambda);
        SID_CHECK_LAUNCH();
    }
    // G = A'A   (LS_nnls.m:82)
    float* Gp = g_given ? G : (G ? G : b.Gw);
    if (!g_given) SID_TRY(contract(c, A, A, false, K, K, P, P, P, Gp, K, 1.f, 0.f, prec, st));
    if (o->use_std) {
        // h = h - A' sum(Y,2) / F   (LS_nnls.m:104)
        DBuf ys;
        SID_TRY(ys.alloc((size_t)P * 4));
        k_movie_rowsum<<<1024, 256, 0, st>>>(Y, f16 ? 1 : 0, P, F, ys.as<float>());
        SID_CHECK_LAUNCH();
        SID_TRY(c->ws.alloc((size_t)std::max<int64_t>(sgemm_ws_elems(K, 1, P), 1) * 4));
        SID_TRY(sgemm_tn(A, ys.as<float>(), K, 1, P, P, P, b.u, K, 1.f, 0.f, c->ws.as<float>(),
                         (int64_t)(c->ws.bytes / 4), st));
        k_sub_colvec<<<1024, 256, 0, st>>>(b.h, b.u, (int)K, (int)F, 1.f / (float)F);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaStreamSynchronize(st));
        ys.release();
    }
    SID_TRY(ensure_gemm_ws(c, K, F, split));
    if (x_given) {
        SID_CUDA_TRY(cudaMemcpyAsync(b.x, X, (size_t)(K * F) * 4, cudaMemcpyDeviceToDevice, st));
    } else {
        SID_CUDA_TRY(cudaMemsetAsync(b.x, 0, (size_t)(K * F) * 4, st));
    }
    if (split) {
        SID_TRY(split16(Gp, K, K, K, b.Ghi, b.Glo, b.ld16, true, 1.f, st));
        k_split_cols<<<1024, 256, 0, st>>>(b.x, (int)K, (int)F, b.xhi, b.xlo, b.ld16);
        SID_CHECK_LAUNCH();
    }
    const std::vector<float> xi = fit_matrix(sample);
    SID_CUDA_TRY(cudaMemcpyAsync(b.xi, xi.data(), xi.size() * 4, cudaMemcpyHostToDevice, st));
    k_fill_int<<<64, 256, 0, st>>>(b.active, (int)F, 1);
    SID_CHECK_LAUNCH();
    NnlsCounters h0{0, (int)F, 0, 0};
    SID_CUDA_TRY(cudaMemcpyAsync(b.cnt, &h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));

    // one contraction outside the capture configures the kernels (its result
    // is overwritten by the first iteration)
    SID_TRY(gmul(c, b, Gp, b.x, b.xhi, b.xlo, K, F, b.g, split, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    const float invF = 1.f / (float)F;
    const int use_std = o->use_std ? 1 : 0;
    const int max_iter = (int)o->max_iter;
    auto body = [&](cudaStream_t s) -> int {
        k_iter_inc<<<1, 1, 0, s>>>(b.cnt);
        SID_CHECK_LAUNCH();
        // df = -h + G(x)
        SID_TRY(gmul(c, b, Gp, b.x, b.xhi, b.xlo, K, F, b.g, split, s));
        const float* gu = nullptr;
        if (use_std) {
            k_rowsum_active<<<cdiv(K, 256), 256, 0, s>>>(b.x, b.active, (int)K, (int)F, b.u);
            SID_CHECK_LAUNCH();
            SID_TRY(sgemm_tn(Gp, b.u, K, 1, K, K, K, b.gu, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4), s));
            gu = b.gu;
        }
        k_ls_grad_col<<<(unsigned)F, 256, 0, s>>>(b.g, b.h, b.x, gu, invF, b.d, b.dhi, b.dlo, b.ld16, b.s1, b.active,
                                                  (int)K);
        SID_CHECK_LAUNCH();
        // G(d_) for the exact line search
        SID_TRY(gmul(c, b, Gp, b.d, b.dhi, b.dlo, K, F, b.g, split, s));
        if (use_std) {
            k_rowsum_active<<<cdiv(K, 256), 256, 0, s>>>(b.d, b.active, (int)K, (int)F, b.u);
            SID_CHECK_LAUNCH();
            SID_TRY(sgemm_tn(Gp, b.u, K, 1, K, K, K, b.gu, K, 1.f, 0.f, c->ws.as<float>(), (int64_t)(c->ws.bytes / 4), s));
        }
        k_ls_step_col<<<(unsigned)F, 256, 0, s>>>(b.x, b.d, b.g, gu, invF, b.s1, b.xhi, b.xlo, b.ld16, b.test,
                                                  sample, b.active, b.cnt, (int)K, (int)F);
        SID_CHECK_LAUNCH();
        k_ls_fit<<<cdiv(F, 256), 256, 0, s>>>(b.test, sample, b.xi, b.active, b.fit, b.cnt, (int)F, max_iter,
                                               use_std);
        SID_CHECK_LAUNCH();
        k_first_active<<<1, 1024, 0, s>>>(b.active, b.cnt, (int)F);
        SID_CHECK_LAUNCH();
        k_ls_retire<<<cdiv(F, 256), 256, 0, s>>>(b.active, b.fit, b.cnt, iters, (int)F, sample, (float)o->tol,
                                                  (float)o->tol_, max_iter, use_std);
        SID_CHECK_LAUNCH();
        return SID_OK;
    };
    SID_TRY(run_iterations(c, b, max_iter, body, st));
    SID_CUDA_TRY(cudaMemcpyAsync(X, b.x, (size_t)(K * F) * 4, cudaMemcpyDeviceToDevice, st));
    if (G && !g_given && Gp != G) SID_CUDA_TRY(cudaMemcpyAsync(G, Gp, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
    return ctx_sync(c, st);
}

extern "C" int sid_fast_nnls(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                             const sid_nnls_opts* o, const float* warm_start, float* X, float* Q_out, int prec,
                             int32_t* iters, void* stream)
{
    SID_TRY(nnls_common_checks(c, A, Y, ydtype, P, K, F, o, prec));
    SID_REQUIRE(X, "fast_nnls: X is NULL");
    SID_REQUIRE(o->tol_p == 1 || o->tol_p == 2, "fast_nnls: tol_p must be 1 or 2");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool split = prec == SID_PREC_SPLIT;
    const int sample = (int)o->sample;
    NnlsBufs b;
    SID_TRY(alloc_nnls(c, K, F, sample, split, &b));
    const bool f16 = ydtype == SID_DTYPE_F16;
    // Q = A'A normalised, hs = 1./sqrt(diag), df = diag(hs)(-A'Y + lambda)   (fast_nnls.m:53-57)
    float* Q = b.Gw;
    SID_TRY(contract(c, A, A, false, K, K, P, P, P, Q, K, 1.f, 0.f, prec, st));
    k_diag_rsqrt<<<cdiv(K, 256), 256, 0, st>>>(Q, b.hs, (int)K);
    SID_CHECK_LAUNCH();
    k_normalise_gram<<<1024, 256, 0, st>>>(Q, b.hs, (int)K);
    SID_CHECK_LAUNCH();
    SID_TRY(contract(c, A, Y, f16, K, F, P, P, P, b.h, K, 1.f, 0.f, f16 ? SID_PREC_SPLIT : prec, st));
    k_fast_df0<<<1024, 256, 0, st>>>(b.h, b.hs, (int)K, (int)F, (float)o->lambda);
    SID_CHECK_LAUNCH();
    SID_TRY(ensure_gemm_ws(c, K, F, split));
    if (split) SID_TRY(split16(Q, K, K, K, b.Ghi, b.Glo, b.ld16, true, 1.f, st));
    float* df = b.h;
    if (warm_start) {
        // x = diag(1./hs) W; df = df + Q x   (fast_nnls.m:72-73)
        k_fast_warm<<<1024, 256, 0, st>>>(b.x, warm_start, b.hs, (int)K, (int)F);
        SID_CHECK_LAUNCH();
        if (split) {
            k_split_cols<<<1024, 256, 0, st>>>(b.x, (int)K, (int)F, b.xhi, b.xlo, b.ld16);
            SID_CHECK_LAUNCH();
        }
        SID_TRY(gmul(c, b, Q, b.x, b.xhi, b.xlo, K, F, b.g, split, st));
        k_axpy<<<1024, 256, 0, st>>>(df, b.g, K * F);
        SID_CHECK_LAUNCH();
    } else {
        SID_CUDA_TRY(cudaMemsetAsync(b.x, 0, (size_t)(K * F) * 4, st));
    }
    const std::vector<float> xi = fit_matrix(sample);
    SID_CUDA_TRY(cudaMemcpyAsync(b.xi, xi.data(), xi.size() * 4, cudaMemcpyHostToDevice, st));
    k_fill_int<<<64, 256, 0, st>>>(b.active, (int)F, 1);
    SID_CHECK_LAUNCH();
    NnlsCounters h0{1, (int)F, 0, 0};  // the reference starts at s = 1
    SID_CUDA_TRY(cudaMemcpyAsync(b.cnt, &h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    // h_ = max(hs) (host copy once)
    std::vector<float> hs(K);
    SID_CUDA_TRY(cudaMemcpyAsync(hs.data(), b.hs, (size_t)K * 4, cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    float hmax = -INFINITY;
    for (float v : hs) hmax = std::max(hmax, v);
    const int max_iter = (int)o->max_iter;
    SID_TRY(gmul(c, b, Q, b.x, b.xhi, b.xlo, K, F, b.g, split, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    // The retirement test needs the statistic of the current step, so the
    // iteration is: mask -> Q d_ -> step (+ statistic) -> retire -> Q step -> df update.
    auto body2 = [&](cudaStream_t s) -> int {
        k_iter_inc<<<1, 1, 0, s>>>(b.cnt);
        SID_CHECK_LAUNCH();
        k_fast_mask_col<<<(unsigned)F, 256, 0, s>>>(b.x, df, b.d, b.dhi, b.dlo, b.ld16, b.s1, b.anyp, b.xmax,
                                                    b.active, (int)K);
        SID_CHECK_LAUNCH();
        SID_TRY(gmul(c, b, Q, b.d, b.dhi, b.dlo, K, F, b.g, split, s));
        k_fast_step_col<<<(unsigned)F, 256, 0, s>>>(b.x, b.d, b.g, b.s1, b.dhi, b.dlo, b.ld16, b.test, sample,
                                                    (int)o->tol_p, b.active, b.cnt, (int)K, (int)F);
        SID_CHECK_LAUNCH();
        // df = df + Q (x_ - x)   (fast_nnls.m:153), for the columns still active
        SID_TRY(gmul(c, b, Q, b.d, b.dhi, b.dlo, K, F, b.g, split, s));
        k_axpy<<<1024, 256, 0, s>>>(df, b.g, K * F);
        SID_CHECK_LAUNCH();
        k_fast_retire<<<cdiv(F, 256), 256, 0, s>>>(b.active, b.test, sample, b.xi, b.anyp, b.xmax, hmax, b.cnt,
                                                    iters, (int)K, (int)F, (float)o->tol, (float)o->tol_, max_iter);
        SID_CHECK_LAUNCH();
        return SID_OK;
    };
    SID_TRY(run_iterations(c, b, max_iter, body2, st));
    k_scale_rows<<<1024, 256, 0, st>>>(X, b.x, b.hs, (int)K, (int)F);
    SID_CHECK_LAUNCH();
    if (Q_out) SID_CUDA_TRY(cudaMemcpyAsync(Q_out, Q, (size_t)(K * K) * 4, cudaMemcpyDeviceToDevice, st));
    return ctx_sync(c, st);
}
