// postproc.cu -- post-processing around the demixing loop:
//   merge_filters.m  merge components whose templates overlap by more than a
//                    third and whose traces correlate above opts.limit
//   SNR_order.m      order the traces by a peak-to-noise ratio
//
// merge_filters: the K x K trace correlation (corrcoef of the rows) is an FP32
// Gram of the centred traces; the template overlap template * template' is a
// Gram of a 0/1 matrix (K_t x P, P ~ 1e6 pixels), exact on the tensor cores:
// 0/1 are exact in BF16 and the counts (< 2^24) exact in the FP32 accumulator.
// The rows of both matrices are strided (MATLAB stores them K x F and K_t x P),
// so each is first transposed into the contraction's operand layout.  The merge
// decisions (merge_filters.m:22-37) are a sequential loop on K x K host data; the
// row operations they imply act on each pixel's column independently, so one
// thread per pixel replays the whole ordered list.
//
// SNR_order: zeroing DFT bins 1..6 (and their mirrors) of [trace flip(trace)]
// and inverting (SNR_order.m:14-18) subtracts the trace's projection on those
// six modes; the kernel computes the six coefficients directly (FP64 sums of
// length 2F), then zscore, MATLAB's moving-average smooth and the ratio, one
// CTA per trace.
#include <algorithm>
#include <cmath>
#include <cuda_bf16.h>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
            float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws, int64_t ws_elems, int* err,
            cudaStream_t st);
void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk);
int sgemm_tn(const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, float* C,
             int64_t ldc, float alpha, float beta, float* ws, int64_t ws_elems, cudaStream_t st);
int64_t sgemm_ws_elems(int64_t m, int64_t n, int64_t k);
int64_t blk16_elems(int64_t k, int64_t rows);
int ctx_sync(sid_ctx* c, cudaStream_t st);

namespace {

constexpr int kT = 256;

// Xc (F x K, column-major) = ts (K x F) - row means, transposed.  One CTA per
// 32-row block: row means first, then a 32 x 32-tiled transpose.
__global__ void __launch_bounds__(kT) k_center_transpose(const float* __restrict__ ts, int64_t K, int64_t F,
                                                         float* __restrict__ xc)
{
    __shared__ double red[32][9];
    __shared__ float mean[32];
    __shared__ float tile[32][33];
    const int k0 = blockIdx.x * 32;
    const int r = threadIdx.x & 31, w = threadIdx.x >> 5;  // 8 warps split the frames
    double acc = 0.0;
    if (k0 + r < K)
        for (int64_t f = w; f < F; f += 8) acc += ts[(k0 + r) + K * f];
    red[r][w] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int q = 0; q < 8; ++q) s += red[threadIdx.x][q];
        mean[threadIdx.x] = (float)(s / (double)F);
    }
    __syncthreads();
    for (int64_t f0 = 0; f0 < F; f0 += 32) {
        for (int q = w; q < 32; q += 8) {  // read: rows k0 + r, frame f0 + q
            const int64_t f = f0 + q;
            tile[q][r] = (k0 + r < K && f < F) ? ts[(k0 + r) + K * f] - mean[r] : 0.f;
        }
        __syncthreads();
        for (int q = w; q < 32; q += 8) {  // write: column k0 + q of xc, frame f0 + r
            const int64_t f = f0 + r;
            if (k0 + q < K && f < F) xc[f + F * (k0 + q)] = tile[r][q];
        }
        __syncthreads();
    }
}

// 0/1 template (Kt x P, column-major) -> BF16 K-blocked operand [p/64][row][64].
__global__ void __launch_bounds__(kT) k_template_blk(const float* __restrict__ t, int64_t Kt, int64_t P,
                                                     uint16_t* __restrict__ dst)
{
    __shared__ uint16_t tile[64][66];
    const int64_t p0 = (int64_t)blockIdx.x * 64;
    const int64_t r0 = (int64_t)blockIdx.y * 64;
    for (int e = threadIdx.x; e < 64 * 64; e += kT) {
        const int pp = e >> 6, rr = e & 63;  // read along rows (contiguous)
        const int64_t p = p0 + pp, r = r0 + rr;
        const float v = (p < P && r < Kt) ? t[r + Kt * p] : 0.f;
        tile[rr][pp] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
    __syncthreads();
    const int64_t kb = p0 / 64;
    for (int e = threadIdx.x; e < 64 * 64; e += kT) {
        const int rr = e >> 6, pp = e & 63;  // write along pixels (contiguous)
        const int64_t r = r0 + rr;
        if (r < Kt) dst[(kb * Kt + r) * 64 + pp] = tile[rr][pp];
    }
}

// Replay the merges on every pixel's column: op o merges rows list[beg[o]..beg[o+1])
// into row dst[o] (OR) and zeroes them (merge_filters.m:33-36).  Then flag the
// non-empty rows.
__global__ void k_apply_merges(float* __restrict__ t, int64_t Kt, int64_t P, const int* __restrict__ dst,
                               const int* __restrict__ beg, const int* __restrict__ list, int nops,
                               int* __restrict__ nonzero)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        float* col = t + Kt * p;
        for (int o = 0; o < nops; ++o) {
            float s = col[dst[o]];
            for (int q = beg[o]; q < beg[o + 1]; ++q) s += col[list[q]];
            col[dst[o]] = s > 0.f ? 1.f : 0.f;
            for (int q = beg[o]; q < beg[o + 1]; ++q) col[list[q]] = 0.f;
        }
        for (int64_t r = 0; r < Kt; ++r)
            if (col[r] > 0.f) nonzero[r] = 1;
    }
}

// MATLAB smooth(y, span): centred moving average with the window shrunk to
// stay symmetric near the ends (span made odd); value at i.
__device__ __forceinline__ double smooth_at(const double* y, int n, int span, int i)
{
    if (span % 2 == 0) span -= 1;
    const int h = min(min(i, n - 1 - i), span / 2);
    double s = 0.0;
    for (int j = i - h; j <= i + h; ++j) s += y[j];
    return s / (double)(2 * h + 1);
}

// One CTA per trace (SNR_order.m:13-24): pp[k] = (max - min of smooth(z, 5)) / std(smooth(z, 8) - z)
// with z = zscore of the trace high-passed by removing DFT bins 1..6 of [x flip(x)].
__global__ void __launch_bounds__(kT) k_snr(const float* __restrict__ traces, int64_t K, int F,
                                            double* __restrict__ work, double* __restrict__ pp)
{
    __shared__ double red[2 * kT];
    __shared__ double coef[12];
    const int k = blockIdx.x;
    double* y = work + (int64_t)blockIdx.x * 2 * F;  // z, then smooth(z, 8) - z
    double* d = y + F;
    const int n2 = 2 * F;
    // bin coefficients X_m = sum_n x_ext(n) e^{-2 pi i m n / 2F}, m = 1..6
    for (int m = 1; m <= 6; ++m) {
        double re = 0.0, im = 0.0;
        for (int n = threadIdx.x; n < n2; n += kT) {
            const double x = traces[k + K * (int64_t)(n < F ? n : n2 - 1 - n)];
            double sn, cs;
            sincospi(2.0 * (double)((int64_t)m * n % n2) / (double)n2, &sn, &cs);
            re += x * cs;
            im -= x * sn;
        }
        red[threadIdx.x] = re;
        red[kT + threadIdx.x] = im;
        __syncthreads();
        for (int s = kT / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                red[threadIdx.x] += red[threadIdx.x + s];
                red[kT + threadIdx.x] += red[kT + threadIdx.x + s];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            coef[2 * (m - 1)] = red[0];
            coef[2 * (m - 1) + 1] = red[kT];
        }
        __syncthreads();
    }
    // x - (1/2F) sum_m (X_m e^{+i..} + conj(X_m) e^{-i..}) for the first F samples
    for (int n = threadIdx.x; n < F; n += kT) {
        double v = traces[k + K * (int64_t)n];
        for (int m = 1; m <= 6; ++m) {
            double sn, cs;
            sincospi(2.0 * (double)((int64_t)m * n % n2) / (double)n2, &sn, &cs);
            v -= 2.0 * (coef[2 * (m - 1)] * cs - coef[2 * (m - 1) + 1] * sn) / (double)n2;
        }
        y[n] = v;
    }
    __syncthreads();
    // zscore (sample standard deviation)
    auto block_sum = [&](double v) {
        red[threadIdx.x] = v;
        __syncthreads();
        for (int s = kT / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        const double r = red[0];
        __syncthreads();
        return r;
    };
    double s = 0.0;
    for (int n = threadIdx.x; n < F; n += kT) s += y[n];
    const double mu = block_sum(s) / F;
    s = 0.0;
    for (int n = threadIdx.x; n < F; n += kT) s += (y[n] - mu) * (y[n] - mu);
    const double sd = sqrt(block_sum(s) / (F - 1));
    for (int n = threadIdx.x; n < F; n += kT) y[n] = (y[n] - mu) / sd;
    __syncthreads();
    // noise: std(smooth(z, 8) - z); peak: max - min of smooth(z) (span 5)
    double lo = 1e300, hi = -1e300;
    s = 0.0;
    for (int n = threadIdx.x; n < F; n += kT) {
        const double dv = smooth_at(y, F, 8, n) - y[n];
        d[n] = dv;
        s += dv;
        const double sm = smooth_at(y, F, 5, n);
        lo = fmin(lo, sm);
        hi = fmax(hi, sm);
    }
    const double md = block_sum(s) / F;
    s = 0.0;
    for (int n = threadIdx.x; n < F; n += kT) s += (d[n] - md) * (d[n] - md);
    const double sn = sqrt(block_sum(s) / (F - 1));
    red[threadIdx.x] = hi;
    __syncthreads();
    for (int st = kT / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
        __syncthreads();
    }
    const double mx = red[0];
    __syncthreads();
    red[threadIdx.x] = lo;
    __syncthreads();
    for (int st = kT / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + st]);
        __syncthreads();
    }
    if (threadIdx.x == 0) pp[k] = (mx - red[0]) / sn;
}

}  // namespace

}  // namespace sid

using namespace sid;

extern "C" int sid_merge_filters(sid_ctx* c, const float* ts, int64_t K, int64_t F, float* templ, int64_t P,
                                 double limit, int bg_sub, int32_t* keep, void* stream)
{
    SID_REQUIRE(c && ts && templ && keep, "sid_merge_filters: NULL argument");
    SID_REQUIRE(bg_sub == 0 || bg_sub == 1, "sid_merge_filters: bg_sub must be 0 or 1");
    SID_REQUIRE(K > 2 * bg_sub && F > 1 && P > 0, "sid_merge_filters: sizes K=%lld F=%lld P=%lld", (long long)K,
                (long long)F, (long long)P);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t Kt = K - bg_sub;  // template rows
    // trace correlation: Gram of the centred traces
    SID_TRY(c->mf[0].alloc((size_t)(F * K) * sizeof(float)));
    SID_TRY(c->mf[1].alloc((size_t)(K * K) * sizeof(float)));
    SID_TRY(c->ws.alloc((size_t)sgemm_ws_elems(K, K, F) * sizeof(float)));
    k_center_transpose<<<(unsigned)cdiv(K, 32), kT, 0, st>>>(ts, K, F, c->mf[0].as<float>());
    SID_CHECK_LAUNCH();
    SID_TRY(sgemm_tn(c->mf[0].as<float>(), c->mf[0].as<float>(), K, K, F, F, F, c->mf[1].as<float>(), K, 1.f, 0.f,
                     c->ws.as<float>(), (int64_t)(c->ws.bytes / 4), st));
    // template overlap: exact 0/1 Gram on the tensor cores
    SID_TRY(c->a_hi.alloc((size_t)blk16_elems(P, Kt) * 2));
    SID_TRY(c->mf[2].alloc((size_t)(Kt * Kt) * sizeof(float)));
    k_template_blk<<<dim3((unsigned)cdiv(P, 64), (unsigned)cdiv(Kt, 64)), kT, 0, st>>>(templ, Kt, P,
                                                                                      c->a_hi.as<uint16_t>());
    SID_CHECK_LAUNCH();
    int bn = 0, sk = 0;
    gemm_autotune((int)Kt, (int)Kt, (int)cdiv(P, 64), &bn, &sk);
    SID_TRY(c->mf[3].alloc((size_t)(sk * Kt * Kt) * sizeof(float)));
    const void* As[1] = {c->a_hi.p};
    SID_TRY(gemm_tn(As, As, 1, Kt, Kt, P, true, c->mf[2].as<float>(), Kt, 1.f, 0.f, bn, sk, c->mf[3].as<float>(),
                    (int64_t)(c->mf[3].bytes / 4), c->errflag.as<int>(), st));
    std::vector<float> G((size_t)(K * K)), O((size_t)(Kt * Kt));
    SID_CUDA_TRY(cudaMemcpyAsync(G.data(), c->mf[1].p, G.size() * 4, cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaMemcpyAsync(O.data(), c->mf[2].p, O.size() * 4, cudaMemcpyDeviceToHost, st));
    SID_TRY(ctx_sync(c, st));
    // merge_filters.m:19-29 with MATLAB's types: single arithmetic, and the
    // comparisons with the double constants 1/3 and 1 + limit made in double
    const int64_t Km = Kt - bg_sub;  // the second crop of merge_filters.m:27
    std::vector<unsigned char> mat((size_t)(Km * Km), 0);  // tril(temp > 1 + limit), column-major
    for (int64_t j = 0; j < Km; ++j)
        for (int64_t i = j; i < Km; ++i) {
            const float corr = (float)((double)G[i + K * j] /
                                       std::sqrt((double)G[i + K * i] * (double)G[j + K * j])) - (i == j ? 1.f : 0.f);
            const float mn = std::min(O[i + Kt * i], O[j + Kt * j]);
            const float ov = (1.f / mn) * O[i + Kt * j] - (i == j ? 1.f : 0.f);
            const float v = ((double)ov > 1.0 / 3.0 ? 1.f : 0.f) + corr;
            mat[i + Km * j] = (double)v > 1.0 + limit;
        }
    // merge_filters.m:33-36: for every column with a partner, in order
    std::vector<int> dst, beg{0}, list;
    for (int64_t j = 0; j < Km; ++j) {
        bool any = false;
        for (int64_t i = j; i < Km; ++i)
            if (mat[i + Km * j]) {
                list.push_back((int)i);
                any = true;
            }
        if (any) {
            dst.push_back((int)j);
            beg.push_back((int)list.size());
        }
    }
    SID_TRY(c->mf[4].alloc((dst.size() + beg.size() + list.size() + (size_t)Kt + 4) * sizeof(int)));
    int* d_dst = c->mf[4].as<int>();
    int* d_beg = d_dst + dst.size();
    int* d_list = d_beg + beg.size();
    int* d_nz = d_list + list.size();
    if (!dst.empty()) {
        SID_CUDA_TRY(cudaMemcpyAsync(d_dst, dst.data(), dst.size() * 4, cudaMemcpyHostToDevice, st));
        SID_CUDA_TRY(cudaMemcpyAsync(d_beg, beg.data(), beg.size() * 4, cudaMemcpyHostToDevice, st));
        SID_CUDA_TRY(cudaMemcpyAsync(d_list, list.data(), list.size() * 4, cudaMemcpyHostToDevice, st));
    }
    SID_CUDA_TRY(cudaMemsetAsync(d_nz, 0, (size_t)Kt * 4, st));
    k_apply_merges<<<(unsigned)std::min<int64_t>(cdiv(P, kT), 152 * 16), kT, 0, st>>>(
        templ, Kt, P, d_dst, d_beg, d_list, (int)dst.size(), d_nz);
    SID_CHECK_LAUNCH();
    std::vector<int> nz((size_t)Kt);
    SID_CUDA_TRY(cudaMemcpyAsync(nz.data(), d_nz, (size_t)Kt * 4, cudaMemcpyDeviceToHost, st));
    SID_TRY(ctx_sync(c, st));
    for (int64_t k = 0; k < Kt; ++k) keep[k] = nz[(size_t)k];
    if (bg_sub) keep[K - 1] = 1;  // the background row is kept (merge_filters.m:39-41)
    return SID_OK;
}

extern "C" int sid_snr_order(sid_ctx* c, const float* traces, int64_t K, int64_t F, int bg_sub, int32_t* order,
                             void* stream)
{
    SID_REQUIRE(c && traces && order, "sid_snr_order: NULL argument");
    SID_REQUIRE(bg_sub == 0 || bg_sub == 1, "sid_snr_order: bg_sub must be 0 or 1");
    SID_REQUIRE(K > bg_sub && F > 12, "sid_snr_order: sizes K=%lld F=%lld", (long long)K, (long long)F);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = K - bg_sub;
    SID_TRY(c->mf[5].alloc((size_t)(n * 2 * F + n) * sizeof(double)));
    double* work = c->mf[5].as<double>();
    double* pp = work + n * 2 * F;
    k_snr<<<(unsigned)n, kT, 0, st>>>(traces, K, (int)F, work, pp);
    SID_CHECK_LAUNCH();
    std::vector<double> h((size_t)n);
    SID_CUDA_TRY(cudaMemcpyAsync(h.data(), pp, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    SID_TRY(ctx_sync(c, st));
    // [~, n] = sort(-pp): ascending in -pp, ties in index order (MATLAB's sort is
    // stable), NaN last
    std::vector<int> idx((size_t)n);
    for (int64_t k = 0; k < n; ++k) idx[(size_t)k] = (int)k;
    auto key = [&](int a) {
        const double v = -h[(size_t)a];
        return std::isnan(v) ? HUGE_VAL : v;
    };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        const bool na = std::isnan(h[(size_t)a]), nb = std::isnan(h[(size_t)b]);
        if (na != nb) return nb;  // non-NaN before NaN
        return !na && key(a) < key(b);
    });
    for (int64_t k = 0; k < n; ++k) order[k] = idx[(size_t)k];
    if (bg_sub) order[n] = (int32_t)(K - 1);
    return SID_OK;
}
