// nmf.cu -- the two projected-gradient steps of the SID matrix factorisation
// Y ~ S*T (fast_NMF.m:185-186): T_update.m:1-78 and S_update.m:1-80.
//
// Shapes (MATLAB column-major): Y P x F (movie, FP32 or FP16), S P x R
// (spatial components), T R x F (timeseries).  Each step is one gradient
// evaluation, a projection onto the non-negativity constraint, an exact line
// search and a clamped update.  The pixel-long contractions (S'S, S'Y) run
// through the tensor-core contraction at the requested precision, and so do
// S_update's pixel-by-rank products (Y T', S Q_T, v Q_T; P x R with an F- or
// R-deep reduction) except at FP32 precision, where they and the frame- and
// rank-long products (R x R, R x F) run on the FP32 SIMT GEMMs.  The line
// search's reductions over R x F accumulate in FP64; those over the P x R
// factors as FP32 two-sum pairs (FP64-grade).  The step sizes and the split
// precision's power-of-two operand scales stay in device memory: neither step
// makes its stream wait on the host, so both can be captured in a CUDA graph
// once their workspaces have been sized by an ordinary call.
#include <cmath>
#include <cstring>

#include "sid_internal.cuh"

namespace sid {

int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st);
int sgemm_nt(const void* A, int a_f16, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb,
             float* C, int64_t ldc, cudaStream_t st);
int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
            float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws, int64_t ws_elems, int* err,
            cudaStream_t st);
void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk);
int split16(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
            float scale, cudaStream_t st);
int split16_t(const float* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* hi, uint16_t* lo, bool bf16,
              float scale, cudaStream_t st);
int copy16_t(const uint16_t* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* dst, cudaStream_t st);
int64_t blk16_elems(int64_t k, int64_t rows);
int absmax(const float* x, int64_t n, unsigned int* out, cudaStream_t st);

namespace {

constexpr int kRedBlocks = 1024;  // partial-sum slots of the global reductions

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float finite_or_zero(double a) { return isfinite(a) ? (float)a : 0.f; }
__device__ __forceinline__ float finite_or_zero_f(float a) { return isfinite(a) ? a : 0.f; }

// FP32 pairs hi + lo for the pixel-long loops of S_update (P x R elements):
// two-sum additions and fmaf two-products give FP64-grade sums on the FP32
// pipes.  GB300's FP64 rate is about 1/64 of its FP32 rate, so FP64 arithmetic
// per element (and a 64-bit integer division per element to find its column)
// held these kernels far below the HBM rate.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    const float l = (a.y + b.y) + e;
    const float hi = s + l;
    return make_float2(hi, l - (hi - s));
}
__device__ __forceinline__ float2 two_prod(float a, float b)
{
    const float p = a * b;
    return make_float2(p, fmaf(a, b, -p));
}
__device__ __forceinline__ float2 ff_from(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ float2 warp_sum_ff(float2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
    return v;
}
// block sum of pairs (blockDim.x a multiple of 32, <= 1024), valid in thread 0
__device__ __forceinline__ float2 block_sum_ff(float2 v)
{
    __shared__ float2 sh[32];
    v = warp_sum_ff(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) v = ff_add(v, sh[i]);
    return v;
}

__global__ void k_nan_zero(float* __restrict__ x, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (isnan(x[i])) x[i] = 0.f;
}

// out (cols x rows) = in' for in (rows x cols), both column-major; 32 x 32 tiles
__global__ void k_transpose_tile(const float* __restrict__ in, int64_t rows, int64_t cols, float* __restrict__ out)
{
    __shared__ float tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t r = r0 + threadIdx.x, c = c0 + j;
        if (r < rows && c < cols) tile[j][threadIdx.x] = in[r + rows * c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t c = c0 + threadIdx.x, r = r0 + j;
        if (r < rows && c < cols) out[c + cols * r] = tile[threadIdx.x][j];
    }
}

int transpose(const float* in, int64_t rows, int64_t cols, float* out, cudaStream_t st)
{
    SID_REQUIRE(cdiv(cols, 32) <= 65535, "transpose: too many columns");
    dim3 grid((unsigned)cdiv(rows, 32), (unsigned)cdiv(cols, 32)), block(32, 8);
    k_transpose_tile<<<grid, block, 0, st>>>(in, rows, cols, out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Per row r of an R x F matrix: sum and sum of squares over the F columns
// (one warp per row).
__global__ void k_row_moments(const float* __restrict__ T, int R, int64_t F, double* __restrict__ s1,
                              double* __restrict__ s2)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= R) return;
    double a = 0.0, b = 0.0;
    for (int64_t f = lane; f < F; f += 32) {
        const double v = T[warp + (int64_t)R * f];
        a += v;
        b += v * v;
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        s1[warp] = a;
        if (s2) s2[warp] = b;
    }
}

// sd(r) = std(T(r, :)) with N-1 normalisation (two passes; 0 for one frame)
__global__ void k_row_std(const float* __restrict__ T, int R, int64_t F, double* __restrict__ sd)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= R) return;
    double a = 0.0;
    for (int64_t f = lane; f < F; f += 32) a += T[warp + (int64_t)R * f];
    const double mu = warp_sum(a) / (double)F;
    double b = 0.0;
    for (int64_t f = lane; f < F; f += 32) {
        const double d = T[warp + (int64_t)R * f] - mu;
        b += d * d;
    }
    b = warp_sum(b);
    if (lane == 0) sd[warp] = F > 1 ? sqrt(b / (double)(F - 1)) : 0.0;
}

// platz = sqrt of the squared row norms, FP32 (once per row, not per element)
__global__ void k_sqrt_f(const double* __restrict__ sq, int R, float* __restrict__ pl)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) pl[r] = (float)sqrt(sq[r]);
}

// T(r, :) /= platz(r)  (T_update.m:14-19)
__global__ void k_renorm_rows_t(float* __restrict__ T, int R, int64_t F, const float* __restrict__ pl)
{
    const int64_t nT = (int64_t)R * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nT; i += (int64_t)gridDim.x * blockDim.x)
        T[i] = T[i] / pl[i % R];
}

// S(:, r) *= platz(r)  (T_update.m:14-19); grid.y = component r
__global__ void k_renorm_cols_s(float* __restrict__ S, int64_t P, const float* __restrict__ pl)
{
    const float m = pl[blockIdx.y];
    float* col = S + P * blockIdx.y;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
        col[p] = col[p] * m;
}

// Sm(p, r) = active(p) ? S(p, r) : 0  (S(opts.active, :), T_update.m:24-25);
// grid.y = component r
__global__ void k_mask_rows(const float* __restrict__ S, const uint8_t* __restrict__ active, int64_t P,
                            float* __restrict__ Sm)
{
    const int64_t o = P * blockIdx.y;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
        Sm[o + p] = active[p] ? S[o + p] : 0.f;
}

// out(r, f) = v(r, f) - rowsum(r) / F: the use_std centring inside Q(x)
// (T_update.m:29: Q_S*x - Q_S*sum(x,2)/F = Q_S*(x - sum(x,2)/F))
__global__ void k_centre_rows(const float* __restrict__ v, const double* __restrict__ rs, int R, int64_t F,
                              float* __restrict__ out)
{
    const int64_t n = (int64_t)R * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)((double)v[i] - rs[i % R] / (double)F);
}

// zscore along the first dimension of an n1 x n2 matrix (MATLAB zscore: N-1
// normalisation, zero deviation replaced by 1), one warp per column.
__global__ void k_zscore_cols(const float* __restrict__ T, int64_t n1, int64_t n2, float* __restrict__ z)
{
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n2) return;
    const float* col = T + n1 * warp;
    double a = 0.0;
    for (int64_t i = lane; i < n1; i += 32) a += col[i];
    const double mu = warp_sum(a) / (double)n1;
    double b = 0.0;
    for (int64_t i = lane; i < n1; i += 32) {
        const double d = col[i] - mu;
        b += d * d;
    }
    b = warp_sum(b);
    double sd = n1 > 1 ? sqrt(b / (double)(n1 - 1)) : 0.0;
    if (sd == 0.0) sd = 1.0;
    for (int64_t i = lane; i < n1; i += 32) z[n1 * warp + i] = (float)((col[i] - mu) / sd);
}

// Correlation-penalty row terms (T_update.m:40-41): with H1 = C1*zsc - zsc,
// rs(r) = sum_f H1(r, f) and dg(r) = sum_f H1(r, f) zsc(r, f).
__global__ void k_corr_rows(const float* __restrict__ C1z, const float* __restrict__ zsc, int R, int64_t F,
                            double* __restrict__ rs, double* __restrict__ dg)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= R) return;
    double a = 0.0, b = 0.0;
    for (int64_t f = lane; f < F; f += 32) {
        const int64_t i = warp + (int64_t)R * f;
        const double h = (double)C1z[i] - (double)zsc[i];
        a += h;
        b += h * (double)zsc[i];
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        rs[warp] = a;
        dg[warp] = b;
    }
}

struct TGrad {
    const float* qT;   // S_a' Y_a  (R x F)
    const float* QT;   // Q(T)      (R x F)
    const float* T;
    const float* zsc;  // lamb_corr terms (or null)
    const float* C1z;
    const double* rs;
    const double* dg;
    const double* sd;  // d = std(T, [], 2)
    const double* wq;  // use_std: S_a' opts.Y(active) (R; divided by F here) or null
    float* dT;         // out: the projected gradient df_T_
    double lamb_temp, lamb_corr, lamb_tv;
    int R;
    int64_t F;
};

// df_T = -q_T + Q(T) + lamb_temp [+ lamb_corr hilf] [+ lamb_temp_TV tv]
// (T_update.m:36-56), then df_T_ = passive .* df_T  (:59-60)
__global__ void k_t_grad(TGrad g)
{
    const int64_t n = (int64_t)g.R * g.F;
    const double Fd = (double)g.F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % g.R);
        const int64_t f = i / g.R;
        double q = (double)g.qT[i];
        if (g.wq) q -= g.wq[r] / Fd;
        double df = -q + (double)g.QT[i] + g.lamb_temp;
        if (g.zsc) {
            const double h1 = (double)g.C1z[i] - (double)g.zsc[i];
            const double hilf = (h1 - g.rs[r] / Fd - g.dg[r] * (double)g.zsc[i] / Fd) / g.sd[r];
            df += g.lamb_corr * hilf;
        }
        if (g.lamb_tv != 0.0) {
            // padded row p(0) = T(1), p(1..F) = T(0..F-1), p(F+1) = T(F-2); tv = -p(f) + 2p(f+1) - p(f+2)
            const float* row = g.T + r;
            const int64_t R = g.R;
            const double left = f == 0 ? row[R * 1] : row[R * (f - 1)];
            const double right = f == g.F - 1 ? row[R * (g.F - 2)] : row[R * (f + 1)];
            df += g.lamb_tv * (-left + 2.0 * (double)row[R * f] - right);
        }
        const bool passive = g.T[i] > 0.f || df < 0.0;
        g.dT[i] = passive ? (float)df : 0.f;
    }
}

// Per column f of two R x F matrices: num(f) = sum_r a^2 (or a.b2), den(f) = sum_r a.b
// (one warp per column; R contiguous)
__global__ void k_col_dots(const float* __restrict__ a, const float* __restrict__ b2, const float* __restrict__ b,
                           int R, int64_t F, double* __restrict__ num, double* __restrict__ den)
{
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= F) return;
    double x = 0.0, y = 0.0;
    for (int r = lane; r < R; r += 32) {
        const int64_t i = r + (int64_t)R * warp;
        const double av = a[i];
        x += av * (b2 ? (double)b2[i] : av);
        y += av * (double)b[i];
    }
    x = warp_sum(x);
    y = warp_sum(y);
    if (lane == 0) {
        num[warp] = x;
        den[warp] = y;
    }
}

// Step sizes from per-slot sums.  pointwise: alpha(i) = num(i) / den(i);
// else alpha(0) = sum num / sum den, optionally max(alpha, floor) with MATLAB's
// NaN-ignoring max.  NaN and Inf become 0 (T_update.m:68-69, S_update.m:59-67).
__global__ void k_alpha(const double* __restrict__ num, const double* __restrict__ den, int64_t n, int pointwise,
                        double floor_, float* __restrict__ alpha)
{
    if (pointwise) {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            alpha[i] = finite_or_zero(num[i] / den[i]);
        return;
    }
    if (blockIdx.x != 0) return;
    __shared__ double sn[32], sd[32];
    double x = 0.0, y = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        x += num[i];
        y += den[i];
    }
    x = warp_sum(x);
    y = warp_sum(y);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sn[w] = x;
        sd[w] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            a += sn[i];
            b += sd[i];
        }
        double al = a / b;
        if (floor_ > 0.0) al = isnan(al) ? floor_ : fmax(al, floor_);
        alpha[0] = finite_or_zero(al);
    }
}

// x = max(x - alpha .* d, 0); alpha per column of a rows x cols matrix
// (per_col), per row (per_row) or one scalar.
__global__ void k_pg_step(float* __restrict__ x, const float* __restrict__ d, int64_t rows, int64_t cols,
                          const float* __restrict__ alpha, int mode)
{
    const int64_t n = rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float a = mode == 0 ? alpha[0] : (mode == 1 ? alpha[i / rows] : alpha[i % rows]);
        const float v = x[i] - d[i] * a;
        x[i] = v < 0.f ? 0.f : v;
    }
}

// ---- S_update kernels ----

// Q_T(i, j) += -ts(i) ts(j) / F (use_std) + l1o * hilf(i, j)   (S_update.m:14,20)
__global__ void k_qt_adjust(float* __restrict__ QT, int R, const double* __restrict__ ts, double invF,
                            const float* __restrict__ hilf, double l1o)
{
    const int64_t n = (int64_t)R * R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double q = QT[i];
        if (ts) q -= ts[i % R] * ts[i / R] * invF;
        if (hilf) q += l1o * (double)hilf[i];
        QT[i] = (float)q;
    }
}

// df_S = -q_S [+ opts.Y .* ts' / F] + S*Q_T + lamb_spat  (S_update.m:8-34), in place
// of SQ; grid.y = component r, the pixels of its column grid-strided in x
__global__ void k_s_grad(const float* __restrict__ qS, float* __restrict__ SQ, int64_t P,
                         const float* __restrict__ ymean, const double* __restrict__ ts, double invF, double lamb_spat)
{
    const int r = blockIdx.y;
    __shared__ float2 tsf, lam;
    if (threadIdx.x == 0) {
        tsf = ymean ? ff_from(ts[r] * invF) : make_float2(0.f, 0.f);
        lam = ff_from(lamb_spat);
    }
    __syncthreads();
    const float* q = qS + P * r;
    float* sq = SQ + P * r;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        float2 a = ff_add(make_float2(sq[p], 0.f), make_float2(-q[p], 0.f));
        if (ymean) {
            const float y = ymean[p];
            const float2 t = two_prod(y, tsf.x);
            a = ff_add(a, make_float2(t.x, fmaf(y, tsf.y, t.y)));
        }
        a = ff_add(a, lam);
        sq[p] = a.x + a.y;
    }
}

// Direction of the S step (S_update.m:38-53), one thread per pixel:
// orth:  v = df [+ l2o * M2]; z = sum_r S.*v; v = v - S.*z; v = passive(S, v) .* v
// else:  v = passive(S, df) .* df
__global__ void k_s_dir(const float* __restrict__ S, const float* __restrict__ df, const float* __restrict__ M2,
                        float l2o, int orth, int64_t P, int R, float* __restrict__ v)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        if (!orth) {
            for (int r = 0; r < R; ++r) {
                const int64_t i = p + P * r;
                const float d = df[i];
                v[i] = (S[i] > 0.f || d < 0.f) ? d : 0.f;
            }
            continue;
        }
        float2 z = make_float2(0.f, 0.f);
        for (int r = 0; r < R; ++r) {
            const int64_t i = p + P * r;
            const float vi = M2 ? fmaf(l2o, M2[i], df[i]) : df[i];
            z = ff_add(z, two_prod(S[i], vi));
        }
        for (int r = 0; r < R; ++r) {
            const int64_t i = p + P * r;
            const float vi = M2 ? fmaf(l2o, M2[i], df[i]) : df[i];
            const float si = S[i];
            const float w = fmaf(-si, z.y, fmaf(-si, z.x, vi));
            v[i] = (si > 0.f || w < 0.f) ? w : 0.f;
        }
    }
}

// Per pixel: num = sum_r v.*df, den = sum_r v.*vQ.  pointwise: alpha(p) directly;
// else per-block partial sums into part[2 * block] (reduced by k_alpha).
__global__ void k_s_sums(const float* __restrict__ v, const float* __restrict__ df, const float* __restrict__ vQ,
                         int64_t P, int R, int pointwise, float* __restrict__ alpha, double* __restrict__ part)
{
    float2 bn = make_float2(0.f, 0.f), bd = bn;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        float2 x = make_float2(0.f, 0.f), y = x;
        for (int r = 0; r < R; ++r) {
            const int64_t i = p + P * r;
            const float vv = v[i];
            x = ff_add(x, two_prod(vv, df[i]));
            y = ff_add(y, two_prod(vv, vQ[i]));
        }
        if (pointwise) alpha[p] = finite_or_zero_f(x.x / y.x);
        bn = ff_add(bn, x);
        bd = ff_add(bd, y);
    }
    if (pointwise) return;
    bn = block_sum_ff(bn);
    __syncthreads();
    bd = block_sum_ff(bd);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = (double)bn.x + (double)bn.y;
        part[kRedBlocks + blockIdx.x] = (double)bd.x + (double)bd.y;
    }
}

// Column norms of S (P x R), one block per column: squared norm (FP64) and
// the norm itself (FP32) for the rescaling
__global__ void k_col_norm2(const float* __restrict__ S, int64_t P, double* __restrict__ out, float* __restrict__ pl)
{
    const float* col = S + P * blockIdx.x;
    float2 a = make_float2(0.f, 0.f);
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) a = ff_add(a, two_prod(col[p], col[p]));
    a = block_sum_ff(a);
    if (threadIdx.x == 0) {
        const double s = (double)a.x + (double)a.y;
        out[blockIdx.x] = s;
        pl[blockIdx.x] = (float)sqrt(s);
    }
}

// S(:, r) /= platz(r)   (S_update.m:75-79); grid.y = component r
__global__ void k_unit_cols_s(float* __restrict__ S, int64_t P, const float* __restrict__ pl)
{
    const float d = pl[blockIdx.y];
    float* col = S + P * blockIdx.y;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
        col[p] = col[p] / d;
}

// T(r, :) *= platz(r)   (S_update.m:75-79)
__global__ void k_unit_rows_t(float* __restrict__ T, int R, int64_t F, const float* __restrict__ pl)
{
    const int64_t n = (int64_t)R * F;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        T[j] = pl[j % R] * T[j];
}

// x(:, r) = max(x(:, r) - alpha .* d(:, r), 0) for a P x R matrix with alpha
// per pixel (per_row != 0) or one scalar; grid.y = column r
__global__ void k_pg_step_cols(float* __restrict__ x, const float* __restrict__ d, int64_t P,
                               const float* __restrict__ alpha, int per_row)
{
    const int64_t o = P * blockIdx.y;
    const float a0 = alpha[0];
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        const float a = per_row ? alpha[p] : a0;
        const float v = x[o + p] - d[o + p] * a;
        x[o + p] = v < 0.f ? 0.f : v;
    }
}

inline unsigned grid_for(int64_t n, int per = 256) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, per), 152 * 16)); }
// P x R column kernels: grid.y = column, about 152 * 16 CTAs in all
inline dim3 grid_cols(int64_t P, int64_t R)
{
    return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(P, 256), cdiv(152 * 16, R))), (unsigned)R);
}

// C (m x n) = A' B, FP32 SIMT (through the contraction entry, which owns the workspace)
inline int tn32(sid_ctx* c, const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb,
                float* C, cudaStream_t st)
{
    return contract(c, A, B, false, m, n, k, lda, ldb, C, m, 1.f, 0.f, SID_PREC_FP32, st);
}

}  // namespace
}  // namespace sid

using namespace sid;

static int nmf_checks(sid_ctx* c, const void* Y, int ydtype, const float* S, const float* T, int64_t P, int64_t R,
                      int64_t F, const sid_nmf_opts* o, int prec, const char* who)
{
    SID_REQUIRE(c && Y && S && T && o, "%s: NULL argument", who);
    SID_REQUIRE(P >= 1 && R >= 1 && F >= 1, "%s: empty problem (P %lld, R %lld, F %lld)", who, (long long)P,
                (long long)R, (long long)F);
    SID_REQUIRE(R <= INT32_MAX && F <= INT32_MAX, "%s: dimension too large", who);
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "%s: unknown Y dtype %d", who, ydtype);
    SID_REQUIRE(prec == SID_PREC_FP32 || prec == SID_PREC_SPLIT || prec == SID_PREC_BF16, "%s: unknown precision %d",
                who, prec);
    return SID_OK;
}

extern "C" void sid_nmf_defaults(sid_nmf_opts* o)
{
    std::memset(o, 0, sizeof(*o));
}

extern "C" int sid_t_update(sid_ctx* c, const void* Y, int ydtype, float* T, float* S, int64_t P, int64_t R,
                            int64_t F, const uint8_t* active, const float* ymean, const sid_nmf_opts* o, int prec,
                            void* stream)
{
    SID_TRY(nmf_checks(c, Y, ydtype, S, T, P, R, F, o, prec, "T_update"));
    SID_REQUIRE(!o->use_std || ymean, "T_update: use_std needs opts.Y (ymean)");
    SID_REQUIRE(o->lamb_temp_TV == 0.0 || F >= 2, "T_update: lamb_temp_TV needs at least 2 frames");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t RF = R * F;
    DBuf* b = c->mf;
    SID_TRY(b[0].alloc((size_t)(R * R) * 4 * 2));  // Q_S, Q_S'
    SID_TRY(b[1].alloc((size_t)RF * 4 * 5));       // q_T, Q(T), dT, Q(dT), scratch
    SID_TRY(b[2].alloc((size_t)(6 * R + 2 * F + 8) * 8));
    SID_TRY(b[3].alloc((size_t)(F + 1) * 4));      // alpha
    float* QS = b[0].as<float>();
    float* QSt = QS + R * R;
    float* qT = b[1].as<float>();
    float* QTm = qT + RF;
    float* dT = QTm + RF;
    float* Qd = dT + RF;
    float* tmp = Qd + RF;
    double* s1 = b[2].as<double>();
    double* s2 = s1 + R;
    double* rs = s2 + R;
    double* dg = rs + R;
    double* wq = dg + R;
    double* vs = wq + R;
    double* num = vs + R;
    double* den = num + F;
    float* alpha = b[3].as<float>();

    // NaN -> 0 (T_update.m:5-6)
    k_nan_zero<<<grid_for(P * R), 256, 0, st>>>(S, P * R);
    k_nan_zero<<<grid_for(RF), 256, 0, st>>>(T, RF);
    SID_CHECK_LAUNCH();
    // unit-norm rows of T, S rescaled (T_update.m:14-19)
    if (o->lamb_corr > 0) {
        SID_REQUIRE(R <= 65535, "T_update: at most 65535 components");
        float* pl = tmp;  // R floats, free until the use_std products below
        k_row_moments<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(T, (int)R, F, s1, s2);
        k_sqrt_f<<<(unsigned)cdiv(R, 256), 256, 0, st>>>(s2, (int)R, pl);
        k_renorm_rows_t<<<grid_for(RF), 256, 0, st>>>(T, (int)R, F, pl);
        k_renorm_cols_s<<<grid_cols(P, R), 256, 0, st>>>(S, P, pl);
        SID_CHECK_LAUNCH();
    }
    // Q_S = S_a' S_a, q_T = S_a' Y_a (T_update.m:24-25)
    const float* Sa = S;
    if (active) {
        SID_TRY(b[4].alloc((size_t)(P * R) * 4));
        SID_REQUIRE(R <= 65535, "T_update: at most 65535 components");
        k_mask_rows<<<grid_cols(P, R), 256, 0, st>>>(S, active, P, b[4].as<float>());
        SID_CHECK_LAUNCH();
        Sa = b[4].as<float>();
    }
    SID_TRY(contract(c, Sa, Sa, false, R, R, P, P, P, QS, R, 1.f, 0.f, prec, st));
    SID_TRY(contract(c, Sa, Y, ydtype == SID_DTYPE_F16, R, F, P, P, P, qT, R, 1.f, 0.f,
                     (ydtype == SID_DTYPE_F16 && prec == SID_PREC_FP32) ? SID_PREC_SPLIT : prec, st));
    SID_TRY(transpose(QS, R, R, QSt, st));
    // use_std: q_T -= S_a' opts.Y(active) / F  (T_update.m:30)
    const double* wqp = nullptr;
    if (o->use_std) {
        float* w32 = tmp;  // R floats
        SID_TRY(tn32(c, Sa, ymean, R, 1, P, P, P, w32, st));
        // wq = w32 widened to FP64 (the row-moment kernel on an R x 1 matrix)
        k_row_moments<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(w32, (int)R, 1, wq, nullptr);
        SID_CHECK_LAUNCH();
        wqp = wq;
    }
    auto Qf = [&](const float* v, float* out) -> int {
        // Q(x) = Q_S x [- Q_S sum(x, 2) / F]  (T_update.m:29,32)
        const float* src = v;
        if (o->use_std) {
            k_row_moments<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(v, (int)R, F, vs, nullptr);
            k_centre_rows<<<grid_for(RF), 256, 0, st>>>(v, vs, (int)R, F, tmp);
            SID_CHECK_LAUNCH();
            src = tmp;
        }
        return tn32(c, QSt, src, R, F, R, R, R, out, st);
    };
    SID_TRY(Qf(T, QTm));
    TGrad g{};
    g.qT = qT;
    g.QT = QTm;
    g.T = T;
    g.wq = wqp;
    g.dT = dT;
    g.lamb_temp = o->lamb_temp;
    g.lamb_corr = o->lamb_corr;
    g.lamb_tv = o->lamb_temp_TV;
    g.R = (int)R;
    g.F = F;
    if (o->lamb_corr != 0.0) {
        // zsc = zscore(T) (columns; a single row is standardised along the frames),
        // C1 = zsc zsc', C1z = C1 zsc  (T_update.m:38-41)
        SID_TRY(b[5].alloc((size_t)(RF * 3 + R * R) * 4));
        float* zsc = b[5].as<float>();
        float* zt = zsc + RF;
        float* C1z = zt + RF;
        float* C1 = C1z + RF;
        if (R > 1) k_zscore_cols<<<(unsigned)cdiv(F * 32, 256), 256, 0, st>>>(T, R, F, zsc);
        else k_zscore_cols<<<1, 256, 0, st>>>(T, F, 1, zsc);
        SID_CHECK_LAUNCH();
        SID_TRY(transpose(zsc, R, F, zt, st));
        SID_TRY(tn32(c, zt, zt, R, R, F, F, F, C1, st));
        SID_TRY(tn32(c, C1, zsc, R, F, R, R, R, C1z, st));  // C1 is symmetric
        // d = std(T, [], 2) of the (renormalised) T
        k_row_std<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(T, (int)R, F, s1);
        k_corr_rows<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(C1z, zsc, (int)R, F, rs, dg);
        SID_CHECK_LAUNCH();
        g.zsc = zsc;
        g.C1z = C1z;
        g.rs = rs;
        g.dg = dg;
        g.sd = s1;
    }
    k_t_grad<<<grid_for(RF), 256, 0, st>>>(g);
    SID_CHECK_LAUNCH();
    // exact line search (T_update.m:64-70)
    SID_TRY(Qf(dT, Qd));
    k_col_dots<<<(unsigned)cdiv(F * 32, 256), 256, 0, st>>>(dT, nullptr, Qd, (int)R, F, num, den);
    k_alpha<<<o->pointwise ? grid_for(F) : 1, 256, 0, st>>>(num, den, F, o->pointwise, 0.0, alpha);
    k_pg_step<<<grid_for(RF), 256, 0, st>>>(T, dT, R, F, alpha, o->pointwise ? 1 : 0);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

namespace sid {

// Products of a pixel-major P x k factor X (pixels contiguous: the movie, S,
// the step direction) with a small k x n matrix W, on the tensor cores:
// C (P x n) = X W.  X is brought once into the K-blocked 16-bit layout of the
// tcgen05 GEMM by a transposing tile kernel.  Split precision: an FP16 movie
// as it is, FP32 factors as FP16 hi/lo of X s (22 significant bits; a
// power-of-two s brings max |X| into [2^13, 2^14)), W likewise, and the three
// products hi*hi + hi*lo + lo*hi.  (BF16 hi/lo keeps 16 bits, which the
// cancellation in S_update's use_std gradient amplifies past FP32-level
// agreement.)  BF16 precision: one BF16 pass.  The scales are found, applied
// and undone on the device (the context's scale words), so these products
// never make the stream wait on the host.
int pix_operand(sid_ctx* c, int slot, const void* X, bool x_f16, int64_t P, int64_t k, int prec, PixOperand* op,
                cudaStream_t st)
{
    const size_t bytes = (size_t)blk16_elems(k, P) * 2;
    DBuf* b = c->pix + 2 * slot;
    SID_TRY(b[0].alloc(bytes));
    if (x_f16) {
        SID_TRY(copy16_t(static_cast<const uint16_t*>(X), P, k, P, b[0].as<uint16_t>(), st));
        *op = {b[0].p, nullptr, true, nullptr};
        return SID_OK;
    }
    const float* xf = static_cast<const float*>(X);
    if (prec != SID_PREC_SPLIT) {
        SID_TRY(split16_t(xf, P, k, P, b[0].as<uint16_t>(), nullptr, true, 1.f, st));
        *op = {b[0].p, nullptr, false, nullptr};
        return SID_OK;
    }
    float* sw = c->scales.as<float>() + 4 * slot;
    SID_TRY(pow2_scale_dev(xf, P * k, reinterpret_cast<unsigned int*>(sw), sw + 1, st));
    SID_TRY(b[1].alloc(bytes));
    SID_TRY(split16_t_ds(xf, P, k, P, b[0].as<uint16_t>(), b[1].as<uint16_t>(), false, 1.f, sw + 1, st));
    *op = {b[0].p, b[1].p, true, sw + 1};
    return SID_OK;
}

// C (P x n, leading dimension P) = X (P x k) * W (k x n, W(kk, j) at W[kk + ldw*j])
int gemm_pix(sid_ctx* c, const PixOperand& x, int64_t P, int64_t k, const float* W, int64_t n, int64_t ldw,
             float* C, int prec, cudaStream_t st)
{
    const bool split = prec == SID_PREC_SPLIT;
    const size_t wbytes = (size_t)blk16_elems(k, n) * 2;
    SID_TRY(c->pix[4].alloc(wbytes));
    if (split) SID_TRY(c->pix[5].alloc(wbytes));
    uint16_t* wh = c->pix[4].as<uint16_t>();
    uint16_t* wl = split ? c->pix[5].as<uint16_t>() : nullptr;
    int bn = 0, sk = 0;
    gemm_autotune((int)P, (int)n, (int)cdiv(k, 64), &bn, &sk);
    const float* dalpha = nullptr;
    const void *As[3], *Bs[3];
    int npass = 1;
    As[0] = As[1] = x.hi;
    As[2] = x.lo;
    Bs[0] = Bs[2] = wh;
    Bs[1] = wl;
    if (x.f16) {
        // W s_w in FP16 hi/lo; alpha = 1 / (s_x s_w) in the epilogue
        float* sw = c->scales.as<float>() + 8;
        SID_TRY(pow2_scale_dev(W, ldw * (n - 1) + k, reinterpret_cast<unsigned int*>(sw), sw + 1, st));
        SID_TRY(split16_ds(W, k, n, ldw, wh, wl, false, 1.f, sw + 1, st));
        SID_TRY(scale_ratio_dev(sw + 1, x.dscale, 1.f, sw + 2, st));
        npass = !split ? 1 : (x.lo ? 3 : 2);
        dalpha = sw + 2;
    } else {
        SID_TRY(split16(W, k, n, ldw, wh, nullptr, true, 1.f, st));
    }
    // a split-K epilogue goes through a P x n workspace (the scale is applied as the tiles are stored)
    const int64_t ws_elems = sk > 1 ? (int64_t)sk * P * n : 1;
    SID_TRY(c->ws.alloc((size_t)ws_elems * sizeof(float)));
    return gemm_tn_ds(As, Bs, npass, P, n, k, !x.f16, C, P, 1.f, dalpha, 0.f, bn, sk, c->ws.as<float>(),
                      (int64_t)(c->ws.bytes / sizeof(float)), c->errflag.as<int>(), st);
}

}  // namespace sid

extern "C" int sid_s_update(sid_ctx* c, const void* Y, int ydtype, float* S, float* T, int64_t P, int64_t R,
                            int64_t F, const float* ymean, const float* hilf, const sid_nmf_opts* o, int prec,
                            void* stream)
{
    SID_TRY(nmf_checks(c, Y, ydtype, S, T, P, R, F, o, prec, "S_update"));
    SID_REQUIRE(!o->use_std || ymean, "S_update: use_std needs opts.Y (ymean)");
    SID_REQUIRE(o->lamb_orth_L1 == 0.0 && o->lamb_orth_L2 == 0.0 ? true : hilf != nullptr,
                "S_update: the orthogonality penalties need opts.hilf");
    SID_REQUIRE(o->lamb_spat_TV == 0.0,
                "S_update: lamb_spat_TV is not supported (the reference's spatial TV term calls an undefined "
                "'laplace')");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t PR = P * R, RF = R * F;
    const bool orth = (o->lamb_orth_L1 + o->lamb_orth_L2) > 0;
    DBuf* b = c->mf;
    SID_TRY(b[0].alloc((size_t)(R * R) * 4 * 4));  // Q_T, Q_T', S'S, M1'
    SID_TRY(b[1].alloc((size_t)RF * 4));           // T'
    SID_REQUIRE(R <= 65535, "S_update: at most 65535 components");
    SID_TRY(b[2].alloc((size_t)(3 * R + 2 * kRedBlocks + 8) * 8));
    SID_TRY(b[3].alloc((size_t)(P + 1) * 4));      // alpha
    SID_TRY(b[4].alloc((size_t)PR * 4 * 3));       // q_S / vQ, df, v
    float* QT = b[0].as<float>();
    float* QTt = QT + R * R;
    float* SS = QTt + R * R;
    float* M1t = SS + R * R;
    float* Tt = b[1].as<float>();
    double* ts = b[2].as<double>();
    double* sq = ts + R;
    double* part = sq + R;
    float* pl = reinterpret_cast<float*>(part + 2 * kRedBlocks + 8);  // column norms
    float* alpha = b[3].as<float>();
    float* qS = b[4].as<float>();
    float* df = qS + PR;
    float* v = df + PR;

    k_nan_zero<<<grid_for(RF), 256, 0, st>>>(T, RF);
    k_nan_zero<<<grid_for(PR), 256, 0, st>>>(S, PR);
    SID_CHECK_LAUNCH();
    // Q_T = T T', q_S = Y T'  (S_update.m:8-9)
    SID_TRY(transpose(T, R, F, Tt, st));
    SID_TRY(tn32(c, Tt, Tt, R, R, F, F, F, QT, st));
    // pixel-long-by-rank products on the tensor cores except at FP32 precision
    const bool tc = prec != SID_PREC_FP32;
    PixOperand Sx{};
    if (tc) {
        PixOperand Yx{};
        SID_TRY(pix_operand(c, 0, Y, ydtype == SID_DTYPE_F16, P, F, prec, &Yx, st));
        SID_TRY(gemm_pix(c, Yx, P, F, Tt, R, F, qS, prec, st));
        SID_TRY(pix_operand(c, 1, S, false, P, R, prec, &Sx, st));
    } else {
        SID_TRY(sgemm_nt(Y, ydtype == SID_DTYPE_F16 ? 1 : 0, T, P, R, F, P, R, qS, P, st));
    }
    // use_std (S_update.m:11-15), orthogonality L1 (:19-21)
    const double invF = 1.0 / (double)F;
    if (o->use_std) {
        k_row_moments<<<(unsigned)cdiv(R * 32, 256), 256, 0, st>>>(T, (int)R, F, ts, nullptr);
        SID_CHECK_LAUNCH();
    }
    if (o->use_std || o->lamb_orth_L1 != 0.0) {
        k_qt_adjust<<<grid_for(R * R), 256, 0, st>>>(QT, (int)R, o->use_std ? ts : nullptr, invF,
                                                     o->lamb_orth_L1 != 0.0 ? hilf : nullptr, o->lamb_orth_L1);
        SID_CHECK_LAUNCH();
    }
    SID_TRY(transpose(QT, R, R, QTt, st));
    // df_S = -q_S + S*Q_T + lamb_spat  (:32)
    if (tc) SID_TRY(gemm_pix(c, Sx, P, R, QT, R, R, df, prec, st));
    else SID_TRY(sgemm_nt(S, 0, QTt, P, R, R, P, R, df, P, st));
    k_s_grad<<<grid_cols(P, R), 256, 0, st>>>(qS, df, P, o->use_std ? ymean : nullptr, ts, invF, o->lamb_spat);
    SID_CHECK_LAUNCH();
    // direction (:38-53); M2 = S*(hilf*(S'*S)) for the L2 orthogonality term, in the q_S buffer
    const float* M2 = nullptr;
    if (orth && o->lamb_orth_L2 != 0.0) {
        SID_TRY(contract(c, S, S, false, R, R, P, P, P, SS, R, 1.f, 0.f, prec, st));
        SID_TRY(b[5].alloc((size_t)(R * R) * 4 * 2));
        float* hT = b[5].as<float>();  // hilf'
        float* M1 = hT + R * R;        // hilf * (S'S)
        SID_TRY(transpose(hilf, R, R, hT, st));
        SID_TRY(tn32(c, hT, SS, R, R, R, R, R, M1, st));
        SID_TRY(transpose(M1, R, R, M1t, st));
        if (tc) SID_TRY(gemm_pix(c, Sx, P, R, M1, R, R, qS, prec, st));
        else SID_TRY(sgemm_nt(S, 0, M1t, P, R, R, P, R, qS, P, st));
        M2 = qS;
    }
    k_s_dir<<<grid_for(P), 256, 0, st>>>(S, df, M2, (float)o->lamb_orth_L2, orth ? 1 : 0, P, (int)R, v);
    SID_CHECK_LAUNCH();
    // exact line search (:57-68): vQ = v*Q_T into the q_S buffer
    if (tc) {
        PixOperand Vx{};
        SID_TRY(pix_operand(c, 0, v, false, P, R, prec, &Vx, st));
        SID_TRY(gemm_pix(c, Vx, P, R, QT, R, R, qS, prec, st));
    } else {
        SID_TRY(sgemm_nt(v, 0, QTt, P, R, R, P, R, qS, P, st));
    }
    if (o->pointwise) {
        k_s_sums<<<grid_for(P), 256, 0, st>>>(v, df, qS, P, (int)R, 1, alpha, part);
    } else {
        k_s_sums<<<kRedBlocks, 256, 0, st>>>(v, df, qS, P, (int)R, 0, alpha, part);
        k_alpha<<<1, 256, 0, st>>>(part, part + kRedBlocks, kRedBlocks, 0, o->lamb_orth_L2 != 0.0 ? 1e-6 : 0.0,
                                   alpha);
    }
    k_pg_step_cols<<<grid_cols(P, R), 256, 0, st>>>(S, v, P, alpha, o->pointwise ? 1 : 0);
    SID_CHECK_LAUNCH();
    // unit-norm columns of S, T rescaled (:75-79)
    if (orth) {
        k_col_norm2<<<(unsigned)R, 256, 0, st>>>(S, P, sq, pl);
        k_unit_cols_s<<<grid_cols(P, R), 256, 0, st>>>(S, P, pl);
        k_unit_rows_t<<<grid_for(RF), 256, 0, st>>>(T, (int)R, F, pl);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}
