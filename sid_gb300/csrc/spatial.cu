// spatial.cu -- SID spatial update: per-pixel regularised NNLS
// (update_spatial_component.m:45-131 -> reg_nnls.m:40-69 -> NQP.m:42-178).
//
// The reference loops over neurons (ascending template size) and, for every
// not-yet-visited pixel of the neuron's template, solves a small non-negative
// quadratic program over the neurons whose templates cover that pixel (plus the
// background component).  Which neurons enter a pixel's problem depends only
// on the original template (a pixel is solved once, by the first neuron that
// reaches it, with every neuron covering it), so all pixel problems are
// independent and run here in one launch:
//   1. G = T T' (R x R, FP32) and C = Y T' (P x R, tensor cores, FP16 hi/lo
//      operands, FP32 accumulation)  -- contractions;
//   2. per pixel: ||y||, sum(y), and the covering neurons in ascending order,
//      background last (update_spatial_component.m:59-79);
//   3. per pixel, FP64: Q = G(idx,idx) + l2*I + lo*hilf [- s s'/F],
//      q = -C(p,idx)/||y|| + l1 [+ s sum(y)/(F ||y||)] (reg_nnls.m:48-67),
//      Lawson-Hanson active set with an incrementally extended Cholesky factor
//      (NQP.m:93-178, default options), x * ||y|| into the forward model;
//   4. pixels outside every template get the background row C(p, bg)
//      (update_spatial_component.m:128-131).
#include <algorithm>
#include <cfloat>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st);
int ctx_sync(sid_ctx* c, cudaStream_t st);
int pix_operand(sid_ctx* c, int slot, const void* X, bool x_f16, int64_t P, int64_t k, int prec, PixOperand* op,
                cudaStream_t st);
int gemm_pix(sid_ctx* c, const PixOperand& x, int64_t P, int64_t k, const float* W, int64_t n, int64_t ldw,
             float* C, int prec, cudaStream_t st);

constexpr int kNqpMax = 32;          // components per problem solved with local working arrays
constexpr int kNqpLargeMax = 4096;   // sid_nqp_batched's largest n (scratch working arrays above kNqpMax)

// --------------------------------------------- C = Y T' (FP32, NT layout) --
// C (m x n, col-major) = A B' with A m x k (m contiguous) and B n x k (n
// contiguous): the frame contraction of a pixel-major movie.  128 x 64 tile,
// 256 threads, 8 x 4 outputs per thread.
__global__ void __launch_bounds__(256)
k_sgemm_nt(const float* __restrict__ A, const void* __restrict__ Bv, const float* __restrict__ Bscale, int m, int n,
           int k, int64_t lda, int64_t ldb, float* __restrict__ C, int64_t ldc, int a_f16)
{
    __shared__ __align__(16) float As[16][128];
    __shared__ __align__(16) float Bs[16][64];
    const float* B = static_cast<const float*>(Bv);
    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 64;
    const int tm = (tid & 31) * 4, tn = (tid >> 5) * 8;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    (void)Bscale;
    for (int k0 = 0; k0 < k; k0 += 16) {
        for (int e = tid; e < 16 * 128; e += 256) {
            const int kk = e >> 7, mm = e & 127;
            const int gm = m0 + mm, gk = k0 + kk;
            float v = 0.f;
            if (gm < m && gk < k) {
                if (a_f16) v = __half2float(reinterpret_cast<const __half*>(A)[gm + lda * (int64_t)gk]);
                else v = A[gm + lda * (int64_t)gk];
            }
            As[kk][mm] = v;
        }
        for (int e = tid; e < 16 * 64; e += 256) {
            const int kk = e >> 6, nn = e & 63;
            const int gn = n0 + nn, gk = k0 + kk;
            Bs[kk][nn] = (gn < n && gk < k) ? B[gn + ldb * (int64_t)gk] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            const float4 a = *reinterpret_cast<const float4*>(&As[kk][tm]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tn]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][tn + 4]);
            const float av[4] = {a.x, a.y, a.z, a.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = m0 + tm + i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = n0 + tn + j;
            if (c < n) C[(int64_t)r + ldc * c] = acc[i][j];
        }
    }
}

// C (m x n) = A B' with A m x k (FP32 or FP16, m contiguous) and B n x k (FP32,
// n contiguous); no split-K (the callers' m is the pixel count).
int sgemm_nt(const void* A, int a_f16, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb,
             float* C, int64_t ldc, cudaStream_t st)
{
    SID_REQUIRE(m > 0 && n > 0 && k > 0, "sgemm_nt: empty problem");
    SID_REQUIRE(m < INT32_MAX && n < INT32_MAX && k < INT32_MAX, "sgemm_nt: dimension too large");
    dim3 grid((unsigned)cdiv(m, 128), (unsigned)cdiv(n, 64));
    k_sgemm_nt<<<grid, 256, 0, st>>>(static_cast<const float*>(A), B, nullptr, (int)m, (int)n, (int)k, lda, ldb, C,
                                     ldc, a_f16);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Tt (F x R, column-major) = T' for T (R x F)
__global__ void k_transpose(const float* __restrict__ T, int R, int F, float* __restrict__ Tt)
{
    const int64_t n = (int64_t)R * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = i % F, r = i / F;
        Tt[i] = T[r + (int64_t)R * f];
    }
}

// per pixel: ||y||, sum(y) (movie P x F, pixel-major)
__global__ void k_pixel_stats(const void* __restrict__ Y, int f16, int64_t P, int64_t F, float* __restrict__ nrm,
                              float* __restrict__ sum)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0;
        for (int64_t f = 0; f < F; ++f) {
            const double v = f16 ? (double)__half2float(static_cast<const __half*>(Y)[p + P * f])
                                 : (double)static_cast<const float*>(Y)[p + P * f];
            s += v;
            q += v * v;
        }
        nrm[p] = (float)sqrt(q);
        sum[p] = (float)s;
    }
}

// s(r) = sum over frames of T(r, :)
__global__ void k_row_sums(const float* __restrict__ T, int R, int F, float* __restrict__ s)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int f = 0; f < F; ++f) a += T[r + (int64_t)R * f];
        s[r] = (float)a;
    }
}

struct SpatialOpts {
    double l1, l2, lo;  // lamb_L1, lamb_L2, lamb_orth_L1
    int use_std, bg_sub;
};

// Lawson-Hanson active set with an incremental Cholesky factor of the passive
// block (NQP.m:93-178, default options, FP64): argmin_{x >= 0} 0.5 x'Qx - b'x
// for n <= kNqpMax.  Qij(i, j) returns Q(i, j); b is NQP's internal right-hand
// side (minus the linear term); w receives the final w = b - Q x.  Returns 0,
// or 2 at the iteration cap (NQP.m:116-119); *iters = iterations taken.
// Working arrays of one solve: z, wsc, t (n each), L (packed lower triangle,
// row-major, n(n+1)/2), pn (n ints), Pset (n flags).  Problems with n <=
// kNqpMax keep them in the thread's local arrays; larger ones in a slice of a
// global scratch buffer.
struct NqpWs {
    double *z, *wsc, *t, *L;
    int* pn;
    uint8_t* Pset;
};

// Scratch of one large problem (n <= nm), in doubles: L, z, wsc, t, b, x, w,
// then pn and idx (nm ints each) and Pset (nm bytes).
__host__ __device__ inline int64_t nqp_scratch_doubles(int64_t nm) { return nm * (nm + 1) / 2 + 6 * nm + nm + nm / 8 + 2; }

__device__ inline NqpWs nqp_ws_at(double* base, int nm, double** b, double** x, double** w, int** idx)
{
    NqpWs ws;
    ws.L = base;
    double* d = base + (int64_t)nm * (nm + 1) / 2;
    ws.z = d;
    ws.wsc = d + nm;
    ws.t = d + 2 * nm;
    *b = d + 3 * nm;
    *x = d + 4 * nm;
    *w = d + 5 * nm;
    ws.pn = reinterpret_cast<int*>(d + 6 * nm);
    *idx = ws.pn + nm;
    ws.Pset = reinterpret_cast<uint8_t*>(*idx + nm);
    return ws;
}

template <class QF>
__device__ int nqp_solve(int n, const QF& Qij, const double* b, double* x, double* w, const NqpWs& ws, int* iters)
{
    double* z = ws.z;
    double* wsc = ws.wsc;
    double* t = ws.t;
    double* L = ws.L;
    int* pn = ws.pn;
    uint8_t* Pset = ws.Pset;
    for (int i = 0; i < n; ++i) {
        w[i] = b[i];  // w = -b_input, NQP.m:122
        x[i] = 0.0;
        wsc[i] = 0.0;
        Pset[i] = 0;
    }
    const double tol = 3.0 * DBL_EPSILON;
    double wsc0 = 0.0;
    for (int i = 0; i < n; ++i) wsc0 += w[i] * w[i];
    wsc0 = sqrt(wsc0);
    const int maxiter = 4 * n;
    int pn1 = 0, pn2 = 0, iter = 0, st = 0;
#define LIJ(r, c) L[(r) * ((r) + 1) / 2 + (c)]
    for (;;) {
        bool all_p = true, any_up = false;
        for (int i = 0; i < n; ++i)
            if (!Pset[i]) {
                all_p = false;
                if (w[i] > wsc[i]) any_up = true;
            }
        if (all_p || !any_up) break;
        int best = -1;
        double bv = 0.0;
        for (int i = 0; i < n; ++i) {
            if (Pset[i]) continue;
            const double v = w[i] - wsc[i];
            if (best < 0 || v > bv) { best = i; bv = v; }
        }
        Pset[best] = 1;
        pn2 = pn1 + 1;
        pn[pn2 - 1] = best;
        for (;;) {
            ++iter;
            if (iter >= 2 * n) {
                if (iter > maxiter) { st = 2; goto done; }
                if (iter % n == 0)
                    for (int i = 0; i < n; ++i) wsc[i] = (wsc[i] + wsc0 * tol) * 2.0;
            }
            for (int i = 0; i < n; ++i) z[i] = 0.0;
            for (int r = pn1; r < pn2; ++r) {
                const int vr = pn[r];
                for (int s = 0; s < r; ++s) {
                    double acc = Qij(pn[s], vr);
                    for (int u = 0; u < s; ++u) acc -= LIJ(s, u) * t[u];
                    t[s] = acc / LIJ(s, s);
                }
                const double AA = Qij(vr, vr);
                double tt = AA;
                for (int s = 0; s < r; ++s) tt -= t[s] * t[s];
                tt = (tt <= AA * tol) ? 1e300 : sqrt(tt);
                for (int s = 0; s < r; ++s) LIJ(r, s) = t[s];
                LIJ(r, r) = tt;
            }
            for (int s = 0; s < pn2; ++s) {
                double acc = b[pn[s]];
                for (int u = 0; u < s; ++u) acc -= LIJ(s, u) * t[u];
                t[s] = acc / LIJ(s, s);
            }
            for (int s = pn2 - 1; s >= 0; --s) {
                double acc = t[s];
                for (int u = s + 1; u < pn2; ++u) acc -= LIJ(u, s) * z[pn[u]];
                z[pn[s]] = acc / LIJ(s, s);
            }
            pn1 = pn2;
            bool all_pos = true;
            for (int i = 0; i < n; ++i)
                if (Pset[i] && z[i] < 0.0) { all_pos = false; break; }
            if (all_pos) {
                for (int i = 0; i < n; ++i) x[i] = z[i];
                for (int i = 0; i < n; ++i) {
                    double acc = b[i];
                    for (int u = 0; u < n; ++u) acc -= Qij(i, u) * x[u];
                    w[i] = acc;
                }
                for (int i = 0; i < n; ++i)
                    if (Pset[i] && 2.0 * fabs(w[i]) > wsc[i]) wsc[i] = 2.0 * fabs(w[i]);
                break;
            }
            int worst = -1;
            double alpha = 0.0;
            for (int i = 0; i < n; ++i) {
                if (!(z[i] < 0.0)) continue;
                const double v = x[i] / (x[i] - z[i] + DBL_MIN);
                if (worst < 0 || v < alpha) { worst = i; alpha = v; }
            }
            if (x[worst] == 0.0) {
                double acc = b[worst];
                for (int u = 0; u < n; ++u) acc -= Qij(worst, u) * x[u];
                wsc[worst] = (fabs(acc) + wsc[worst]) * 2.0;
                w[worst] = acc;
            }
            Pset[worst] = 0;
            for (int i = 0; i < n; ++i) x[i] = x[i] - alpha * (x[i] - z[i]);
            int pos = 0;
            while (pn[pos] != worst) ++pos;
            for (int s = pos; s + 1 < pn2; ++s) pn[s] = pn[s + 1];
            pn1 = pos;
            pn2 = pn2 - 1;
        }
    }
done:
#undef LIJ
    *iters = iter;
    return st;
}

struct PixelArgs {
    const uint8_t* tmpl;
    int Rt;
    int64_t P;
    const float* G;
    int R;
    const float* C;
    int64_t ldc;
    const float *pnrm, *psum, *tsum;
    int F;
    SpatialOpts o;
    float* out;
    int* status;
    int* nfail;
};

// Solve pixel p's problem over the components idx[0..n) (background last when
// bg_sub): Q(i,j) and b = -q (NQP works with b = -q, NQP.m:145), reg_nnls.m:48-67.
__device__ void pixel_solve(const PixelArgs& a, int64_t p, const int* idx, int n, double* b, double* x, double* w,
                            const NqpWs& ws)
{
    const SpatialOpts& o = a.o;
    const double yn = (double)a.pnrm[p];
    if (!(yn > 0.0)) {
        for (int i = 0; i < n; ++i) a.out[idx[i] + (int64_t)a.R * p] = 0.f;
        a.status[p] = 0;
        return;
    }
    auto Qij = [&](int i, int j) -> double {
        double v = (double)a.G[idx[i] + (int64_t)a.R * idx[j]];
        if (i == j) v += o.l2;
        else if (!(o.bg_sub && (i == n - 1 || j == n - 1))) v += o.lo;  // hilf = ones - eye, bg row/col zero
        if (o.use_std) v -= (double)a.tsum[idx[i]] * (double)a.tsum[idx[j]] / (double)a.F;
        return v;
    };
    for (int i = 0; i < n; ++i) {
        double q = -(double)a.C[p + a.ldc * idx[i]] / yn;
        if (o.use_std) q += (double)a.tsum[idx[i]] * (double)a.psum[p] / yn / (double)a.F;
        q += o.l1;
        b[i] = -q;
    }
    int iters = 0;
    const int st = nqp_solve(n, Qij, b, x, w, ws, &iters);
    a.status[p] = st;
    if (st) {
        atomicAdd(a.nfail, 1);
        return;
    }
    for (int i = 0; i < n; ++i) a.out[idx[i] + (int64_t)a.R * p] = (float)(x[i] * yn);
}

// One thread per pixel: collect the covering components and solve the NQP in
// FP64 with the working arrays in registers / local memory.  A pixel covered by
// more than kNqpMax components is put on the large-problem list (status 3
// until k_pixel_nqp_large solves it); nlarge[0] counts them, nlarge[1] keeps
// the largest n.  status[p]: 0 ok, 2 iteration cap (NQP.m:116-119).
__global__ void __launch_bounds__(128)
k_pixel_nqp(PixelArgs a, int* __restrict__ large, int* __restrict__ nlarge)
{
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    int idx[kNqpMax];
    int n = 0;
    for (int r = 0; r < a.Rt; ++r) {
        if (a.tmpl[r + (int64_t)a.Rt * p]) {
            if (n < kNqpMax) idx[n] = r;
            ++n;
        }
    }
    if (n == 0) {
        // outside every template: background row, if any (update_spatial_component.m:128-131)
        if (a.o.bg_sub) a.out[(a.R - 1) + (int64_t)a.R * p] = a.C[p + a.ldc * (a.R - 1)];
        a.status[p] = 0;
        return;
    }
    if (a.o.bg_sub) {
        if (n < kNqpMax) idx[n] = a.R - 1;
        ++n;
    }
    if (n > kNqpMax) {
        const int pos = atomicAdd(&nlarge[0], 1);
        large[pos] = (int)p;
        atomicMax(&nlarge[1], n);
        a.status[p] = 3;
        return;
    }
    double z[kNqpMax], wsc[kNqpMax], t[kNqpMax], L[kNqpMax * (kNqpMax + 1) / 2];
    int pn[kNqpMax];
    uint8_t Pset[kNqpMax];
    const NqpWs ws{z, wsc, t, L, pn, Pset};
    double b[kNqpMax], x[kNqpMax], w[kNqpMax];
    pixel_solve(a, p, idx, n, b, x, w, ws);
}

// Pixels of the large-problem list large[off .. off+cnt): one thread each,
// working arrays in a slice of `scratch` sized for nm components.
__global__ void __launch_bounds__(128)
k_pixel_nqp_large(PixelArgs a, const int* __restrict__ large, int off, int cnt, int nm, double* __restrict__ scratch)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cnt) return;
    const int64_t p = large[off + e];
    double *b, *x, *w;
    int* idx;
    const NqpWs ws = nqp_ws_at(scratch + (int64_t)e * nqp_scratch_doubles(nm), nm, &b, &x, &w, &idx);
    int n = 0;
    for (int r = 0; r < a.Rt; ++r)
        if (a.tmpl[r + (int64_t)a.Rt * p] && n < nm) idx[n++] = r;
    if (a.o.bg_sub && n < nm) idx[n++] = a.R - 1;
    pixel_solve(a, p, idx, n, b, x, w, ws);
}

// One thread per problem k: Q (n x n, column-major, FP64) at Q + n*n*k, the
// linear term at q + n*k; x and w (optional) n x B; NQP's [x, w, info]
// (NQP.m:42-178) for independent problems of one size.  n <= kNqpMax keeps
// the working arrays in local memory (scratch == nullptr); larger n uses a
// slice of `scratch` per problem, for problems k0 .. k0+cnt.
__global__ void __launch_bounds__(128) k_nqp_batched(const double* __restrict__ Q, const double* __restrict__ q,
                                                     int n, int64_t k0, int64_t cnt, double* __restrict__ x,
                                                     double* __restrict__ w, int32_t* __restrict__ iters,
                                                     int32_t* __restrict__ status, int* __restrict__ nfail,
                                                     double* __restrict__ scratch)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= cnt) return;
    const int64_t k = k0 + e;
    const double* Qk = Q + (int64_t)n * n * k;
    auto Qij = [&](int i, int j) -> double { return Qk[i + (int64_t)n * j]; };
    double zl[kNqpMax], wscl[kNqpMax], tl[kNqpMax], Ll[kNqpMax * (kNqpMax + 1) / 2];
    int pnl[kNqpMax];
    uint8_t Psl[kNqpMax];
    double bl[kNqpMax], xl[kNqpMax], wl[kNqpMax];
    double *bb = bl, *xx = xl, *ww = wl;
    NqpWs ws{zl, wscl, tl, Ll, pnl, Psl};
    if (scratch) {
        int* idx;
        ws = nqp_ws_at(scratch + e * nqp_scratch_doubles(n), n, &bb, &xx, &ww, &idx);
    }
    for (int i = 0; i < n; ++i) bb[i] = -q[i + (int64_t)n * k];  // NQP works with b = -q (NQP.m:145)
    int it = 0;
    const int st = nqp_solve(n, Qij, bb, xx, ww, ws, &it);
    for (int i = 0; i < n; ++i) {
        x[i + (int64_t)n * k] = xx[i];
        if (w) w[i + (int64_t)n * k] = ww[i];
    }
    if (iters) iters[k] = it;
    if (status) status[k] = st;
    if (st) atomicAdd(nfail, 1);
}

// reg_nnls.m:40-66: Q = A'A [- t t'/m] + l2 I + lo hilf, q = -A'd [+ t sum(d)/m] + l1,
// t = column sums of A (use_std); one CTA per entry of Q (and per entry of q,
// row n of the grid), FP64 sums over the m rows.  Q n x n and q n, column-major.
__global__ void __launch_bounds__(256) k_reg_form(const double* __restrict__ A, int64_t m, int n,
                                                  const double* __restrict__ d, double l1, double l2, double lo,
                                                  int use_std, int bg_sub, const double* __restrict__ hilf,
                                                  double* __restrict__ Q, double* __restrict__ q)
{
    __shared__ double red[3][8];
    const int i = blockIdx.x, j = blockIdx.y;  // j == n: the linear term of row i
    const double* ai = A + (int64_t)i * m;
    const double* bj = (j < n) ? A + (int64_t)j * m : d;
    double s = 0.0, si = 0.0, sj = 0.0;
    for (int64_t r = threadIdx.x; r < m; r += blockDim.x) {
        const double a = ai[r], b = bj[r];
        s = fma(a, b, s);
        si += a;
        sj += b;
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, off);
        si += __shfl_xor_sync(0xffffffffu, si, off);
        sj += __shfl_xor_sync(0xffffffffu, sj, off);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s;
        red[1][threadIdx.x >> 5] = si;
        red[2][threadIdx.x >> 5] = sj;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    s = si = sj = 0.0;
    for (int w = 0; w < 8; ++w) {
        s += red[0][w];
        si += red[1][w];
        sj += red[2][w];
    }
    if (use_std) s -= si * sj / (double)m;
    if (j < n) {
        if (i == j) s += l2;
        const double h = hilf ? hilf[i + (int64_t)n * j]
                              : ((i == j || (bg_sub && (i == n - 1 || j == n - 1))) ? 0.0 : 1.0);
        s += lo * h;
        Q[i + (int64_t)n * j] = s;
    } else {
        q[i] = -s + l1;
    }
}

// problems of nm components whose scratch fits in the budget (at least one)
inline int64_t nqp_chunk(int64_t total, int64_t nm)
{
    const int64_t budget = (int64_t)1 << 30;  // bytes of scratch per launch
    return std::max<int64_t>(1, std::min<int64_t>(total, budget / (nqp_scratch_doubles(nm) * 8)));
}

}  // namespace sid

using namespace sid;

extern "C" int sid_spatial_update(sid_ctx* c, const float* T, const void* Y, int ydtype, const uint8_t* tmpl,
                                  int64_t R, int64_t F, int64_t P, double lamb_L1, double lamb_L2,
                                  double lamb_orth_L1, int use_std, int bg_sub, float* forward_model,
                                  int32_t* status, void* stream)
{
    SID_REQUIRE(c && T && Y && tmpl && forward_model, "sid_spatial_update: NULL argument");
    SID_REQUIRE(R >= 1 && F >= 1 && P >= 1, "sid_spatial_update: empty problem");
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "sid_spatial_update: unknown Y dtype");
    SID_REQUIRE(!bg_sub || R >= 2, "sid_spatial_update: bg_sub needs a background component");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t Rt = bg_sub ? R - 1 : R;
    DBuf* nn = c->nn;
    SID_TRY(nn[0].alloc((size_t)(F * R) * 4));   // T'
    SID_TRY(nn[1].alloc((size_t)(R * R) * 4));   // G
    SID_TRY(nn[2].alloc((size_t)(P * R) * 4));   // C = Y T'
    SID_TRY(nn[3].alloc((size_t)(2 * P + R + 4) * 4));
    SID_TRY(nn[4].alloc((size_t)P * 4));         // status (when the caller passes none)
    float* Tt = nn[0].as<float>();
    float* G = nn[1].as<float>();
    float* Cm = nn[2].as<float>();
    float* pn = nn[3].as<float>();
    float* ps = pn + P;
    float* ts = ps + P;
    int* nfail = reinterpret_cast<int*>(ts + R);
    int* stat = status ? status : nn[4].as<int>();
    k_transpose<<<1024, 256, 0, st>>>(T, (int)R, (int)F, Tt);
    SID_CHECK_LAUNCH();
    // G = T T' (contraction over frames)
    SID_TRY(contract(c, Tt, Tt, false, R, R, F, F, F, G, R, 1.f, 0.f, SID_PREC_FP32, st));
    // C = Y T' (P x R) on the tensor cores: the pixel-major movie brought once into
    // the GEMM's K-blocked layout (an FP16 movie as it is, an FP32 one as FP16
    // hi/lo), T' as FP16 hi/lo with a power-of-two scale; FP32 accumulation
    PixOperand yop;
    SID_TRY(pix_operand(c, 0, Y, ydtype == SID_DTYPE_F16, P, F, SID_PREC_SPLIT, &yop, st));
    SID_TRY(gemm_pix(c, yop, P, F, Tt, R, F, Cm, SID_PREC_SPLIT, st));
    k_pixel_stats<<<1024, 256, 0, st>>>(Y, ydtype == SID_DTYPE_F16 ? 1 : 0, P, F, pn, ps);
    SID_CHECK_LAUNCH();
    k_row_sums<<<cdiv(R, 256), 256, 0, st>>>(T, (int)R, (int)F, ts);
    SID_CHECK_LAUNCH();
    SID_CUDA_TRY(cudaMemsetAsync(forward_model, 0, (size_t)(R * P) * 4, st));
    SID_CUDA_TRY(cudaMemsetAsync(nfail, 0, sizeof(int), st));
    SpatialOpts o{lamb_L1, lamb_L2, lamb_orth_L1, use_std ? 1 : 0, bg_sub ? 1 : 0};
    PixelArgs pa{tmpl, (int)Rt, P, G, (int)R, Cm, P, pn, ps, ts, (int)F, o, forward_model, stat, nfail};
    SID_TRY(nn[5].alloc((size_t)P * 4 + 16));  // large-problem list, then its count and largest n
    int* large = nn[5].as<int>();
    int* nlarge = reinterpret_cast<int*>(nn[5].as<uint8_t>() + (size_t)P * 4);
    SID_CUDA_TRY(cudaMemsetAsync(nlarge, 0, 2 * sizeof(int), st));
    k_pixel_nqp<<<(unsigned)cdiv(P, 128), 128, 0, st>>>(pa, large, nlarge);
    SID_CHECK_LAUNCH();
    int hl[2] = {0, 0};
    SID_CUDA_TRY(cudaMemcpyAsync(hl, nlarge, sizeof(hl), cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    if (hl[0] > 0) {
        // pixels covered by more than kNqpMax components: working arrays in global scratch
        const int nm = hl[1];
        const int64_t chunk = nqp_chunk(hl[0], nm);
        SID_TRY(nn[6].alloc((size_t)(chunk * nqp_scratch_doubles(nm)) * 8));
        for (int64_t off = 0; off < hl[0]; off += chunk) {
            const int cnt = (int)std::min<int64_t>(chunk, hl[0] - off);
            k_pixel_nqp_large<<<(unsigned)cdiv(cnt, 128), 128, 0, st>>>(pa, large, (int)off, cnt, nm,
                                                                          nn[6].as<double>());
            SID_CHECK_LAUNCH();
        }
    }
    int hf = 0;
    SID_CUDA_TRY(cudaMemcpyAsync(&hf, nfail, sizeof(int), cudaMemcpyDeviceToHost, st));
    SID_TRY(ctx_sync(c, st));
    if (hf) {
        set_error("sid_spatial_update: %d pixel problems hit the NQP iteration cap of NQP.m:116-119; see the "
                  "status array",
                  hf);
        return SID_ENOCONV;
    }
    return SID_OK;
}

extern "C" int sid_nqp_batched(sid_ctx* c, const double* Q, const double* q, int n, int64_t B, double* x, double* w,
                               int32_t* iters, int32_t* status, void* stream)
{
    SID_REQUIRE(c && Q && q && x, "sid_nqp_batched: NULL argument");
    SID_REQUIRE(n >= 1 && n <= kNqpLargeMax, "sid_nqp_batched: n = %d outside [1, %d]", n, kNqpLargeMax);
    SID_REQUIRE(B >= 1, "sid_nqp_batched: no problems");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SID_TRY(c->scal.alloc(64));
    int* nfail = c->scal.as<int>();
    SID_CUDA_TRY(cudaMemsetAsync(nfail, 0, sizeof(int), st));
    if (n <= kNqpMax) {
        k_nqp_batched<<<(unsigned)cdiv(B, 128), 128, 0, st>>>(Q, q, n, 0, B, x, w, iters, status, nfail, nullptr);
        SID_CHECK_LAUNCH();
    } else {
        const int64_t chunk = nqp_chunk(B, n);
        SID_TRY(c->nn[13].alloc((size_t)(chunk * nqp_scratch_doubles(n)) * 8));
        for (int64_t k0 = 0; k0 < B; k0 += chunk) {
            const int64_t cnt = std::min<int64_t>(chunk, B - k0);
            k_nqp_batched<<<(unsigned)cdiv(cnt, 128), 128, 0, st>>>(Q, q, n, k0, cnt, x, w, iters, status, nfail,
                                                                     c->nn[13].as<double>());
            SID_CHECK_LAUNCH();
        }
    }
    int hf = 0;
    SID_CUDA_TRY(cudaMemcpyAsync(&hf, nfail, sizeof(int), cudaMemcpyDeviceToHost, st));
    SID_TRY(ctx_sync(c, st));
    if (hf) {
        set_error("nnls Failed to converge: %d of %lld problems hit the NQP iteration cap (NQP.m:116-119)", hf,
                  (long long)B);
        return SID_ENOCONV;
    }
    return SID_OK;
}

extern "C" int sid_reg_nnls(sid_ctx* c, const double* A, int64_t m, int n, const double* d, double lamb_L1,
                            double lamb_L2, double lamb_orth_L1, int use_std, int bg_sub, const double* hilf,
                            double* x, void* stream)
{
    SID_REQUIRE(c && A && d && x, "sid_reg_nnls: NULL argument");
    SID_REQUIRE(m >= 1 && n >= 1 && n <= kNqpLargeMax, "sid_reg_nnls: need m >= 1 and 1 <= n <= %d", kNqpLargeMax);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SID_TRY(c->nn[14].alloc((size_t)((int64_t)n * n + n) * 8));
    double* Q = c->nn[14].as<double>();
    double* q = Q + (int64_t)n * n;
    k_reg_form<<<dim3((unsigned)n, (unsigned)n + 1), 256, 0, st>>>(A, m, n, d, lamb_L1, lamb_L2, lamb_orth_L1,
                                                                  use_std ? 1 : 0, bg_sub ? 1 : 0, hilf, Q, q);
    SID_CHECK_LAUNCH();
    return sid_nqp_batched(c, Q, q, n, 1, x, nullptr, nullptr, nullptr, stream);
}
