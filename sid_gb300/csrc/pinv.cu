// pinv.cu -- least-squares timeseries extraction with the forward model's
// pseudo-inverse (incremental_temporal_update_gpu.m:76-100, LS branch):
//
//   Q = inv(F*F') * F            once   (:83-84)
//   T_chunk = Q * (Y_chunk ./ b) per chunk of frames (:66-68, 89, 99)
//
// F is the K x P forward model, Y a P x n chunk of frames, b the per-frame
// baseline.  Here G = F*F' is formed by the tensor-core contraction, factorised
// by an FP64 blocked Cholesky and inverted in FP64 (the reference inverts G
// too); each chunk then costs one contraction F*Y (K x n) and one FP64 product
// inv(G) * (F*Y).  This is the reference's product re-associated
// ((inv(G)*F)*Y = inv(G)*(F*Y)), which never forms the K x P matrix Q.
#include <cmath>
#include <cstring>

#include "sid_internal.cuh"

namespace sid {

int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st);

namespace {

constexpr int NB = 32;  // Cholesky / triangular-solve block

// out (cols x rows) = in' (FP32, column-major), 32 x 32 tiles
__global__ void k_transpose_f32(const float* __restrict__ in, int64_t rows, int64_t cols, float* __restrict__ out)
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

__global__ void k_widen(const float* __restrict__ in, int64_t n, double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// Factor the nb x nb diagonal block at (j0, j0) of A (K x K, lower) in place.
// One block of 256 threads, the block staged in shared memory.  A pivot that
// is not finite or not above kPivotTol times the original diagonal entry dg
// (a footprint that is zero or a combination of others: the pivot is then
// rounding noise) sets *err to its 1-based index.
constexpr double kPivotTol = 1e-10;

__global__ void k_chol_diag(double* __restrict__ A, int K, int j0, const double* __restrict__ dg,
                            int* __restrict__ err)
{
    __shared__ double s[NB][NB + 1];
    __shared__ int bad;
    const int nb = min(NB, K - j0);
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) {
        const int r = i % nb, c = i / nb;
        s[r][c] = A[(j0 + r) + (int64_t)K * (j0 + c)];
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int c = 0; c < nb; ++c) {
        if (threadIdx.x == 0) {
            const double d = s[c][c];
            if (!(d > kPivotTol * dg[j0 + c]) || !isfinite(d)) {
                bad = j0 + c + 1;
                s[c][c] = 1.0;
            } else {
                s[c][c] = sqrt(d);
            }
        }
        __syncthreads();
        const double d = s[c][c];
        for (int r = c + 1 + threadIdx.x; r < nb; r += blockDim.x) s[r][c] /= d;
        __syncthreads();
        // trailing update of the block's lower triangle
        const int m = nb - c - 1;
        for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
            const int r = c + 1 + i % m, q = c + 1 + i / m;
            if (r >= q) s[r][q] -= s[r][c] * s[q][c];
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) {
        const int r = i % nb, c = i / nb;
        A[(j0 + r) + (int64_t)K * (j0 + c)] = r >= c ? s[r][c] : 0.0;
    }
    if (threadIdx.x == 0 && bad && *err == 0) *err = bad;
}

// Panel below the diagonal block: L21 = A21 * inv(L11)'  (one thread per row)
__global__ void k_chol_panel(double* __restrict__ A, int K, int j0)
{
    __shared__ double L[NB][NB + 1];
    const int nb = min(NB, K - j0);
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) L[i % nb][i / nb] = A[(j0 + i % nb) + (int64_t)K * (j0 + i / nb)];
    __syncthreads();
    const int r = j0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= K) return;
    double x[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        if (c < nb) {
            double a = A[r + (int64_t)K * (j0 + c)];
            for (int q = 0; q < c; ++q) a -= x[q] * L[c][q];
            x[c] = a / L[c][c];
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) A[r + (int64_t)K * (j0 + c)] = x[c];
}

// Trailing update A22 -= L21 L21' on the lower tiles (32 x 32 tiles, 256 threads, 4 outputs each)
__global__ void k_chol_update(double* __restrict__ A, int K, int j0)
{
    const int nb = min(NB, K - j0);
    const int base = j0 + nb;
    const int tr = blockIdx.x, tc = blockIdx.y;
    if (tc > tr) return;
    __shared__ double Lr[32][NB + 1], Lc[32][NB + 1];
    const int r0 = base + tr * 32, c0 = base + tc * 32;
    for (int i = threadIdx.x; i < 32 * nb; i += blockDim.x) {
        const int a = i % 32, q = i / 32;
        Lr[a][q] = (r0 + a < K) ? A[(r0 + a) + (int64_t)K * (j0 + q)] : 0.0;
        Lc[a][q] = (c0 + a < K) ? A[(c0 + a) + (int64_t)K * (j0 + q)] : 0.0;
    }
    __syncthreads();
    const int lr = threadIdx.x % 32, lc0 = threadIdx.x / 32;
    for (int lc = lc0; lc < 32; lc += 8) {
        const int r = r0 + lr, c = c0 + lc;
        if (r >= K || c >= K || c > r) continue;
        double s = 0.0;
        for (int q = 0; q < nb; ++q) s += Lr[lr][q] * Lc[lc][q];
        A[r + (int64_t)K * c] -= s;
    }
}

// Forward substitution on the block rows [j0, j0+nb) of B (K x n, FP64):
// B1 = inv(L11) B1, then B2 -= L21 B1.  One thread per right-hand side.
__global__ void k_trsv_fwd(const double* __restrict__ L, int K, int j0, double* __restrict__ B, int n)
{
    __shared__ double s[NB][NB + 1];
    const int nb = min(NB, K - j0);
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) s[i % nb][i / nb] = L[(j0 + i % nb) + (int64_t)K * (j0 + i / nb)];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double* b = B + (int64_t)K * j + j0;
    double x[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        if (c < nb) {
            double a = b[c];
            for (int q = 0; q < c; ++q) a -= s[c][q] * x[q];
            x[c] = a / s[c][c];
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) b[c] = x[c];
}

// B2 (rows below the block) -= L21 * B1   (one thread per (row, rhs))
__global__ void k_trsm_below(const double* __restrict__ L, int K, int j0, double* __restrict__ B, int n)
{
    const int nb = min(NB, K - j0);
    const int64_t rows = K - j0 - nb;
    const int64_t total = rows * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = j0 + nb + (int)(i % rows);
        const int64_t j = i / rows;
        double a = 0.0;
        for (int q = 0; q < nb; ++q) a += L[r + (int64_t)K * (j0 + q)] * B[(j0 + q) + (int64_t)K * j];
        B[r + (int64_t)K * j] -= a;
    }
}

// Backward substitution on block rows [j0, j0+nb): B1 = inv(L11') B1.
__global__ void k_trsv_bwd(const double* __restrict__ L, int K, int j0, double* __restrict__ B, int n)
{
    __shared__ double s[NB][NB + 1];
    const int nb = min(NB, K - j0);
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) s[i % nb][i / nb] = L[(j0 + i % nb) + (int64_t)K * (j0 + i / nb)];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double* b = B + (int64_t)K * j + j0;
    double x[NB];
#pragma unroll
    for (int c = NB - 1; c >= 0; --c) {
        if (c < nb) {
            double a = b[c];
            for (int q = c + 1; q < nb; ++q) a -= s[q][c] * x[q];
            x[c] = a / s[c][c];
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) b[c] = x[c];
}

// B[0:j0) -= L(j0:j0+nb, 0:j0)' * B1   (one thread per (row, rhs))
__global__ void k_trsm_above(const double* __restrict__ L, int K, int j0, double* __restrict__ B, int n)
{
    const int nb = min(NB, K - j0);
    const int64_t total = (int64_t)j0 * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % j0);
        const int64_t j = i / j0;
        double a = 0.0;
        for (int q = 0; q < nb; ++q) a += L[(j0 + q) + (int64_t)K * r] * B[(j0 + q) + (int64_t)K * j];
        B[r + (int64_t)K * j] -= a;
    }
}

__global__ void k_diag_copy(const double* __restrict__ A, int K, double* __restrict__ dg)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
        dg[i] = A[i + (int64_t)K * i];
}

__global__ void k_identity(double* __restrict__ X, int K)
{
    const int64_t n = (int64_t)K * K;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        X[i] = (i % K == i / K) ? 1.0 : 0.0;
}

// T (K x n, ldt) = (Ginv * B)(:, j) / baseline(j); Ginv K x K FP64, B K x n FP32.
// 64 x 64 output tile, 256 threads with 4 x 4 outputs each, K staged by 16.
__global__ void __launch_bounds__(256)
k_dgemm_apply(const double* __restrict__ Gi, const float* __restrict__ B, int K, int n,
              const float* __restrict__ baseline, float* __restrict__ T, int64_t ldt)
{
    __shared__ double As[16][64 + 1];
    __shared__ double Bs[16][64 + 1];
    const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
    const int tm = (threadIdx.x % 16) * 4, tn = (threadIdx.x / 16) * 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int i = threadIdx.x; i < 16 * 64; i += 256) {
            const int mm = i % 64, kk = i / 64;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < K && gk < K) ? Gi[gm + (int64_t)K * gk] : 0.0;
            const int kb = i % 16, nn = i / 16;
            const int gn = n0 + nn, gkb = k0 + kb;
            Bs[kb][nn] = (gn < n && gkb < K) ? (double)B[gkb + (int64_t)K * gn] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][tm + u];
                b[u] = Bs[kk][tn + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const int c = n0 + tn + v;
        if (c >= n) continue;
        const double sc = baseline ? 1.0 / (double)baseline[c] : 1.0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = m0 + tm + u;
            if (r < K) T[r + ldt * c] = (float)(acc[u][v] * sc);
        }
    }
}

}  // namespace
}  // namespace sid

struct sid_pinv {
    sid_ctx* ctx;
    int64_t K, P;
    int prec;
    sid::DBuf fpm;   // P x K pixel-major copy of the forward model
    sid::DBuf ginv;  // K x K FP64 inverse of F*F'
    sid::DBuf tmp;   // K x n FP32 products
    sid::DBuf err;
};

using namespace sid;

static int chol_solve_identity(double* L, double* X, int K, cudaStream_t st)
{
    // X = inv(L L') = inv(L') inv(L) I
    k_identity<<<1024, 256, 0, st>>>(X, K);
    SID_CHECK_LAUNCH();
    const unsigned gj = (unsigned)cdiv(K, 128);
    for (int j0 = 0; j0 < K; j0 += NB) {
        k_trsv_fwd<<<gj, 128, 0, st>>>(L, K, j0, X, K);
        if (K - j0 - NB > 0) k_trsm_below<<<1024, 256, 0, st>>>(L, K, j0, X, K);
        SID_CHECK_LAUNCH();
    }
    for (int j0 = (int)(cdiv(K, NB) - 1) * NB; j0 >= 0; j0 -= NB) {
        k_trsv_bwd<<<gj, 128, 0, st>>>(L, K, j0, X, K);
        if (j0 > 0) k_trsm_above<<<1024, 256, 0, st>>>(L, K, j0, X, K);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

extern "C" int sid_pinv_create(sid_ctx* c, const float* F, int64_t K, int64_t P, int layout, int prec,
                               sid_pinv** out, void* stream)
{
    SID_REQUIRE(c && F && out, "sid_pinv_create: NULL argument");
    *out = nullptr;
    SID_REQUIRE(K >= 1 && P >= 1, "sid_pinv_create: empty forward model");
    SID_REQUIRE(K <= 16384, "sid_pinv_create: K %lld above 16384", (long long)K);
    SID_REQUIRE(layout == 0 || layout == 1, "sid_pinv_create: layout must be 0 (K x P) or 1 (P x K)");
    SID_REQUIRE(prec == SID_PREC_FP32 || prec == SID_PREC_SPLIT, "sid_pinv_create: precision must be FP32 or SPLIT");
    SID_REQUIRE(layout == 1 || cdiv(P, 32) <= 65535, "sid_pinv_create: P too large for the K x P layout");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    sid_pinv* q = new sid_pinv();
    q->ctx = c;
    q->K = K;
    q->P = P;
    q->prec = prec;
    auto fail = [&](int rc) {
        q->fpm.release();
        q->ginv.release();
        q->tmp.release();
        q->err.release();
        delete q;
        return rc;
    };
    int rc = q->fpm.alloc((size_t)(P * K) * 4);
    if (rc == SID_OK) rc = q->ginv.alloc((size_t)(K * K) * 8 * 2);
    if (rc == SID_OK) rc = q->tmp.alloc((size_t)(K * K) * 4);
    if (rc == SID_OK) rc = q->err.alloc(16 + (size_t)K * sizeof(double));  // flag + original diagonal
    if (rc != SID_OK) return fail(rc);
    float* Fp = q->fpm.as<float>();
    if (layout == 0) {
        dim3 grid((unsigned)cdiv(K, 32), (unsigned)cdiv(P, 32)), block(32, 8);
        k_transpose_f32<<<grid, block, 0, st>>>(F, K, P, Fp);
    } else if (cudaMemcpyAsync(Fp, F, (size_t)(P * K) * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
        set_error("sid_pinv_create: copy of the forward model failed");
        return fail(SID_ECUDA);
    }
    // G = F F' (K x K)   incremental_temporal_update_gpu.m:83
    float* G32 = q->tmp.as<float>();
    rc = contract(c, Fp, Fp, false, K, K, P, P, P, G32, K, 1.f, 0.f, prec, st);
    if (rc != SID_OK) return fail(rc);
    double* L = q->ginv.as<double>() + K * K;  // factor, then inv(G) in the first half
    double* Gi = q->ginv.as<double>();
    int* err = q->err.as<int>();
    double* dg = reinterpret_cast<double*>(q->err.as<char>() + 16);
    k_widen<<<1024, 256, 0, st>>>(G32, K * K, L);
    k_diag_copy<<<(unsigned)cdiv(K, 256), 256, 0, st>>>(L, (int)K, dg);
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return fail(SID_ECUDA);
    // blocked right-looking Cholesky, FP64
    const int Ki = (int)K;
    for (int j0 = 0; j0 < Ki; j0 += NB) {
        k_chol_diag<<<1, 256, 0, st>>>(L, Ki, j0, dg, err);
        const int below = Ki - j0 - NB;
        if (below > 0) {
            k_chol_panel<<<(unsigned)cdiv(below, 128), 128, 0, st>>>(L, Ki, j0);
            const unsigned t = (unsigned)cdiv(below, 32);
            k_chol_update<<<dim3(t, t), 256, 0, st>>>(L, Ki, j0);
        }
    }
    if (cudaGetLastError() != cudaSuccess) {
        set_error("sid_pinv_create: Cholesky launch failed");
        return fail(SID_ECUDA);
    }
    rc = chol_solve_identity(L, Gi, Ki, st);
    if (rc != SID_OK) return fail(rc);
    int h_err = 0;
    if (cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("sid_pinv_create: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(SID_ECUDA);
    }
    if (h_err) {
        set_error("sid_pinv_create: F*F' is not positive definite (pivot %d): a footprint is zero or dependent",
                  h_err);
        return fail(SID_EINVAL);
    }
    *out = q;
    return SID_OK;
}

extern "C" int sid_pinv_apply(sid_pinv* q, const void* Y, int ydtype, int64_t n, const float* baseline, float* T,
                              int64_t ldt, void* stream)
{
    SID_REQUIRE(q && Y && T, "sid_pinv_apply: NULL argument");
    SID_REQUIRE(n >= 1, "sid_pinv_apply: no frames");
    SID_REQUIRE(ldt >= q->K, "sid_pinv_apply: ldt %lld < K %lld", (long long)ldt, (long long)q->K);
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "sid_pinv_apply: unknown Y dtype");
    SID_REQUIRE(n <= (int64_t)65535 * 64, "sid_pinv_apply: chunk of %lld frames too large", (long long)n);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t K = q->K, P = q->P;
    SID_TRY(q->tmp.alloc((size_t)(K * n) * 4));
    float* B = q->tmp.as<float>();
    // B = F Y (K x n)   :89,99
    const bool f16 = ydtype == SID_DTYPE_F16;
    SID_TRY(contract(q->ctx, q->fpm.as<float>(), Y, f16, K, n, P, P, P, B, K, 1.f, 0.f,
                     (f16 && q->prec == SID_PREC_FP32) ? SID_PREC_SPLIT : q->prec, st));
    dim3 grid((unsigned)cdiv(K, 64), (unsigned)cdiv(n, 64));
    k_dgemm_apply<<<grid, 256, 0, st>>>(q->ginv.as<double>(), B, (int)K, (int)n, baseline, T, ldt);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

extern "C" int sid_pinv_destroy(sid_pinv* q)
{
    if (!q) return SID_OK;
    q->fpm.release();
    q->ginv.release();
    q->tmp.release();
    q->err.release();
    delete q;
    return SID_OK;
}
