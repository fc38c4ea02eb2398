// spectral.cu -- lenslet-grid spectral projector (the "FFT variant for large
// PSFs" of the reference's forwardProjectGPU.m / conv2FFT_.m).
//
// The reference multiplies full-frame spectra of every PSF slice, recomputed on
// every call (conv2FFT_.m:14, 3 transforms of exsize^2 per slice).  Here the
// multichannel lenslet-grid convolution of direct.cu is diagonalised by an
// L x L DFT on the lenslet grid (L >= Lx + max(dhi,-dlo), so the circular
// convolution never wraps into the kept outputs):
//   Ihat[b'a'](f) = sum_abc Khat[f][b'a'][abc] * Vhat[abc](f)            (forward)
//   Bhat[abc](f)  = sum_b'a' conj(Khat[f][b'a'][abc]) * Ihat[b'a'](f)    (adjoint)
// The tap spectra Khat are computed once per plan and kept resident (FP32, or
// FP16 with one power-of-two scale).  Per projection the cost is one streaming
// pass over Khat (HBM bound) plus small real DFTs of the N*N*Z input and N*N
// output channels.  Real inputs use the half spectrum f1 in [0, L/2].
#include <cmath>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

static inline int64_t spec_nin_pad(const sid_plan* p) { return cdiv(p->N * p->N * p->Z, 8) * 8; }

// ----------------------------------------------------------------- helpers --
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// --------------------------------------------------------- tap spectra -----
// grid (n_out, ceil(n_in/8)); each CTA transforms the tap arrays of 8
// consecutive input channels for one output phase and writes 8 consecutive
// entries of every frequency row.
constexpr int KB_CH = 8;

__global__ void k_build_khat(const float* __restrict__ taps, const float2* __restrict__ tw,
                             float2* __restrict__ k32, __half2* __restrict__ k16, float scale, int N,
                             int n_in, int64_t n_in_pad, int D, int dlo, int L, int64_t tbs)
{
    extern __shared__ float2 sm[];
    const int H1 = L / 2 + 1;
    const int nf = H1 * L;
    float2* G = sm;                                  // [KB_CH][D][H1]
    float2* stw = G + KB_CH * D * H1;                // [L]
    float* tap = reinterpret_cast<float*>(stw + L);  // [KB_CH][D*D]
    const int o = blockIdx.x;  // b'a' = b'*N + a'
    const int bp = o / N, ap = o - (o / N) * N;
    const int k0 = blockIdx.y * KB_CH;
    const int n_out = N * N;
    for (int i = threadIdx.x; i < L; i += blockDim.x) stw[i] = tw[i];
    for (int i = threadIdx.x; i < KB_CH * D * D; i += blockDim.x) {
        const int ch = i / (D * D), m = i - ch * D * D;
        const int abc = k0 + ch;
        tap[i] = (abc < n_in) ? taps[((int64_t)abc * N + bp) * tbs + (int64_t)ap * D * D + m] : 0.f;
    }
    __syncthreads();
    // stage 1 (along m1 / u): G[ch][m2][f1] = sum_m1 tap[ch][m1][m2] w^{-f1 p1}
    for (int i = threadIdx.x; i < KB_CH * D * H1; i += blockDim.x) {
        const int ch = i / (D * H1);
        const int r = i - ch * D * H1;
        const int m2 = r / H1, f1 = r - (r / H1) * H1;
        float2 acc = make_float2(0.f, 0.f);
        for (int m1 = 0; m1 < D; ++m1) {
            const float t = tap[ch * D * D + m1 * D + m2];
            int p1 = (m1 + dlo) % L;
            if (p1 < 0) p1 += L;
            const float2 w = stw[(f1 * p1) % L];
            acc.x += t * w.x;
            acc.y -= t * w.y;
        }
        G[i] = acc;
    }
    __syncthreads();
    // stage 2 (along m2 / v): Khat[f][o][k0+ch] = sum_m2 G[ch][m2][f1] w^{-f2 p2}
    for (int i = threadIdx.x; i < nf * KB_CH; i += blockDim.x) {
        const int f = i / KB_CH, ch = i - (i / KB_CH) * KB_CH;
        const int f2 = f / H1, f1 = f - (f / H1) * H1;
        float2 acc = make_float2(0.f, 0.f);
        for (int m2 = 0; m2 < D; ++m2) {
            int p2 = (m2 + dlo) % L;
            if (p2 < 0) p2 += L;
            float2 w = stw[(f2 * p2) % L];
            w.y = -w.y;
            const float2 g = G[(ch * D + m2) * H1 + f1];
            acc.x += g.x * w.x - g.y * w.y;
            acc.y += g.x * w.y + g.y * w.x;
        }
        const int64_t idx = ((int64_t)f * n_out + o) * n_in_pad + k0 + ch;
        if (k0 + ch < n_in_pad) {
            if (k32) k32[idx] = acc;
            if (k16) k16[idx] = __floats2half2_rn(acc.x * scale, acc.y * scale);
        }
    }
}

// Largest l1 norm of one tap array (an upper bound of |Khat|).  Tap array
// (abc, b', a') starts at (abc*N + b')*tbs + a'*D*D.
__global__ void k_tap_l1(const float* __restrict__ taps, float* __restrict__ out, int64_t narr, int N,
                         int D2, int64_t tbs)
{
    __shared__ float red[256];
    float m = 0.f;
    for (int64_t ai = blockIdx.x; ai < narr; ai += gridDim.x) {
        const float* t = taps + (ai / N) * tbs + (ai % N) * (int64_t)D2;
        float s = 0.f;
        for (int i = threadIdx.x; i < D2; i += blockDim.x) s += fabsf(t[i]);
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) m = fmaxf(m, red[0]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = m;
}

int build_spectra(sid_plan* p)
{
    const int64_t N = p->N, Z = p->Z, D = p->g.D;
    const int64_t Lmin = std::max(p->Lx, p->Ly) + std::max(p->g.dhi, -p->g.dlo);
    const int64_t L = cdiv(Lmin, 4) * 4;
    const int64_t H1 = L / 2 + 1;
    p->L = L;
    p->nf = H1 * L;
    const int64_t n_out = N * N, n_in = N * N * Z, n_in_pad = spec_nin_pad(p);
    // twiddles exp(2 pi i k / L) (sign applied by the kernels)
    std::vector<float2> tw(L);
    for (int64_t k = 0; k < L; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)L;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    SID_TRY(p->twiddle.alloc(L * sizeof(float2)));
    SID_CUDA_TRY(cudaMemcpy(p->twiddle.p, tw.data(), L * sizeof(float2), cudaMemcpyHostToDevice));

    const int64_t tbs = cdiv(N * D * D, 32) * 32;
    float scale = 1.f;
    if (p->flags & SID_PLAN_SPECTRAL_F16) {
        // one power-of-two scale keeps the largest |Khat| near 2^14 in FP16
        const int64_t narr = Z * N * N * N * N;  // one tap array per (abc, b'a')
        DBuf part;
        SID_TRY(part.alloc(1024 * sizeof(float)));
        k_tap_l1<<<1024, 256>>>(p->taps_f.as<float>(), part.as<float>(), narr, (int)N, (int)(D * D), tbs);
        cudaError_t e = cudaGetLastError();
        std::vector<float> h(1024);
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), part.p, 1024 * sizeof(float), cudaMemcpyDeviceToHost);
        part.release();
        SID_CUDA_TRY(e);
        float mx = 0.f;
        for (float v : h) mx = std::max(mx, v);
        if (mx > 0.f) scale = std::ldexp(1.0f, (int)std::floor(std::log2(16384.0 / (double)mx)));
    }
    p->spec_scale = scale;
    const size_t nent = (size_t)(p->nf * n_out * n_in_pad);
    if (p->flags & SID_PLAN_SPECTRAL_F32) {
        SID_TRY(p->khat_f32.alloc(nent * sizeof(float2)));
        SID_CUDA_TRY(cudaMemset(p->khat_f32.p, 0, nent * sizeof(float2)));
        p->spec_f32 = true;
    }
    if (p->flags & SID_PLAN_SPECTRAL_F16) {
        SID_TRY(p->khat_f16.alloc(nent * sizeof(__half2)));
        SID_CUDA_TRY(cudaMemset(p->khat_f16.p, 0, nent * sizeof(__half2)));
        p->spec_f16 = true;
    }
    const size_t smem = (size_t)(KB_CH * D * H1 + L) * sizeof(float2) + (size_t)(KB_CH * D * D) * sizeof(float);
    SID_REQUIRE(smem <= 200 * 1024, "spectral plan: tap arrays too large for the spectra builder (D=%lld, L=%lld)",
                (long long)D, (long long)L);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_build_khat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)n_out, (unsigned)cdiv(n_in, KB_CH));
    k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), p->twiddle.as<float2>(),
                                      p->spec_f32 ? p->khat_f32.as<float2>() : nullptr,
                                      p->spec_f16 ? p->khat_f16.as<__half2>() : nullptr, scale, (int)N,
                                      (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
    SID_CHECK_LAUNCH();
    SID_CUDA_TRY(cudaDeviceSynchronize());
    if (!(p->flags & SID_PLAN_DIRECT)) p->taps_f.release();
    return SID_OK;
}

// -------------------------------------------------------------- real DFTs --
// Analysis: polyphase planes [ch][Ly][Lx] (zero-extended to L x L) -> half
// spectra [ch][nf], f = f1 + H1*f2, X(f1,f2) = sum_{u,v} x(u,v) w^{-(f1 u + f2 v)}.
__global__ void k_dft_r2c(const float* __restrict__ in, float2* __restrict__ out,
                          const float2* __restrict__ tw, int Lx, int Ly, int L)
{
    extern __shared__ float2 sm2[];
    const int H1 = L / 2 + 1, nf = H1 * L;
    float2* G = sm2;               // [Ly][H1]
    float2* stw = G + Ly * H1;     // [L]
    float* img = reinterpret_cast<float*>(stw + L);  // [Ly][Lx]
    const int64_t ch = blockIdx.x;
    const float* src = in + ch * (int64_t)Ly * Lx;
    for (int i = threadIdx.x; i < L; i += blockDim.x) stw[i] = tw[i];
    for (int i = threadIdx.x; i < Ly * Lx; i += blockDim.x) img[i] = src[i];
    __syncthreads();
    for (int i = threadIdx.x; i < Ly * H1; i += blockDim.x) {
        const int v = i / H1, f1 = i - (i / H1) * H1;
        const float* row = img + v * Lx;
        float ax = 0.f, ay = 0.f;
        int k = 0;
        for (int u = 0; u < Lx; ++u) {
            const float2 w = stw[k];
            ax = fmaf(row[u], w.x, ax);
            ay = fmaf(-row[u], w.y, ay);
            k += f1;
            if (k >= L) k -= L;
        }
        G[i] = make_float2(ax, ay);
    }
    __syncthreads();
    float2* dst = out + ch * (int64_t)nf;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
        const int f2 = i / H1, f1 = i - (i / H1) * H1;
        float ax = 0.f, ay = 0.f;
        int k = 0;
        for (int v = 0; v < Ly; ++v) {
            const float2 g = G[v * H1 + f1];
            const float2 w = stw[k];  // multiply by conj(w)
            ax += g.x * w.x + g.y * w.y;
            ay += g.y * w.x - g.x * w.y;
            k += f2;
            if (k >= L) k -= L;
        }
        dst[i] = make_float2(ax, ay);
    }
}

// Synthesis: half spectra [ch][nf] -> planes [ch][Ly][Lx], x = (1/L^2) sum X w^{+...}.
// Lattice positions outside the X x Y frame are written as zero.
__global__ void k_dft_c2r(const float2* __restrict__ in, float* __restrict__ out,
                          const float2* __restrict__ tw, int Lx, int Ly, int L, int N, int64_t X,
                          int64_t Y)
{
    extern __shared__ float2 sm2[];
    const int H1 = L / 2 + 1, nf = H1 * L;
    float2* S = sm2;              // [nf]
    float2* G = S + nf;           // [Ly][H1]
    float2* stw = G + Ly * H1;    // [L]
    const int64_t ch = blockIdx.x;
    const int a = (int)(ch % N), b = (int)((ch / N) % N);
    const float2* src = in + ch * (int64_t)nf;
    for (int i = threadIdx.x; i < L; i += blockDim.x) stw[i] = tw[i];
    for (int i = threadIdx.x; i < nf; i += blockDim.x) S[i] = src[i];
    __syncthreads();
    for (int i = threadIdx.x; i < Ly * H1; i += blockDim.x) {
        const int t = i / H1, f1 = i - (i / H1) * H1;
        float ax = 0.f, ay = 0.f;
        int k = 0;
        for (int f2 = 0; f2 < L; ++f2) {
            const float2 s = S[f2 * H1 + f1];
            const float2 w = stw[k];
            ax += s.x * w.x - s.y * w.y;
            ay += s.x * w.y + s.y * w.x;
            k += t;
            if (k >= L) k -= L;
        }
        G[i] = make_float2(ax, ay);
    }
    __syncthreads();
    const float inv = 1.0f / ((float)L * (float)L);
    const bool even = (L % 2) == 0;
    float* dst = out + ch * (int64_t)Ly * Lx;
    for (int i = threadIdx.x; i < Ly * Lx; i += blockDim.x) {
        const int t = i / Lx, s = i - (i / Lx) * Lx;
        const float2* g = G + t * H1;
        float acc = g[0].x;
        int k = s;
        if (k >= L) k -= L;
        const int last = even ? H1 - 1 : H1;
        for (int f1 = 1; f1 < last; ++f1) {
            const float2 w = stw[k];
            acc += 2.f * (g[f1].x * w.x - g[f1].y * w.y);
            k += s;
            if (k >= L) k -= L;
        }
        if (even) acc += (s & 1) ? -g[H1 - 1].x : g[H1 - 1].x;
        const bool inside = (a + (int64_t)N * s) < X && (b + (int64_t)N * t) < Y;
        dst[i] = inside ? acc * inv : 0.f;
    }
}

// ------------------------------------------------------------ GEMV kernels --
// Forward: per frequency f, Ihat[o][f] = (1/scale) sum_k Khat[f][o][k] Vhat[k][f].
template <bool F16>
__global__ void __launch_bounds__(512)
k_spec_fwd(const void* __restrict__ khat, const float2* __restrict__ vhat, float2* __restrict__ ihat,
           int n_in, int64_t n_in_pad, int n_out, int nf, float inv_scale)
{
    extern __shared__ float2 xv[];  // [n_in_pad]
    const int f = blockIdx.x;
    for (int k = threadIdx.x; k < n_in_pad; k += blockDim.x)
        xv[k] = (k < n_in) ? vhat[(int64_t)k * nf + f] : make_float2(0.f, 0.f);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = warp; o < n_out; o += nw) {
        float ar = 0.f, ai = 0.f;
        const int64_t row = ((int64_t)f * n_out + o) * n_in_pad;
        if (F16) {
            // 4 complex (16 bytes) per lane per step
            const uint4* kr = reinterpret_cast<const uint4*>(reinterpret_cast<const __half2*>(khat) + row);
            const int nvec = (int)(n_in_pad / 4);
#pragma unroll 4
            for (int j = lane; j < nvec; j += 32) {
                const uint4 q = __ldcs(kr + j);
                const __half2* h = reinterpret_cast<const __half2*>(&q);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float2 kk = __half22float2(h[e]);
                    const float2 x = xv[4 * j + e];
                    ar = fmaf(kk.x, x.x, ar);
                    ar = fmaf(-kk.y, x.y, ar);
                    ai = fmaf(kk.x, x.y, ai);
                    ai = fmaf(kk.y, x.x, ai);
                }
            }
        } else {
            const float4* kr = reinterpret_cast<const float4*>(reinterpret_cast<const float2*>(khat) + row);
            const int nvec = (int)(n_in_pad / 2);
#pragma unroll 4
            for (int j = lane; j < nvec; j += 32) {
                const float4 q = __ldcs(kr + j);
                const float2 x0 = xv[2 * j], x1 = xv[2 * j + 1];
                ar = fmaf(q.x, x0.x, ar); ar = fmaf(-q.y, x0.y, ar);
                ai = fmaf(q.x, x0.y, ai); ai = fmaf(q.y, x0.x, ai);
                ar = fmaf(q.z, x1.x, ar); ar = fmaf(-q.w, x1.y, ar);
                ai = fmaf(q.z, x1.y, ai); ai = fmaf(q.w, x1.x, ai);
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, off);
            ai += __shfl_xor_sync(0xffffffffu, ai, off);
        }
        if (lane == 0) ihat[(int64_t)o * nf + f] = make_float2(ar * inv_scale, ai * inv_scale);
    }
}

// Adjoint: per frequency f, Bhat[k][f] = (1/scale) sum_o conj(Khat[f][o][k]) Ihat[o][f].
template <bool F16>
__global__ void __launch_bounds__(512)
k_spec_adj(const void* __restrict__ khat, const float2* __restrict__ ihat, float2* __restrict__ bhat,
           int n_in, int64_t n_in_pad, int n_out, int nf, float inv_scale)
{
    extern __shared__ float2 yv[];  // [n_out]
    const int f = blockIdx.x;
    for (int o = threadIdx.x; o < n_out; o += blockDim.x) yv[o] = ihat[(int64_t)o * nf + f];
    __syncthreads();
    constexpr int V = F16 ? 4 : 2;  // complex entries per 16-byte load
    const int nvec = (int)(n_in_pad / V);
    const int64_t base = (int64_t)f * n_out * n_in_pad;
    for (int j = threadIdx.x; j < nvec; j += blockDim.x) {
        float ar[V], ai[V];
#pragma unroll
        for (int e = 0; e < V; ++e) ar[e] = ai[e] = 0.f;
#pragma unroll 4
        for (int o = 0; o < n_out; ++o) {
            const float2 y = yv[o];
            if (F16) {
                const uint4 q = __ldcs(reinterpret_cast<const uint4*>(
                                           reinterpret_cast<const __half2*>(khat) + base + (int64_t)o * n_in_pad) + j);
                const __half2* h = reinterpret_cast<const __half2*>(&q);
#pragma unroll
                for (int e = 0; e < V; ++e) {
                    const float2 kk = __half22float2(h[e]);
                    ar[e] = fmaf(kk.x, y.x, ar[e]); ar[e] = fmaf(kk.y, y.y, ar[e]);
                    ai[e] = fmaf(kk.x, y.y, ai[e]); ai[e] = fmaf(-kk.y, y.x, ai[e]);
                }
            } else {
                const float4 q = __ldcs(reinterpret_cast<const float4*>(
                                            reinterpret_cast<const float2*>(khat) + base + (int64_t)o * n_in_pad) + j);
                const float kx[2] = {q.x, q.z}, ky[2] = {q.y, q.w};
#pragma unroll
                for (int e = 0; e < V; ++e) {
                    ar[e] = fmaf(kx[e], y.x, ar[e]); ar[e] = fmaf(ky[e], y.y, ar[e]);
                    ai[e] = fmaf(kx[e], y.y, ai[e]); ai[e] = fmaf(-ky[e], y.x, ai[e]);
                }
            }
        }
#pragma unroll
        for (int e = 0; e < V; ++e) {
            const int k = V * j + e;
            if (k < n_in) bhat[(int64_t)k * nf + f] = make_float2(ar[e] * inv_scale, ai[e] * inv_scale);
        }
    }
}

// ------------------------------------------------------------- launchers --
static int ensure_spec_ws(sid_plan* p)
{
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N;
    SID_TRY(p->vhat.alloc((size_t)(n_in * p->nf) * sizeof(float2)));
    SID_TRY(p->ihat.alloc((size_t)(n_out * p->nf) * sizeof(float2)));
    return SID_OK;
}

static size_t r2c_smem(const sid_plan* p)
{
    const int64_t H1 = p->L / 2 + 1;
    return (size_t)(p->Ly * H1 + p->L) * sizeof(float2) + (size_t)(p->Ly * p->Lx) * sizeof(float);
}
static size_t c2r_smem(const sid_plan* p)
{
    const int64_t H1 = p->L / 2 + 1;
    return (size_t)(p->nf + p->Ly * H1 + p->L) * sizeof(float2);
}

static int configure_dft(const sid_plan* p)
{
    SID_REQUIRE(r2c_smem(p) <= 220 * 1024 && c2r_smem(p) <= 220 * 1024,
                "spectral projector: lenslet grid %lldx%lld (L=%lld) exceeds the DFT kernels' shared memory",
                (long long)p->Lx, (long long)p->Ly, (long long)p->L);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_dft_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r2c_smem(p)));
    SID_CUDA_TRY(cudaFuncSetAttribute(k_dft_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c2r_smem(p)));
    return SID_OK;
}

static int spec_check(const sid_plan* p, bool f16)
{
    if (f16 && !p->spec_f16) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_F16");
        return SID_ENOTSUP;
    }
    if (!f16 && !p->spec_f32) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_F32");
        return SID_ENOTSUP;
    }
    return SID_OK;
}

int spectral_forward(sid_plan* p, bool f16, const float* vp, float* ip, cudaStream_t st)
{
    SID_TRY(spec_check(p, f16));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    k_dft_r2c<<<(unsigned)n_in, 256, r2c_smem(p), st>>>(vp, p->vhat.as<float2>(), p->twiddle.as<float2>(),
                                                         (int)p->Lx, (int)p->Ly, (int)p->L);
    SID_CHECK_LAUNCH();
    const size_t sm = (size_t)n_in_pad * sizeof(float2);
    const float inv = 1.0f / (f16 ? p->spec_scale : 1.0f);
    p->timer.begin(st);
    if (f16) {
        SID_CUDA_TRY(cudaFuncSetAttribute(k_spec_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_spec_fwd<true><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f16.p, p->vhat.as<float2>(), p->ihat.as<float2>(),
                                                          (int)n_in, n_in_pad, (int)n_out, (int)p->nf, inv);
    } else {
        SID_CUDA_TRY(cudaFuncSetAttribute(k_spec_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_spec_fwd<false><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.p, p->vhat.as<float2>(), p->ihat.as<float2>(),
                                                           (int)n_in, n_in_pad, (int)n_out, (int)p->nf, inv);
    }
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    k_dft_c2r<<<(unsigned)n_out, 256, c2r_smem(p), st>>>(p->ihat.as<float2>(), ip, p->twiddle.as<float2>(),
                                                          (int)p->Lx, (int)p->Ly, (int)p->L, (int)p->N, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_adjoint(sid_plan* p, bool f16, const float* ip, float* bp, cudaStream_t st)
{
    SID_TRY(spec_check(p, f16));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    k_dft_r2c<<<(unsigned)n_out, 256, r2c_smem(p), st>>>(ip, p->ihat.as<float2>(), p->twiddle.as<float2>(),
                                                          (int)p->Lx, (int)p->Ly, (int)p->L);
    SID_CHECK_LAUNCH();
    const size_t sm = (size_t)n_out * sizeof(float2);
    const float inv = 1.0f / (f16 ? p->spec_scale : 1.0f);
    p->timer.begin(st);
    if (f16)
        k_spec_adj<true><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f16.p, p->ihat.as<float2>(), p->vhat.as<float2>(),
                                                          (int)n_in, n_in_pad, (int)n_out, (int)p->nf, inv);
    else
        k_spec_adj<false><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.p, p->ihat.as<float2>(), p->vhat.as<float2>(),
                                                           (int)n_in, n_in_pad, (int)n_out, (int)p->nf, inv);
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    k_dft_c2r<<<(unsigned)n_in, 256, c2r_smem(p), st>>>(p->vhat.as<float2>(), bp, p->twiddle.as<float2>(),
                                                         (int)p->Lx, (int)p->Ly, (int)p->L, (int)p->N, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace sid
