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
// The tap spectra Khat are computed once per plan and kept resident, in FP32
// or in 16-bit block floating point (int16 mantissas, one FP32 step per
// frequency row: 15-bit precision relative to the row's largest entry).  Per projection the cost is one streaming
// pass over Khat (HBM bound) plus small real DFTs of the N*N*Z input and N*N
// output channels.  Real inputs use the half spectrum f1 in [0, L/2].
#include <cmath>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

static inline int64_t spec_nin_pad(const sid_plan* p) { return cdiv(p->N * p->N * p->Z, 8) * 8; }

// --------------------------------------------------------- tap spectra -----
// grid (n_out, ceil(n_in/8)); each CTA transforms the tap arrays of 8
// consecutive input channels for one output phase and writes 8 consecutive
// entries of every frequency row.
//   mode 0: write FP32 spectra (if k32) and the per-row max |Re|,|Im| (rowmax,
//           float bits, atomicMax; values are >= 0 so integer order = float order)
//   mode 1: write 16-bit block-floating-point spectra: int16 mantissas with the
//           row's step rstep[f*n_out + o] = rowmax/32767 (value = mantissa * step)
constexpr int KB_CH = 8;

__global__ void k_build_khat(const float* __restrict__ taps, const float2* __restrict__ tw,
                             float2* __restrict__ k32, short2* __restrict__ k16,
                             unsigned int* __restrict__ rowmax, const float* __restrict__ rstep, int mode,
                             int N, int n_in, int64_t n_in_pad, int D, int dlo, int L, int64_t tbs)
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
    // (blockDim is a multiple of KB_CH, so the KB_CH lanes of one f are adjacent)
    const int nitems = nf * KB_CH;
    for (int i0 = 0; i0 < nitems; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        const bool live = i < nitems;
        const int f = live ? i / KB_CH : 0, ch = i - (i / KB_CH) * KB_CH;
        const int f2 = f / H1, f1 = f - (f / H1) * H1;
        float2 acc = make_float2(0.f, 0.f);
        if (live) {
            for (int m2 = 0; m2 < D; ++m2) {
                int p2 = (m2 + dlo) % L;
                if (p2 < 0) p2 += L;
                float2 w = stw[(f2 * p2) % L];
                w.y = -w.y;
                const float2 g = G[(ch * D + m2) * H1 + f1];
                acc.x += g.x * w.x - g.y * w.y;
                acc.y += g.x * w.y + g.y * w.x;
            }
        }
        const int64_t idx = ((int64_t)f * n_out + o) * n_in_pad + k0 + ch;
        if (mode == 0) {
            if (live && k32) k32[idx] = acc;
            float m = fmaxf(fabsf(acc.x), fabsf(acc.y));
#pragma unroll
            for (int off = KB_CH / 2; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
            if (live && ch == 0 && m > 0.f) atomicMax(rowmax + (int64_t)f * n_out + o, __float_as_uint(m));
        } else if (live) {
            const float st = rstep[(int64_t)f * n_out + o];
            const float re = fminf(fmaxf(rintf(acc.x / st), -32767.f), 32767.f);
            const float im = fminf(fmaxf(rintf(acc.y / st), -32767.f), 32767.f);
            k16[idx] = make_short2((short)re, (short)im);
        }
    }
}

// step = rowmax / 32767 (the row's largest component maps to +-32767), 1 for empty rows
__global__ void k_row_steps(const unsigned int* __restrict__ rowmax, float* __restrict__ rstep, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float m = __uint_as_float(rowmax[i]);
        rstep[i] = (m > 0.f) ? m / 32767.f : 1.f;
    }
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
    const size_t nent = (size_t)(p->nf * n_out * n_in_pad);
    const int64_t nrows = p->nf * n_out;
    if (p->flags & SID_PLAN_SPECTRAL_F32) {
        SID_TRY(p->khat_f32.alloc(nent * sizeof(float2)));
        SID_CUDA_TRY(cudaMemset(p->khat_f32.p, 0, nent * sizeof(float2)));
        p->spec_f32 = true;
    }
    const bool want16 = (p->flags & SID_PLAN_SPECTRAL_I16) != 0;
    if (want16) {
        SID_TRY(p->khat_i16.alloc(nent * sizeof(short2)));
        SID_CUDA_TRY(cudaMemset(p->khat_i16.p, 0, nent * sizeof(short2)));
        SID_TRY(p->rstep.alloc((size_t)nrows * sizeof(float)));
        SID_CUDA_TRY(cudaMemset(p->rstep.p, 0, (size_t)nrows * sizeof(float)));  // row max bits first
        p->spec_i16 = true;
    }
    const size_t smem = (size_t)(KB_CH * D * H1 + L) * sizeof(float2) + (size_t)(KB_CH * D * D) * sizeof(float);
    SID_REQUIRE(smem <= 200 * 1024, "spectral plan: tap arrays too large for the spectra builder (D=%lld, L=%lld)",
                (long long)D, (long long)L);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_build_khat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)n_out, (unsigned)cdiv(n_in, KB_CH));
    unsigned int* rowmax = want16 ? p->rstep.as<unsigned int>() : nullptr;
    // pass 1: FP32 spectra and row maxima
    if (p->spec_f32 || want16) {
        DBuf dummy;
        if (!rowmax) { SID_TRY(dummy.alloc((size_t)nrows * sizeof(unsigned))); rowmax = dummy.as<unsigned int>(); }
        k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), p->twiddle.as<float2>(),
                                          p->spec_f32 ? p->khat_f32.as<float2>() : nullptr, nullptr, rowmax,
                                          nullptr, 0, (int)N, (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaDeviceSynchronize());
        dummy.release();
    }
    // pass 2: 16-bit mantissas with per-row power-of-two steps
    if (want16) {
        k_row_steps<<<1024, 256>>>(p->rstep.as<unsigned int>(), p->rstep.as<float>(), nrows);
        SID_CHECK_LAUNCH();
        k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), p->twiddle.as<float2>(), nullptr,
                                          p->khat_i16.as<short2>(), nullptr, p->rstep.as<float>(), 1, (int)N,
                                          (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaDeviceSynchronize());
    }
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
// Storage formats of the tap spectra: FP32 complex (float2, 2 per 16-byte
// load) or 16-bit block floating point (short2 mantissas, 4 per load, with a
// power-of-two step per frequency row).
template <bool I16> struct KLoad;
template <> struct KLoad<false> {
    static constexpr int EPL = 2;
    __device__ static void unpack(const uint4& q, float2 (&k)[2])
    {
        k[0] = make_float2(__uint_as_float(q.x), __uint_as_float(q.y));
        k[1] = make_float2(__uint_as_float(q.z), __uint_as_float(q.w));
    }
};
template <> struct KLoad<true> {
    static constexpr int EPL = 4;
    __device__ static void unpack(const uint4& q, float2 (&k)[4])
    {
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int e = 0; e < 4; ++e)
            k[e] = make_float2((float)(short)(w[e] & 0xffffu), (float)(short)(w[e] >> 16));
    }
};

// Forward: per frequency f, Ihat[o][f] = step(f,o) * sum_k Khat[f][o][k] Vhat[k][f].
// One CTA per frequency; each warp streams RB rows at once (RB independent
// 16-byte loads in flight per lane) and reduces them with warp shuffles.
constexpr int kRB = 4;

template <bool I16>
__global__ void __launch_bounds__(512)
k_spec_fwd(const uint4* __restrict__ khat, const float* __restrict__ rstep, const float2* __restrict__ vhat,
           float2* __restrict__ ihat, int n_in, int64_t n_in_pad, int n_out, int nf)
{
    using KL = KLoad<I16>;
    constexpr int EPL = KL::EPL;
    extern __shared__ float2 xv[];  // [n_in_pad]
    const int f = blockIdx.x;
    for (int k = threadIdx.x; k < n_in_pad; k += blockDim.x)
        xv[k] = (k < n_in) ? vhat[(int64_t)k * nf + f] : make_float2(0.f, 0.f);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nvec = (int)(n_in_pad / EPL);
    const int64_t rowvec = n_in_pad / EPL;  // uint4 per row
    for (int o0 = warp * kRB; o0 < n_out; o0 += nw * kRB) {
        float ar[kRB], ai[kRB];
        const uint4* kr[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            ar[r] = ai[r] = 0.f;
            const int o = min(o0 + r, n_out - 1);
            kr[r] = khat + ((int64_t)f * n_out + o) * rowvec;
        }
#pragma unroll 2
        for (int j = lane; j < nvec; j += 32) {
            uint4 q[kRB];
#pragma unroll
            for (int r = 0; r < kRB; ++r) q[r] = __ldcs(kr[r] + j);
            float2 x[EPL];
#pragma unroll
            for (int e = 0; e < EPL; ++e) x[e] = xv[EPL * j + e];
#pragma unroll
            for (int r = 0; r < kRB; ++r) {
                float2 kk[EPL];
                KL::unpack(q[r], kk);
#pragma unroll
                for (int e = 0; e < EPL; ++e) {
                    ar[r] = fmaf(kk[e].x, x[e].x, ar[r]);
                    ar[r] = fmaf(-kk[e].y, x[e].y, ar[r]);
                    ai[r] = fmaf(kk[e].x, x[e].y, ai[r]);
                    ai[r] = fmaf(kk[e].y, x[e].x, ai[r]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                ar[r] += __shfl_xor_sync(0xffffffffu, ar[r], off);
                ai[r] += __shfl_xor_sync(0xffffffffu, ai[r], off);
            }
        }
        if (lane < kRB && o0 + lane < n_out) {
            float re = ar[0], im = ai[0];
#pragma unroll
            for (int r = 1; r < kRB; ++r)
                if (lane == r) { re = ar[r]; im = ai[r]; }
            const int o = o0 + lane;
            const float st = I16 ? rstep[(int64_t)f * n_out + o] : 1.f;
            ihat[(int64_t)o * nf + f] = make_float2(re * st, im * st);
        }
    }
}

// Adjoint: per frequency f, Bhat[k][f] = sum_o conj(Khat[f][o][k]) * step(f,o) * Ihat[o][f].
template <bool I16>
__global__ void __launch_bounds__(512)
k_spec_adj(const uint4* __restrict__ khat, const float* __restrict__ rstep, const float2* __restrict__ ihat,
           float2* __restrict__ bhat, int n_in, int64_t n_in_pad, int n_out, int nf)
{
    using KL = KLoad<I16>;
    constexpr int V = KL::EPL;
    extern __shared__ float2 yv[];  // [n_out], pre-multiplied by the row steps
    const int f = blockIdx.x;
    for (int o = threadIdx.x; o < n_out; o += blockDim.x) {
        const float2 y = ihat[(int64_t)o * nf + f];
        const float st = I16 ? rstep[(int64_t)f * n_out + o] : 1.f;
        yv[o] = make_float2(y.x * st, y.y * st);
    }
    __syncthreads();
    const int nvec = (int)(n_in_pad / V);
    const int64_t rowvec = n_in_pad / V;
    const uint4* base = khat + (int64_t)f * n_out * rowvec;
    for (int j = threadIdx.x; j < nvec; j += blockDim.x) {
        float ar[V], ai[V];
#pragma unroll
        for (int e = 0; e < V; ++e) ar[e] = ai[e] = 0.f;
        const uint4* col = base + j;
#pragma unroll 4
        for (int o = 0; o < n_out; ++o) {
            const float2 y = yv[o];
            float2 kk[V];
            KL::unpack(__ldcs(col + (int64_t)o * rowvec), kk);
#pragma unroll
            for (int e = 0; e < V; ++e) {
                ar[e] = fmaf(kk[e].x, y.x, ar[e]); ar[e] = fmaf(kk[e].y, y.y, ar[e]);
                ai[e] = fmaf(kk[e].x, y.y, ai[e]); ai[e] = fmaf(-kk[e].y, y.x, ai[e]);
            }
        }
#pragma unroll
        for (int e = 0; e < V; ++e) {
            const int k = V * j + e;
            if (k < n_in) bhat[(int64_t)k * nf + f] = make_float2(ar[e], ai[e]);
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

static int spec_check(const sid_plan* p, bool i16)
{
    if (i16 && !p->spec_i16) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_I16");
        return SID_ENOTSUP;
    }
    if (!i16 && !p->spec_f32) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_F32");
        return SID_ENOTSUP;
    }
    return SID_OK;
}

int spectral_forward(sid_plan* p, bool i16, const float* vp, float* ip, cudaStream_t st)
{
    SID_TRY(spec_check(p, i16));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    k_dft_r2c<<<(unsigned)n_in, 256, r2c_smem(p), st>>>(vp, p->vhat.as<float2>(), p->twiddle.as<float2>(),
                                                         (int)p->Lx, (int)p->Ly, (int)p->L);
    SID_CHECK_LAUNCH();
    const size_t sm = (size_t)n_in_pad * sizeof(float2);
    p->timer.begin(st);
    if (i16) {
        SID_CUDA_TRY(cudaFuncSetAttribute(k_spec_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_spec_fwd<true><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_i16.as<uint4>(), p->rstep.as<float>(),
                                                          p->vhat.as<float2>(), p->ihat.as<float2>(), (int)n_in,
                                                          n_in_pad, (int)n_out, (int)p->nf);
    } else {
        SID_CUDA_TRY(cudaFuncSetAttribute(k_spec_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_spec_fwd<false><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.as<uint4>(), nullptr, p->vhat.as<float2>(),
                                                           p->ihat.as<float2>(), (int)n_in, n_in_pad, (int)n_out,
                                                           (int)p->nf);
    }
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    k_dft_c2r<<<(unsigned)n_out, 256, c2r_smem(p), st>>>(p->ihat.as<float2>(), ip, p->twiddle.as<float2>(),
                                                          (int)p->Lx, (int)p->Ly, (int)p->L, (int)p->N, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_adjoint(sid_plan* p, bool i16, const float* ip, float* bp, cudaStream_t st)
{
    SID_TRY(spec_check(p, i16));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    k_dft_r2c<<<(unsigned)n_out, 256, r2c_smem(p), st>>>(ip, p->ihat.as<float2>(), p->twiddle.as<float2>(),
                                                          (int)p->Lx, (int)p->Ly, (int)p->L);
    SID_CHECK_LAUNCH();
    const size_t sm = (size_t)n_out * sizeof(float2);
    p->timer.begin(st);
    if (i16)
        k_spec_adj<true><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_i16.as<uint4>(), p->rstep.as<float>(),
                                                          p->ihat.as<float2>(), p->vhat.as<float2>(), (int)n_in,
                                                          n_in_pad, (int)n_out, (int)p->nf);
    else
        k_spec_adj<false><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.as<uint4>(), nullptr, p->ihat.as<float2>(),
                                                           p->vhat.as<float2>(), (int)n_in, n_in_pad, (int)n_out,
                                                           (int)p->nf);
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    k_dft_c2r<<<(unsigned)n_in, 256, c2r_smem(p), st>>>(p->vhat.as<float2>(), bp, p->twiddle.as<float2>(),
                                                         (int)p->Lx, (int)p->Ly, (int)p->L, (int)p->N, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace sid
