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

bool fft_factor(int64_t L, int* P, int* Q);

static inline int64_t spec_nin_pad(const sid_plan* p) { return cdiv(p->N * p->N * p->Z, 8) * 8; }

// --------------------------------------------------------- tap spectra -----
// grid (n_out, ceil(n_in/8)); each CTA transforms the tap arrays of 8
// consecutive input channels for one output phase and writes 8 consecutive
// entries of every frequency row.
//   mode 0: write FP32 spectra (if k32) and the per-row max |Re|,|Im| (rowmax,
//           float bits, atomicMax; values are >= 0 so integer order = float order)
//           and, when k24h is set, the 24-bit float planes (f24_split)
//   mode 1: write 16-bit block-floating-point spectra: int16 mantissas with the
//           row's step rstep[f*n_out + o] = rowmax/32767 (value = mantissa * step)
constexpr int KB_CH = 8;

// 24-bit floats: the top 24 bits of an FP32 value (sign, 8-bit exponent, 15
// mantissa bits; round to nearest, ties to even) stored as a 16-bit high part
// and an 8-bit low part.  The rounding increment is added to the magnitude bits
// (sign and magnitude are separate in FP32), so a carry moves into the exponent
// as it should; spectra are far from the largest finite float.
__device__ __forceinline__ void f24_split(float v, unsigned short& hi, unsigned char& lo)
{
    unsigned u = __float_as_uint(v);
    u += 0x7Fu + ((u >> 8) & 1u);
    hi = (unsigned short)(u >> 16);
    lo = (unsigned char)((u >> 8) & 0xFFu);
}

__global__ void k_build_khat(const float* __restrict__ taps, const float2* __restrict__ tw,
                             float2* __restrict__ k32, short2* __restrict__ k16, ushort2* __restrict__ k24h,
                             uchar2* __restrict__ k24l, unsigned int* __restrict__ rowmax,
                             const float* __restrict__ rstep, int mode, int N, int n_in, int64_t n_in_pad, int D,
                             int dlo, int L, int64_t tbs)
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
            if (live && k24h) {
                unsigned short hr, hi_;
                unsigned char lr, li;
                f24_split(acc.x, hr, lr);
                f24_split(acc.y, hi_, li);
                k24h[idx] = make_ushort2(hr, hi_);
                k24l[idx] = make_uchar2(lr, li);
            }
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
    // the smallest multiple of 4 >= Lmin whose odd part is at most 15 (the FFT
    // kernels' factorisation), or the smallest multiple of 4 if none is near
    int64_t L = cdiv(Lmin, 4) * 4;
    for (int64_t c = L; c < L + 64; c += 4) {
        int fp = 0, fq = 0;
        if (fft_factor(c, &fp, &fq)) {
            L = c;
            break;
        }
    }
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
    if (p->flags & SID_PLAN_SPECTRAL_F24) {
        SID_TRY(p->khat_f24h.alloc(nent * sizeof(ushort2)));
        SID_TRY(p->khat_f24l.alloc(nent * sizeof(uchar2)));
        SID_CUDA_TRY(cudaMemset(p->khat_f24h.p, 0, nent * sizeof(ushort2)));
        SID_CUDA_TRY(cudaMemset(p->khat_f24l.p, 0, nent * sizeof(uchar2)));
        p->spec_f24 = true;
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
    // pass 1: FP32 and 24-bit spectra, row maxima
    if (p->spec_f32 || want16 || p->spec_f24) {
        DBuf dummy;
        if (!rowmax) { SID_TRY(dummy.alloc((size_t)nrows * sizeof(unsigned))); rowmax = dummy.as<unsigned int>(); }
        k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), p->twiddle.as<float2>(),
                                          p->spec_f32 ? p->khat_f32.as<float2>() : nullptr, nullptr,
                                          p->spec_f24 ? p->khat_f24h.as<ushort2>() : nullptr,
                                          p->spec_f24 ? p->khat_f24l.as<uchar2>() : nullptr, rowmax, nullptr, 0,
                                          (int)N, (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaDeviceSynchronize());
        dummy.release();
    }
    // pass 2: 16-bit mantissas with per-row power-of-two steps
    if (want16) {
        k_row_steps<<<1024, 256>>>(p->rstep.as<unsigned int>(), p->rstep.as<float>(), nrows);
        SID_CHECK_LAUNCH();
        k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), p->twiddle.as<float2>(), nullptr,
                                          p->khat_i16.as<short2>(), nullptr, nullptr, nullptr, p->rstep.as<float>(),
                                          1, (int)N, (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaDeviceSynchronize());
    }
    // the weakly observed voxels keep exact back projections from the taps
    // (kept for that even without the direct form)
    return weak_build(p);
}

// 24-bit tap spectra [f][b'a'][abc] of the plan's forward taps on an L x L
// lenslet grid other than the plan's own (the library's neuron windows):
// twiddles tw[k] = exp(2 pi i k / L), planes h / l of nf = (L/2+1) L rows.
int build_khat_f24(const sid_plan* p, int64_t L, const float2* tw, ushort2* h, uchar2* l)
{
    const int64_t N = p->N, Z = p->Z, D = p->g.D;
    const int64_t H1 = L / 2 + 1, nf = H1 * L;
    const int64_t n_out = N * N, n_in = N * N * Z, n_in_pad = spec_nin_pad(p);
    const int64_t tbs = cdiv(N * D * D, 32) * 32;
    const size_t nent = (size_t)(nf * n_out * n_in_pad);
    SID_CUDA_TRY(cudaMemset(h, 0, nent * sizeof(ushort2)));
    SID_CUDA_TRY(cudaMemset(l, 0, nent * sizeof(uchar2)));
    const size_t smem = (size_t)(KB_CH * D * H1 + L) * sizeof(float2) + (size_t)(KB_CH * D * D) * sizeof(float);
    SID_REQUIRE(smem <= 200 * 1024, "spectral plan: tap arrays too large for the spectra builder (D=%lld, L=%lld)",
                (long long)D, (long long)L);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_build_khat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DBuf rowmax;  // written by the builder, not needed here
    SID_TRY(rowmax.alloc((size_t)(nf * n_out) * sizeof(unsigned)));
    dim3 grid((unsigned)n_out, (unsigned)cdiv(n_in, KB_CH));
    k_build_khat<<<grid, 256, smem>>>(p->taps_f.as<float>(), tw, nullptr, nullptr, h, l, rowmax.as<unsigned int>(),
                                      nullptr, 0, (int)N, (int)n_in, n_in_pad, (int)D, (int)p->g.dlo, (int)L, tbs);
    SID_CHECK_LAUNCH();
    SID_CUDA_TRY(cudaDeviceSynchronize());
    rowmax.release();
    return SID_OK;
}

// -------------------------------------------------------------- real DFTs --
// Both transforms are small complex matrix products per channel, computed as
// register-blocked GEMMs against twiddle tables held in shared memory (built
// once per CTA; the CTAs are persistent over channels):
//   analysis   G(v, f1)  = sum_u  x(v, u) conj(w^(u f1))         (real x complex, K = Lx)
//              X(f2, f1) = sum_v  conj(w^(v f2)) G(v, f1)         (complex, K = Ly)
//   synthesis  Gt(f1, t) = sum_f2 w^(t f2) S(f2, f1)              (complex, K = L)
//              x(t, s)   = 1/L^2 sum_f1 c(f1) Re(Gt(f1, t) w^(s f1))  (K = H1; c = 1 at f1 = 0
//                          and at the Nyquist column of an even L, 2 elsewhere)
// with w = exp(2 pi i / L), planes [ch][Ly][Lx] zero-extended to L x L and
// half spectra [ch][nf], f = f1 + H1 f2.  Each thread owns an 8 x 2 (complex)
// or 8 x 4 (real) output block: per reduction step it reads 4-6 16-byte words
// from shared memory for 32-64 FMAs.
struct DftDims {
    int Lx, Ly, L, H1;
    int H1p, Lyp, Lxp, Lp;  // padded: 2 | H1p, 8 | Lyp, 4 | Lxp, 8 | Lp
    int N;
    int64_t X, Y;
};

constexpr int kDftThreads = 224;

static DftDims dft_dims(const sid_plan* p)
{
    DftDims d;
    d.Lx = (int)p->Lx;
    d.Ly = (int)p->Ly;
    d.L = (int)p->L;
    d.H1 = d.L / 2 + 1;
    d.H1p = (int)cdiv(d.H1, 2) * 2;
    d.Lyp = (int)cdiv(d.Ly, 8) * 8;
    d.Lxp = (int)cdiv(d.Lx, 4) * 4;
    d.Lp = (int)cdiv(d.L, 8) * 8;
    d.N = (int)p->N;
    d.X = p->X;
    d.Y = p->Y;
    return d;
}

static size_t r2c_smem(const DftDims& d)
{
    return (size_t)(d.Lx * d.H1p + d.Ly * d.Lp + d.Lyp * d.H1p) * sizeof(float2) +
           (size_t)(d.Lx * d.Lyp) * sizeof(float);
}
static size_t c2r_smem(const DftDims& d)
{
    const size_t u = std::max((size_t)d.L * d.H1p, (size_t)d.H1 * d.Lxp);
    return ((size_t)d.L * d.Lyp + (size_t)d.H1p * d.Lyp + u) * sizeof(float2);
}

__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

__global__ void __launch_bounds__(kDftThreads, 2)
k_dft_r2c(const float* __restrict__ in, float2* __restrict__ out, const float2* __restrict__ tw, DftDims d,
          int64_t nch)
{
    extern __shared__ __align__(16) unsigned char dft_sm[];
    float2* C1 = reinterpret_cast<float2*>(dft_sm);         // [Lx][H1p]  conj(w^(u f1))
    float2* C2 = C1 + d.Lx * d.H1p;                          // [Ly][Lp]   conj(w^(v f2))
    float2* G = C2 + d.Ly * d.Lp;                            // [Lyp][H1p]
    float* img = reinterpret_cast<float*>(G + d.Lyp * d.H1p);  // [Lx][Lyp] (transposed plane)
    const int L = d.L, H1 = d.H1, nf = H1 * L;
    for (int i = threadIdx.x; i < d.Lx * d.H1p; i += blockDim.x) {
        const int u = i / d.H1p, f1 = i - u * d.H1p;
        C1[i] = f1 < H1 ? cconj(tw[(u * f1) % L]) : make_float2(0.f, 0.f);
    }
    for (int i = threadIdx.x; i < d.Ly * d.Lp; i += blockDim.x) {
        const int v = i / d.Lp, f2 = i - v * d.Lp;
        C2[i] = f2 < L ? cconj(tw[(v * f2) % L]) : make_float2(0.f, 0.f);
    }
    for (int i = threadIdx.x; i < d.Lx * d.Lyp; i += blockDim.x) img[i] = 0.f;  // rows v >= Ly stay zero
    __syncthreads();
    const int nvb = d.Lyp / 8, nfb = d.H1p / 2, nf2b = d.Lp / 8;
    for (int64_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        const float* src = in + ch * (int64_t)d.Ly * d.Lx;
        for (int i = threadIdx.x; i < d.Ly * d.Lx; i += blockDim.x) {
            const int v = i / d.Lx, u = i - v * d.Lx;
            img[u * d.Lyp + v] = src[i];
        }
        __syncthreads();
        // G = x * C1: rows v (8 per thread), column pairs f1
        for (int task = threadIdx.x; task < nvb * nfb; task += blockDim.x) {
            const int fb = task % nfb, vb = task / nfb;
            float acc[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            const float* ap = img + vb * 8;
            const float2* cp = C1 + fb * 2;
#pragma unroll 2
            for (int u = 0; u < d.Lx; ++u) {
                const float4 a0 = *reinterpret_cast<const float4*>(ap + u * d.Lyp);
                const float4 a1 = *reinterpret_cast<const float4*>(ap + u * d.Lyp + 4);
                const float4 c = *reinterpret_cast<const float4*>(cp + u * d.H1p);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    acc[j][0] = fmaf(a[j], c.x, acc[j][0]);
                    acc[j][1] = fmaf(a[j], c.y, acc[j][1]);
                    acc[j][2] = fmaf(a[j], c.z, acc[j][2]);
                    acc[j][3] = fmaf(a[j], c.w, acc[j][3]);
                }
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<float4*>(G + (vb * 8 + j) * d.H1p + fb * 2) =
                    make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
        }
        __syncthreads();
        // X = C2' * G: rows f2 (8 per thread), column pairs f1
        float2* dst = out + ch * (int64_t)nf;
        for (int task = threadIdx.x; task < nf2b * nfb; task += blockDim.x) {
            const int fb = task % nfb, f2b = task / nfb;
            float acc[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            const float2* gp = G + fb * 2;
            const float2* wp = C2 + f2b * 8;
#pragma unroll 2
            for (int v = 0; v < d.Ly; ++v) {
                const float4 g = *reinterpret_cast<const float4*>(gp + v * d.H1p);
                float2 w[8];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 t = *reinterpret_cast<const float4*>(wp + v * d.Lp + 2 * q);
                    w[2 * q] = make_float2(t.x, t.y);
                    w[2 * q + 1] = make_float2(t.z, t.w);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    acc[j][0] = fmaf(w[j].x, g.x, fmaf(-w[j].y, g.y, acc[j][0]));
                    acc[j][1] = fmaf(w[j].x, g.y, fmaf(w[j].y, g.x, acc[j][1]));
                    acc[j][2] = fmaf(w[j].x, g.z, fmaf(-w[j].y, g.w, acc[j][2]));
                    acc[j][3] = fmaf(w[j].x, g.w, fmaf(w[j].y, g.z, acc[j][3]));
                }
            }
            const int f1 = fb * 2;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int f2 = f2b * 8 + j;
                if (f2 >= L) break;
                dst[f2 * H1 + f1] = make_float2(acc[j][0], acc[j][1]);
                if (f1 + 1 < H1) dst[f2 * H1 + f1 + 1] = make_float2(acc[j][2], acc[j][3]);
            }
        }
        // no barrier: the next plane load writes only img, which this pass does not read
    }
}

// Lattice positions outside the X x Y frame are written as zero.
__global__ void __launch_bounds__(kDftThreads, 2)
k_dft_c2r(const float2* __restrict__ in, float* __restrict__ out, const float2* __restrict__ tw, DftDims d,
          int64_t nch)
{
    extern __shared__ __align__(16) unsigned char dft_sm[];
    float2* D1 = reinterpret_cast<float2*>(dft_sm);  // [L][Lyp]  w^(t f2)
    float2* Gt = D1 + d.L * d.Lyp;                   // [H1p][Lyp]
    float2* S = Gt + d.H1p * d.Lyp;                  // [L][H1p] spectrum, then E [H1][Lxp]
    float2* E = S;
    const int L = d.L, H1 = d.H1, nf = H1 * L;
    const bool even = (L % 2) == 0;
    for (int i = threadIdx.x; i < d.L * d.Lyp; i += blockDim.x) {
        const int f2 = i / d.Lyp, t = i - f2 * d.Lyp;
        D1[i] = t < d.Ly ? tw[(t * f2) % L] : make_float2(0.f, 0.f);
    }
    const float inv = 1.0f / ((float)L * (float)L);
    const int ntb = d.Lyp / 8, nfb = d.H1p / 2, nsb = d.Lxp / 4;
    for (int64_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        const float2* src = in + ch * (int64_t)nf;
        for (int i = threadIdx.x; i < d.L * d.H1p; i += blockDim.x) {
            const int f2 = i / d.H1p, f1 = i - f2 * d.H1p;
            S[i] = f1 < H1 ? src[f2 * H1 + f1] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        // Gt = (D1' S)': rows t (8 per thread), column pairs f1
        for (int task = threadIdx.x; task < ntb * nfb; task += blockDim.x) {
            const int fb = task % nfb, tb = task / nfb;
            float acc[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            const float2* sp = S + fb * 2;
            const float2* wp = D1 + tb * 8;
#pragma unroll 2
            for (int f2 = 0; f2 < L; ++f2) {
                const float4 g = *reinterpret_cast<const float4*>(sp + f2 * d.H1p);
                float2 w[8];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 t = *reinterpret_cast<const float4*>(wp + f2 * d.Lyp + 2 * q);
                    w[2 * q] = make_float2(t.x, t.y);
                    w[2 * q + 1] = make_float2(t.z, t.w);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    acc[j][0] = fmaf(w[j].x, g.x, fmaf(-w[j].y, g.y, acc[j][0]));
                    acc[j][1] = fmaf(w[j].x, g.y, fmaf(w[j].y, g.x, acc[j][1]));
                    acc[j][2] = fmaf(w[j].x, g.z, fmaf(-w[j].y, g.w, acc[j][2]));
                    acc[j][3] = fmaf(w[j].x, g.w, fmaf(w[j].y, g.z, acc[j][3]));
                }
            }
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                float2* gr = Gt + (fb * 2 + m) * d.Lyp + tb * 8;
#pragma unroll
                for (int j = 0; j < 8; j += 2)
                    *reinterpret_cast<float4*>(gr + j) =
                        make_float4(acc[j][2 * m], acc[j][2 * m + 1], acc[j + 1][2 * m], acc[j + 1][2 * m + 1]);
            }
        }
        __syncthreads();
        // E(f1, s) = c(f1) w^(s f1) over the spectrum's space
        for (int i = threadIdx.x; i < H1 * d.Lxp; i += blockDim.x) {
            const int f1 = i / d.Lxp, s = i - f1 * d.Lxp;
            const float c = (f1 == 0 || (even && f1 == H1 - 1)) ? 1.f : 2.f;
            const float2 w = tw[(s * f1) % L];
            E[i] = s < d.Lx ? make_float2(c * w.x, c * w.y) : make_float2(0.f, 0.f);
        }
        __syncthreads();
        // x = Re(Gt' E) / L^2: rows t (8 per thread), columns s (4 per thread)
        const int a = (int)(ch % d.N), b = (int)((ch / d.N) % d.N);
        float* dst = out + ch * (int64_t)d.Ly * d.Lx;
        for (int task = threadIdx.x; task < ntb * nsb; task += blockDim.x) {
            const int sb = task % nsb, tb = task / nsb;
            float acc[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            const float2* gp = Gt + tb * 8;
            const float2* ep = E + sb * 4;
#pragma unroll 2
            for (int f1 = 0; f1 < H1; ++f1) {
                float2 g[8];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 t = *reinterpret_cast<const float4*>(gp + f1 * d.Lyp + 2 * q);
                    g[2 * q] = make_float2(t.x, t.y);
                    g[2 * q + 1] = make_float2(t.z, t.w);
                }
                const float4 e0 = *reinterpret_cast<const float4*>(ep + f1 * d.Lxp);
                const float4 e1 = *reinterpret_cast<const float4*>(ep + f1 * d.Lxp + 2);
                const float2 e[4] = {make_float2(e0.x, e0.y), make_float2(e0.z, e0.w), make_float2(e1.x, e1.y),
                                     make_float2(e1.z, e1.w)};
#pragma unroll
                for (int j = 0; j < 8; ++j)
#pragma unroll
                    for (int k = 0; k < 4; ++k) acc[j][k] = fmaf(g[j].x, e[k].x, fmaf(-g[j].y, e[k].y, acc[j][k]));
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int t = tb * 8 + j;
                if (t >= d.Ly) break;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int s = sb * 4 + k;
                    if (s >= d.Lx) break;
                    const bool inside = (a + (int64_t)d.N * s) < d.X && (b + (int64_t)d.N * t) < d.Y;
                    dst[t * d.Lx + s] = inside ? acc[j][k] * inv : 0.f;
                }
            }
        }
        __syncthreads();
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

// The reduction may be restricted to the vectors [jv0, jv1) of each row (input
// channels [EPL jv0, EPL jv1)); accum adds the result to ihat instead of
// storing it (a projection formed depth slab by depth slab).
template <bool I16>
__global__ void __launch_bounds__(512)
k_spec_fwd(const uint4* __restrict__ khat, const float* __restrict__ rstep, const float2* __restrict__ vhat,
           float2* __restrict__ ihat, int n_in, int64_t n_in_pad, int n_out, int nf, int jv0, int jv1, int accum)
{
    using KL = KLoad<I16>;
    constexpr int EPL = KL::EPL;
    extern __shared__ float2 xv[];  // [EPL (jv1 - jv0)]: channels EPL jv0 ..
    const int f = blockIdx.x;
    const int kb = EPL * jv0, nk = EPL * (jv1 - jv0);
    for (int k = threadIdx.x; k < nk; k += blockDim.x)
        xv[k] = (kb + k < n_in) ? vhat[(int64_t)(kb + k) * nf + f] : make_float2(0.f, 0.f);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
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
        for (int j = jv0 + lane; j < jv1; j += 32) {
            uint4 q[kRB];
#pragma unroll
            for (int r = 0; r < kRB; ++r) q[r] = __ldcs(kr[r] + j);
            float2 x[EPL];
#pragma unroll
            for (int e = 0; e < EPL; ++e) x[e] = xv[EPL * (j - jv0) + e];
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
            float2* dst = ihat + (int64_t)o * nf + f;
            if (accum) {
                const float2 prev = *dst;
                *dst = make_float2(prev.x + re * st, prev.y + im * st);
            } else {
                *dst = make_float2(re * st, im * st);
            }
        }
    }
}

// 24-bit float spectra: eight complex entries per two 16-byte high-plane
// words (re, im high halves) and one 16-byte low-plane word (re, im low bytes).
__device__ __forceinline__ void unpack_f24(const uint4& q0, const uint4& q1, const uint4& l, float2 (&k)[8])
{
    const unsigned w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
    const unsigned lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const unsigned lb = lw[e >> 1] >> (16 * (e & 1));
        k[e].x = __uint_as_float(((w[e] & 0xFFFFu) << 16) | ((lb & 0xFFu) << 8));
        k[e].y = __uint_as_float((w[e] & 0xFFFF0000u) | (((lb >> 8) & 0xFFu) << 8));
    }
}

// Adjoint: per frequency f, Bhat[k][f] = sum_o conj(Khat[f][o][k]) * step(f,o) * Ihat[o][f].
// FMT: FMT_F32 (khat float2), FMT_I16 (short2 mantissas and row steps) or
// FMT_F24 (khat = high plane, klo = low plane).
template <int FMT>
__global__ void __launch_bounds__(512)
k_spec_adj(const uint4* __restrict__ khat, const uint4* __restrict__ klo, const float* __restrict__ rstep,
           const float2* __restrict__ ihat, float2* __restrict__ bhat, int n_in, int64_t n_in_pad, int n_out, int nf)
{
    // channels per thread: one 16-byte word of FP32 (2) or 16-bit (4) entries;
    // three 16-byte words (two high, one low) of 24-bit entries (8)
    constexpr int V = FMT == FMT_F32 ? 2 : (FMT == FMT_I16 ? 4 : 8);
    extern __shared__ float2 yv[];  // [n_out], pre-multiplied by the row steps
    const int f = blockIdx.x;
    for (int o = threadIdx.x; o < n_out; o += blockDim.x) {
        const float2 y = ihat[(int64_t)o * nf + f];
        const float st = FMT == FMT_I16 ? rstep[(int64_t)f * n_out + o] : 1.f;
        yv[o] = make_float2(y.x * st, y.y * st);
    }
    __syncthreads();
    const int nvec = (int)(n_in_pad / V);
    // 16-byte words per row: high plane (or the only plane) and low plane
    const int64_t rowvec = FMT == FMT_F24 ? n_in_pad / 4 : n_in_pad / V;
    const int64_t rowlo = n_in_pad / 8;
    const uint4* base = khat + (int64_t)f * n_out * rowvec;
    const uint4* lbase = FMT == FMT_F24 ? klo + (int64_t)f * n_out * rowlo : nullptr;
    for (int j = threadIdx.x; j < nvec; j += blockDim.x) {
        float ar[V], ai[V];
#pragma unroll
        for (int e = 0; e < V; ++e) ar[e] = ai[e] = 0.f;
        const uint4* col = base + (FMT == FMT_F24 ? 2 * j : j);
        const uint4* lcol = FMT == FMT_F24 ? lbase + j : nullptr;
#pragma unroll 4
        for (int o = 0; o < n_out; ++o) {
            const float2 y = yv[o];
            float2 kk[V];
            if constexpr (FMT == FMT_F24) {
                unpack_f24(__ldcs(col + (int64_t)o * rowvec), __ldcs(col + (int64_t)o * rowvec + 1),
                           __ldcs(lcol + (int64_t)o * rowlo), kk);
            } else {
                KLoad<FMT == FMT_I16>::unpack(__ldcs(col + (int64_t)o * rowvec), kk);
            }
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

// ------------------------------------------------ several volumes at once --
// The same contractions for NB volumes per launch (reconstruct_S.m:162-212
// reconstructs components side by side): each tap-spectrum entry read from
// HBM is applied to NB volume spectra, so the spectra stream once per NB
// volumes and the contraction turns from memory- to FMA-bound.  Layouts:
// vhat [b][k][f], ihat [b][o][f] (NB consecutive single-volume blocks).
template <bool I16, int NB>
__global__ void __launch_bounds__(512)
k_spec_fwd_b(const uint4* __restrict__ khat, const float* __restrict__ rstep, const float2* __restrict__ vhat,
             float2* __restrict__ ihat, int n_in, int64_t n_in_pad, int n_out, int nf)
{
    using KL = KLoad<I16>;
    constexpr int EPL = KL::EPL;
    constexpr int RBB = 2;  // rows per warp pass (NB x RBB complex accumulators per lane)
    extern __shared__ float2 xv[];  // [NB][n_in_pad]
    const int f = blockIdx.x;
    for (int b = 0; b < NB; ++b)
        for (int k = threadIdx.x; k < n_in_pad; k += blockDim.x)
            xv[b * n_in_pad + k] = (k < n_in) ? vhat[((int64_t)b * n_in + k) * nf + f] : make_float2(0.f, 0.f);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nvec = (int)(n_in_pad / EPL);
    const int64_t rowvec = n_in_pad / EPL;
    for (int o0 = warp * RBB; o0 < n_out; o0 += nw * RBB) {
        float ar[RBB][NB], ai[RBB][NB];
        const uint4* kr[RBB];
#pragma unroll
        for (int r = 0; r < RBB; ++r) {
#pragma unroll
            for (int b = 0; b < NB; ++b) ar[r][b] = ai[r][b] = 0.f;
            kr[r] = khat + ((int64_t)f * n_out + min(o0 + r, n_out - 1)) * rowvec;
        }
#pragma unroll 2
        for (int j = lane; j < nvec; j += 32) {
            uint4 q[RBB];
#pragma unroll
            for (int r = 0; r < RBB; ++r) q[r] = __ldcs(kr[r] + j);
            float2 kk[RBB][EPL];
#pragma unroll
            for (int r = 0; r < RBB; ++r) KL::unpack(q[r], kk[r]);
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                float2 x[EPL];
#pragma unroll
                for (int e = 0; e < EPL; ++e) x[e] = xv[b * n_in_pad + EPL * j + e];
#pragma unroll
                for (int r = 0; r < RBB; ++r)
#pragma unroll
                    for (int e = 0; e < EPL; ++e) {
                        ar[r][b] = fmaf(kk[r][e].x, x[e].x, ar[r][b]);
                        ar[r][b] = fmaf(-kk[r][e].y, x[e].y, ar[r][b]);
                        ai[r][b] = fmaf(kk[r][e].x, x[e].y, ai[r][b]);
                        ai[r][b] = fmaf(kk[r][e].y, x[e].x, ai[r][b]);
                    }
            }
        }
#pragma unroll
        for (int r = 0; r < RBB; ++r)
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    ar[r][b] += __shfl_xor_sync(0xffffffffu, ar[r][b], off);
                    ai[r][b] += __shfl_xor_sync(0xffffffffu, ai[r][b], off);
                }
        // lane r * NB + b writes row o0 + r of volume b
#pragma unroll
        for (int r = 0; r < RBB; ++r)
#pragma unroll
            for (int b = 0; b < NB; ++b)
                if (lane == r * NB + b && o0 + r < n_out) {
                    const int o = o0 + r;
                    const float st = I16 ? rstep[(int64_t)f * n_out + o] : 1.f;
                    ihat[((int64_t)b * n_out + o) * nf + f] = make_float2(ar[r][b] * st, ai[r][b] * st);
                }
    }
}

template <int FMT, int NB>
__global__ void __launch_bounds__(512)
k_spec_adj_b(const uint4* __restrict__ khat, const uint4* __restrict__ klo, const float* __restrict__ rstep,
             const float2* __restrict__ ihat, float2* __restrict__ bhat, int n_in, int64_t n_in_pad, int n_out, int nf)
{
    constexpr int V = FMT == FMT_F32 ? 2 : (FMT == FMT_I16 ? 4 : 8);
    extern __shared__ float2 yv[];  // [NB][n_out], pre-multiplied by the row steps
    const int f = blockIdx.x;
    for (int i = threadIdx.x; i < NB * n_out; i += blockDim.x) {
        const int b = i / n_out, o = i - b * n_out;
        const float2 y = ihat[((int64_t)b * n_out + o) * nf + f];
        const float st = FMT == FMT_I16 ? rstep[(int64_t)f * n_out + o] : 1.f;
        yv[i] = make_float2(y.x * st, y.y * st);
    }
    __syncthreads();
    const int nvec = (int)(n_in_pad / V);
    const int64_t rowvec = FMT == FMT_F24 ? n_in_pad / 4 : n_in_pad / V;
    const int64_t rowlo = n_in_pad / 8;
    const uint4* base = khat + (int64_t)f * n_out * rowvec;
    const uint4* lbase = FMT == FMT_F24 ? klo + (int64_t)f * n_out * rowlo : nullptr;
    for (int j = threadIdx.x; j < nvec; j += blockDim.x) {
        float ar[NB][V], ai[NB][V];
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int e = 0; e < V; ++e) ar[b][e] = ai[b][e] = 0.f;
        const uint4* col = base + (FMT == FMT_F24 ? 2 * j : j);
        const uint4* lcol = FMT == FMT_F24 ? lbase + j : nullptr;
#pragma unroll 2
        for (int o = 0; o < n_out; ++o) {
            float2 kk[V];
            if constexpr (FMT == FMT_F24) {
                unpack_f24(__ldcs(col + (int64_t)o * rowvec), __ldcs(col + (int64_t)o * rowvec + 1),
                           __ldcs(lcol + (int64_t)o * rowlo), kk);
            } else {
                KLoad<FMT == FMT_I16>::unpack(__ldcs(col + (int64_t)o * rowvec), kk);
            }
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                const float2 y = yv[b * n_out + o];
#pragma unroll
                for (int e = 0; e < V; ++e) {
                    ar[b][e] = fmaf(kk[e].x, y.x, ar[b][e]); ar[b][e] = fmaf(kk[e].y, y.y, ar[b][e]);
                    ai[b][e] = fmaf(kk[e].x, y.y, ai[b][e]); ai[b][e] = fmaf(-kk[e].y, y.x, ai[b][e]);
                }
            }
        }
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int e = 0; e < V; ++e) {
                const int k = V * j + e;
                if (k < n_in) bhat[((int64_t)b * n_in + k) * nf + f] = make_float2(ar[b][e], ai[b][e]);
            }
    }
}

// ------------------------------------------------------------- launchers --
int ensure_spec_ws(sid_plan* p)
{
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N;
    SID_TRY(p->vhat.alloc((size_t)(n_in * p->nf) * sizeof(float2)));
    SID_TRY(p->ihat.alloc((size_t)(n_out * p->nf) * sizeof(float2)));
    return SID_OK;
}

static int configure_dft(const sid_plan* p)
{
    const DftDims d = dft_dims(p);
    SID_REQUIRE(r2c_smem(d) <= 220 * 1024 && c2r_smem(d) <= 220 * 1024,
                "spectral projector: lenslet grid %lldx%lld (L=%lld) exceeds the DFT kernels' shared memory",
                (long long)p->Lx, (long long)p->Ly, (long long)p->L);
    SID_TRY(smem_attr((const void*)k_dft_r2c, r2c_smem(d)));
    SID_TRY(smem_attr((const void*)k_dft_c2r, c2r_smem(d)));
    return SID_OK;
}

// persistent DFT grids: at most two CTAs per SM (shared-memory bound)
static unsigned dft_grid(int64_t nch) { return (unsigned)std::min<int64_t>(nch, 2 * 152); }

int fft_r2c(const sid_plan* p, const float* in, float2* out, int64_t nch, cudaStream_t st);
int fft_c2r(const sid_plan* p, const float2* in, float* out, int64_t nch, cudaStream_t st);

// lenslet-grid transforms: mixed-radix FFTs (fft.cu) when L factors as 2^a * odd,
// else the matrix DFTs above
static int dft_r2c(const sid_plan* p, const float* in, float2* out, int64_t nch, cudaStream_t st)
{
    int P = 0, Q = 0;
    if (fft_factor(p->L, &P, &Q)) return fft_r2c(p, in, out, nch, st);
    const DftDims d = dft_dims(p);
    k_dft_r2c<<<dft_grid(nch), kDftThreads, r2c_smem(d), st>>>(in, out, p->twiddle.as<float2>(), d, nch);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

static int dft_c2r(const sid_plan* p, const float2* in, float* out, int64_t nch, cudaStream_t st)
{
    int P = 0, Q = 0;
    if (fft_factor(p->L, &P, &Q)) return fft_c2r(p, in, out, nch, st);
    const DftDims d = dft_dims(p);
    k_dft_c2r<<<dft_grid(nch), kDftThreads, c2r_smem(d), st>>>(in, out, p->twiddle.as<float2>(), d, nch);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spec_r2c(sid_plan* p, const float* in, float2* out, int64_t nch, cudaStream_t st)
{
    SID_TRY(configure_dft(p));
    return dft_r2c(p, in, out, nch, st);
}

int spec_c2r(sid_plan* p, const float2* in, float* out, int64_t nch, cudaStream_t st)
{
    SID_TRY(configure_dft(p));
    return dft_c2r(p, in, out, nch, st);
}

static int spec_check(const sid_plan* p, int fmt)
{
    if (fmt == FMT_I16 && !p->spec_i16) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_I16");
        return SID_ENOTSUP;
    }
    if (fmt == FMT_F32 && !p->spec_f32) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_F32");
        return SID_ENOTSUP;
    }
    if (fmt == FMT_F24 && !p->spec_f24) {
        set_error("spectral projector: plan was built without SID_PLAN_SPECTRAL_F24");
        return SID_ENOTSUP;
    }
    return SID_OK;
}

int spectral_forward(sid_plan* p, bool i16, const float* vp, float* ip, cudaStream_t st)
{
    SID_TRY(spec_check(p, i16 ? FMT_I16 : FMT_F32));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    SID_TRY(dft_r2c(p, vp, p->vhat.as<float2>(), n_in, st));
    SID_TRY(spectral_forward_part(p, i16, 0, n_in, false, st));
    (void)n_in_pad;
    SID_TRY(dft_c2r(p, p->ihat.as<float2>(), ip, n_out, st));
    return SID_OK;
}

int spectral_forward_part(sid_plan* p, bool i16, int64_t c0, int64_t c1, bool accum, cudaStream_t st)
{
    SID_TRY(spec_check(p, i16 ? FMT_I16 : FMT_F32));
    SID_TRY(ensure_spec_ws(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    const int epl = i16 ? 4 : 2;
    SID_REQUIRE(c0 >= 0 && c0 < c1 && c1 <= n_in && c0 % epl == 0,
                "spectral forward: channel range [%lld, %lld) not on a %d-channel boundary", (long long)c0,
                (long long)c1, epl);
    const int jv0 = (int)(c0 / epl), jv1 = (int)(c1 == n_in ? n_in_pad / epl : cdiv(c1, epl));
    const size_t sm = (size_t)(jv1 - jv0) * epl * sizeof(float2);
    p->timer.begin(st);
    if (i16) {
        SID_TRY(smem_attr((const void*)k_spec_fwd<true>, sm));
        k_spec_fwd<true><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_i16.as<uint4>(), p->rstep.as<float>(),
                                                          p->vhat.as<float2>(), p->ihat.as<float2>(), (int)n_in,
                                                          n_in_pad, (int)n_out, (int)p->nf, jv0, jv1, accum ? 1 : 0);
    } else {
        SID_TRY(smem_attr((const void*)k_spec_fwd<false>, sm));
        k_spec_fwd<false><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.as<uint4>(), nullptr, p->vhat.as<float2>(),
                                                           p->ihat.as<float2>(), (int)n_in, n_in_pad, (int)n_out,
                                                           (int)p->nf, jv0, jv1, accum ? 1 : 0);
    }
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_adjoint_spectra(sid_plan* p, int fmt, const float* ip, cudaStream_t st)
{
    SID_TRY(spec_check(p, fmt));
    SID_TRY(ensure_spec_ws(p));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    SID_TRY(dft_r2c(p, ip, p->ihat.as<float2>(), n_out, st));
    const size_t sm = (size_t)n_out * sizeof(float2);
    p->timer.begin(st);
    if (fmt == FMT_I16)
        k_spec_adj<FMT_I16><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_i16.as<uint4>(), nullptr, p->rstep.as<float>(),
                                                             p->ihat.as<float2>(), p->vhat.as<float2>(), (int)n_in,
                                                             n_in_pad, (int)n_out, (int)p->nf);
    else if (fmt == FMT_F24)
        k_spec_adj<FMT_F24><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f24h.as<uint4>(), p->khat_f24l.as<uint4>(),
                                                             nullptr, p->ihat.as<float2>(), p->vhat.as<float2>(),
                                                             (int)n_in, n_in_pad, (int)n_out, (int)p->nf);
    else
        k_spec_adj<FMT_F32><<<(unsigned)p->nf, 512, sm, st>>>(p->khat_f32.as<uint4>(), nullptr, nullptr,
                                                             p->ihat.as<float2>(), p->vhat.as<float2>(), (int)n_in,
                                                             n_in_pad, (int)n_out, (int)p->nf);
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_adjoint(sid_plan* p, int fmt, const float* ip, float* bp, cudaStream_t st)
{
    SID_TRY(spectral_adjoint_spectra(p, fmt, ip, st));
    return dft_c2r(p, p->vhat.as<float2>(), bp, p->N * p->N * p->Z, st);
}

// nb (2..4) volumes per call: vp holds nb polyphase volumes, ip nb polyphase images
constexpr int kSpecBatchMax = 4;

static int ensure_spec_ws_b(sid_plan* p, int nb)
{
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N;
    SID_TRY(p->vhat.alloc((size_t)(nb * n_in * p->nf) * sizeof(float2)));
    SID_TRY(p->ihat.alloc((size_t)(nb * n_out * p->nf) * sizeof(float2)));
    return SID_OK;
}

template <bool I16, int NB>
static int launch_fwd_b(sid_plan* p, int64_t n_in, int64_t n_in_pad, int64_t n_out, cudaStream_t st)
{
    const size_t sm = (size_t)NB * n_in_pad * sizeof(float2);
    SID_REQUIRE(sm <= 227 * 1024, "spectral projector: %d volumes of %lld channels exceed shared memory", NB,
                (long long)n_in);
    SID_TRY(smem_attr((const void*)k_spec_fwd_b<I16, NB>, sm));
    k_spec_fwd_b<I16, NB><<<(unsigned)p->nf, 512, sm, st>>>(I16 ? p->khat_i16.as<uint4>() : p->khat_f32.as<uint4>(),
                                                           I16 ? p->rstep.as<float>() : nullptr, p->vhat.as<float2>(),
                                                           p->ihat.as<float2>(), (int)n_in, n_in_pad, (int)n_out,
                                                           (int)p->nf);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

template <int FMT, int NB>
static int launch_adj_b(sid_plan* p, int64_t n_in, int64_t n_in_pad, int64_t n_out, cudaStream_t st)
{
    const size_t sm = (size_t)NB * n_out * sizeof(float2);
    const uint4* kh = FMT == FMT_I16 ? p->khat_i16.as<uint4>() : (FMT == FMT_F24 ? p->khat_f24h.as<uint4>()
                                                                                  : p->khat_f32.as<uint4>());
    k_spec_adj_b<FMT, NB><<<(unsigned)p->nf, 512, sm, st>>>(kh, FMT == FMT_F24 ? p->khat_f24l.as<uint4>() : nullptr,
                                                           FMT == FMT_I16 ? p->rstep.as<float>() : nullptr,
                                                           p->ihat.as<float2>(), p->vhat.as<float2>(), (int)n_in,
                                                           n_in_pad, (int)n_out, (int)p->nf);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int spectral_forward_batch(sid_plan* p, bool i16, const float* vp, float* ip, int nb, cudaStream_t st)
{
    if (nb == 1) return spectral_forward(p, i16, vp, ip, st);
    SID_REQUIRE(nb >= 2 && nb <= kSpecBatchMax, "spectral projector: batch of %d volumes outside [1, %d]", nb,
                kSpecBatchMax);
    SID_TRY(spec_check(p, i16 ? FMT_I16 : FMT_F32));
    SID_TRY(ensure_spec_ws_b(p, nb));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    SID_TRY(dft_r2c(p, vp, p->vhat.as<float2>(), nb * n_in, st));
    p->timer.begin(st);
    int rc;
    if (i16) rc = nb == 2 ? launch_fwd_b<true, 2>(p, n_in, n_in_pad, n_out, st)
                          : (nb == 3 ? launch_fwd_b<true, 3>(p, n_in, n_in_pad, n_out, st)
                                     : launch_fwd_b<true, 4>(p, n_in, n_in_pad, n_out, st));
    else rc = nb == 2 ? launch_fwd_b<false, 2>(p, n_in, n_in_pad, n_out, st)
                      : (nb == 3 ? launch_fwd_b<false, 3>(p, n_in, n_in_pad, n_out, st)
                                 : launch_fwd_b<false, 4>(p, n_in, n_in_pad, n_out, st));
    p->timer.finish(st);
    SID_TRY(rc);
    return dft_c2r(p, p->ihat.as<float2>(), ip, nb * n_out, st);
}

int spectral_adjoint_batch(sid_plan* p, int fmt, const float* ip, float* bp, int nb, cudaStream_t st)
{
    if (nb == 1) return spectral_adjoint(p, fmt, ip, bp, st);
    SID_REQUIRE(nb >= 2 && nb <= kSpecBatchMax, "spectral projector: batch of %d volumes outside [1, %d]", nb,
                kSpecBatchMax);
    SID_TRY(spec_check(p, fmt));
    SID_TRY(ensure_spec_ws_b(p, nb));
    SID_TRY(configure_dft(p));
    const int64_t n_in = p->N * p->N * p->Z, n_out = p->N * p->N, n_in_pad = spec_nin_pad(p);
    SID_TRY(dft_r2c(p, ip, p->ihat.as<float2>(), nb * n_out, st));
    p->timer.begin(st);
    int rc;
#define SID_ADJ_B(F)                                                                                        \
    (nb == 2 ? launch_adj_b<F, 2>(p, n_in, n_in_pad, n_out, st)                                             \
             : (nb == 3 ? launch_adj_b<F, 3>(p, n_in, n_in_pad, n_out, st) : launch_adj_b<F, 4>(p, n_in, n_in_pad, n_out, st)))
    if (fmt == FMT_I16) rc = SID_ADJ_B(FMT_I16);
    else if (fmt == FMT_F24) rc = SID_ADJ_B(FMT_F24);
    else rc = SID_ADJ_B(FMT_F32);
#undef SID_ADJ_B
    p->timer.finish(st);
    SID_TRY(rc);
    return dft_c2r(p, p->vhat.as<float2>(), bp, nb * n_in, st);
}

}  // namespace sid
