// fft.cu -- lenslet-grid real DFTs of the spectral projector as mixed-radix
// FFTs (the replacement for the matrix DFTs of spectral.cu when the DFT length
// L factors as P * Q, P a power of two in [4, 64], Q odd and at most 15).
//
// A length-L transform X[k] = sum_n x[n] w^(-+nk) (w = exp(2 pi i / L)) is
// split with n = Q n1 + n2 and k = k1 + P k2 (Cooley-Tukey):
//   A[n2][k1] = w^(-+ n2 k1) sum_{n1 < P} x[Q n1 + n2] w_P^(-+ n1 k1)   P-point FFTs
//   X[k1 + P k2] = sum_{n2 < Q} A[n2][k1] w_Q^(-+ n2 k2)                 Q-point DFTs
// The P-point FFTs run in registers (radix-2, decimation in frequency, fully
// unrolled), one per thread; the Q-point DFTs are direct sums.  A 2-D real
// transform of a plane [Ly][Lx] (zero-extended to L x L) is
//   analysis:  rows paired as z = x_v + i x_{v+1}, one complex FFT per pair;
//              one thread computes the Q-point sums of k1 and P - k1, so it
//              holds Z(f) and Z(-f) and separates the two half spectra in
//              registers; then the columns (complex, length L) of the
//              Ly x (L/2 + 1) half plane;
//   synthesis: the columns inverse-transformed (only t < Ly computed), then
//              row pairs packed as Z = S_t + i S_{t+1} over the
//              Hermitian-extended spectrum, one inverse complex FFT per pair,
//              real part -> row t, imaginary part -> row t + 1.
// Layouts are those of the matrix DFTs: planes [ch][Ly][Lx], half spectra
// [ch][f] with f = f1 + H1 f2, H1 = L/2 + 1.  CTAs are persistent over channels
// and fetch the next channel's input into registers while transforming the
// current one.  Shared-memory layout per CTA:
//   stw [L]                 twiddles
//   A   [nseq][Q][P + 1]    step-A outputs (row pitch P + 1: conflict-free)
//   U   plane [Ly][Lx] | half plane [Ly][gs] (analysis)
//       half spectrum [L][gs] | half plane [Ly][gs] (synthesis)
// with gs >= H1, gs = Q^-1 (mod 16): the stride-Q column gathers of 16 threads
// then touch 16 distinct 8-byte bank pairs.
#include <algorithm>
#include <cmath>

#include "sid_internal.cuh"

namespace sid {

namespace {

constexpr int kFftThreads = 256;
// two CTAs per SM at least (128 registers; the measured optimum at L = 80:
// three CTAs at 80 registers spill and run no faster)
constexpr int kFftMinBlocks = 2;
constexpr int kPfR = 18;  // analysis: input floats per thread prefetched in registers
constexpr int kPfC = 13;  // synthesis: input float2 per thread prefetched in registers

struct FftDims {
    int Lx, Ly, L, H1, Q, npair, nseq, gs;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// w^m (inverse transform) or its conjugate (forward transform)
template <bool INV> __device__ __forceinline__ float2 twid(const float2* stw, int m)
{
    const float2 w = stw[m];
    return INV ? w : make_float2(w.x, -w.y);
}

constexpr int bitrev(int i, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
constexpr int ilog2(int p) { return p <= 1 ? 0 : 1 + ilog2(p >> 1); }

// In-place P-point FFT of v (radix-2 decimation in frequency): natural-order
// input, bit-reversed output.  Twiddles w_{2h}^j = w^(j L / 2h) from stw.
template <int P, bool INV>
__device__ __forceinline__ void fft_regs(float2 (&v)[P], const float2* stw, int L)
{
#pragma unroll
    for (int half = P / 2; half >= 1; half >>= 1) {
        const int step = L / (2 * half);
#pragma unroll
        for (int b = 0; b < P; b += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 a = v[b + j], c = v[b + j + half];
                v[b + j] = cadd(a, c);
                const float2 d = csub(a, c);
                v[b + j + half] = (j == 0) ? d : cmul(d, twid<INV>(stw, j * step));
            }
        }
    }
}

// Step A for one sequence: load x[Q n1 + n2] (n1 < P) through `get`, FFT, apply
// the inter-stage twiddle and store A[k1] = row[k1] (k1 < P).
template <int P, bool INV, class Get>
__device__ __forceinline__ void step_a(Get get, int n2, float2* row, const float2* stw, int Q)
{
    float2 v[P];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) v[n1] = get(Q * n1 + n2);
    const int L = P * Q;
    fft_regs<P, INV>(v, stw, L);
    constexpr int BITS = ilog2(P);
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const int k1 = bitrev(i, BITS);
        row[k1] = (n2 == 0 || k1 == 0) ? v[i] : cmul(v[i], twid<INV>(stw, n2 * k1));
    }
}

// Step C for one (sequence, k1): X[k1 + P k2] = sum_{n2 < Q} A[n2][k1] w_Q^(+- n2 k2)
// for the k2 < Q with k1 + P k2 < lim, handed to `put(k2, value)`.  A is the
// sequence's [Q][P + 1] block.  QT = Q at compile time (registers), or 0 for a
// runtime Q <= 15.
template <int P, int QT, bool INV, class Put>
__device__ __forceinline__ void step_c(const float2* A, int k1, const float2* stw, int Qr, int lim, Put put)
{
    const int Q = QT > 0 ? QT : Qr;
    constexpr int QM = QT > 0 ? QT : 15;
    float2 a[QM];
#pragma unroll
    for (int n2 = 0; n2 < QM; ++n2)
        if (n2 < Q) a[n2] = A[n2 * (P + 1) + k1];
    const int qs = P;  // w_Q = w^(L / Q) = w^P
#pragma unroll
    for (int k2 = 0; k2 < QM; ++k2) {
        if (k2 >= Q) break;
        if (k1 + P * k2 >= lim) break;
        float2 acc = a[0];
#pragma unroll
        for (int n2 = 1; n2 < QM; ++n2) {
            if (n2 >= Q) break;
            const int r = (n2 * k2) % Q;
            acc = cadd(acc, r == 0 ? a[n2] : cmul(a[n2], twid<INV>(stw, r * qs)));
        }
        put(k2, acc);
    }
}

// Analysis of planes [ch][Ly][Lx] -> half spectra [ch][nf].
template <int P, int QT>
__global__ void __launch_bounds__(kFftThreads, kFftMinBlocks)
k_fft_r2c(const float* __restrict__ in, float2* __restrict__ out, const float2* __restrict__ tw, FftDims d,
          int64_t nch)
{
    extern __shared__ __align__(16) unsigned char fft_sm[];
    const int L = d.L, H1 = d.H1, Q = QT > 0 ? QT : d.Q, Lx = d.Lx, Ly = d.Ly, gs = d.gs, npair = d.npair;
    const int nf = H1 * L, nin = Ly * Lx;
    constexpr int QM = QT > 0 ? QT : 15;
    constexpr int KH = P / 2 + 1;  // threads per row pair in the fused step C
    float2* stw = reinterpret_cast<float2*>(fft_sm);  // [L]
    float2* A = stw + L;                                 // [nseq][Q][P + 1]
    float2* G = A + (size_t)d.nseq * Q * (P + 1);        // [Ly][gs] (aliases img)
    float* img = reinterpret_cast<float*>(G);            // [Ly][Lx]
    const int tid = threadIdx.x;
    for (int i = tid; i < L; i += kFftThreads) stw[i] = tw[i];
    int64_t ch = blockIdx.x;
    if (ch < nch)
        for (int i = tid; i < nin; i += kFftThreads) img[i] = in[ch * nin + i];
    float pf[kPfR];
    for (; ch < nch; ch += gridDim.x) {
        __syncthreads();
        // rows: pair (2p, 2p+1) as one complex sequence, zero beyond Lx
        for (int it = tid; it < npair * Q; it += kFftThreads) {
            const int pr = it / Q, n2 = it - pr * Q;
            const float* r0 = img + (2 * pr) * Lx;
            const bool two = 2 * pr + 1 < Ly;
            auto get = [&](int n) -> float2 {
                if (n >= Lx) return make_float2(0.f, 0.f);
                return make_float2(r0[n], two ? r0[Lx + n] : 0.f);
            };
            step_a<P, false>(get, n2, A + ((size_t)pr * Q + n2) * (P + 1), stw, Q);
        }
        __syncthreads();
        // the plane is consumed: fetch the next channel's
        const int64_t nx = ch + gridDim.x;
        const float* nsrc = in + nx * nin;
        if (nx < nch) {
#pragma unroll
            for (int j = 0; j < kPfR; ++j) {
                const int i = tid + j * kFftThreads;
                if (i < nin) pf[j] = nsrc[i];
            }
        }
        // Q-point sums of k1 and P - k1, pair separation in registers:
        // X_a = (Z_f + conj Z_-f) / 2, X_b = (Z_f - conj Z_-f) / 2i
        for (int it = tid; it < npair * KH; it += kFftThreads) {
            const int pr = it / KH, k1 = it - pr * KH, kb = P - k1;
            const bool pairk = k1 != 0 && k1 != P / 2;
            const float2* As = A + (size_t)pr * Q * (P + 1);
            float2 za[QM], zb[QM];
            step_c<P, QT, false>(As, k1, stw, Q, L, [&](int k2, float2 v) { za[k2] = v; });
            if (pairk) step_c<P, QT, false>(As, kb, stw, Q, L, [&](int k2, float2 v) { zb[k2] = v; });
            float2* g0 = G + (size_t)(2 * pr) * gs;
            const bool two = 2 * pr + 1 < Ly;
            auto emit = [&](int f, float2 zf, float2 zm) {
                g0[f] = make_float2(0.5f * (zf.x + zm.x), 0.5f * (zf.y - zm.y));
                if (two) g0[gs + f] = make_float2(0.5f * (zf.y + zm.y), 0.5f * (zm.x - zf.x));
            };
#pragma unroll
            for (int k2 = 0; k2 < QM; ++k2) {
                if (k2 >= Q) break;
                const int f = k1 + P * k2;
                if (f < H1) {
                    const float2 zm = k1 == 0 ? za[(Q - k2) % Q] : (pairk ? zb[Q - 1 - k2] : za[Q - 1 - k2]);
                    emit(f, za[k2], zm);
                }
                const int fb = kb + P * k2;
                if (pairk && fb < H1) emit(fb, zb[k2], za[Q - 1 - k2]);
            }
        }
        __syncthreads();
        // columns f1: complex sequences over v (zero beyond Ly)
        for (int it = tid; it < H1 * Q; it += kFftThreads) {
            const int f1 = it / Q, n2 = it - f1 * Q;
            auto get = [&](int v) -> float2 { return v < Ly ? G[(size_t)v * gs + f1] : make_float2(0.f, 0.f); };
            step_a<P, false>(get, n2, A + ((size_t)f1 * Q + n2) * (P + 1), stw, Q);
        }
        __syncthreads();
        float2* dst = out + ch * (int64_t)nf;
        for (int it = tid; it < H1 * P; it += kFftThreads) {
            const int k1 = it / H1, f1 = it - k1 * H1;
            step_c<P, QT, false>(A + (size_t)f1 * Q * (P + 1), k1, stw, Q, L,
                                 [&](int k2, float2 v) { dst[(k1 + P * k2) * H1 + f1] = v; });
        }
        // the half plane is consumed: stage the next channel's plane
        if (nx < nch) {
#pragma unroll
            for (int j = 0; j < kPfR; ++j) {
                const int i = tid + j * kFftThreads;
                if (i < nin) img[i] = pf[j];
            }
            for (int i = tid + kPfR * kFftThreads; i < nin; i += kFftThreads) img[i] = nsrc[i];
        }
    }
}

// Synthesis of half spectra [ch][nf] -> planes [ch][Ly][Lx] (scaled by 1/L^2);
// lattice positions outside the X x Y frame are written as zero.
template <int P, int QT>
__global__ void __launch_bounds__(kFftThreads, kFftMinBlocks)
k_fft_c2r(const float2* __restrict__ in, float* __restrict__ out, const float2* __restrict__ tw, FftDims d, int N,
          int64_t X, int64_t Y, int64_t nch)
{
    extern __shared__ __align__(16) unsigned char fft_sm[];
    const int L = d.L, H1 = d.H1, Q = QT > 0 ? QT : d.Q, Lx = d.Lx, Ly = d.Ly, gs = d.gs, npair = d.npair;
    const int nf = H1 * L;
    const bool even = (L % 2) == 0;
    float2* stw = reinterpret_cast<float2*>(fft_sm);  // [L]
    float2* A = stw + L;                                 // [nseq][Q][P + 1]
    float2* S = A + (size_t)d.nseq * Q * (P + 1);        // [L][gs]
    float2* Gt = S;                                      // [Ly][gs] (aliases S)
    const int tid = threadIdx.x;
    for (int i = tid; i < L; i += kFftThreads) stw[i] = tw[i];
    int64_t ch = blockIdx.x;
    if (ch < nch)
        for (int i = tid; i < nf; i += kFftThreads) {
            const int f2 = i / H1;
            S[(size_t)f2 * gs + (i - f2 * H1)] = in[ch * nf + i];
        }
    float2 pf[kPfC];
    const float inv = 1.0f / ((float)L * (float)L);
    for (; ch < nch; ch += gridDim.x) {
        __syncthreads();
        // columns f1: inverse over f2
        for (int it = tid; it < H1 * Q; it += kFftThreads) {
            const int f1 = it / Q, n2 = it - f1 * Q;
            auto get = [&](int f2) -> float2 { return S[(size_t)f2 * gs + f1]; };
            step_a<P, true>(get, n2, A + ((size_t)f1 * Q + n2) * (P + 1), stw, Q);
        }
        __syncthreads();
        // the half spectrum is consumed: fetch the next channel's
        const int64_t nx = ch + gridDim.x;
        const float2* nsrc = in + nx * nf;
        if (nx < nch) {
#pragma unroll
            for (int j = 0; j < kPfC; ++j) {
                const int i = tid + j * kFftThreads;
                if (i < nf) pf[j] = nsrc[i];
            }
        }
        // keep t < Ly
        for (int it = tid; it < H1 * P; it += kFftThreads) {
            const int f1 = it / P, k1 = it - f1 * P;
            step_c<P, QT, true>(A + (size_t)f1 * Q * (P + 1), k1, stw, Q, Ly,
                                [&](int k2, float2 v) { Gt[(size_t)(k1 + P * k2) * gs + f1] = v; });
        }
        __syncthreads();
        // rows: Z = S_t + i S_{t+1} over the Hermitian-extended spectrum; the DC
        // and Nyquist terms of a real row are real
        for (int it = tid; it < npair * Q; it += kFftThreads) {
            const int pr = it / Q, n2 = it - pr * Q;
            const float2* g0 = Gt + (size_t)(2 * pr) * gs;
            const bool two = 2 * pr + 1 < Ly;
            auto get = [&](int f) -> float2 {
                float2 a, b;
                if (f < H1) {
                    a = g0[f];
                    b = two ? g0[gs + f] : make_float2(0.f, 0.f);
                    if (f == 0 || (even && f == H1 - 1)) {
                        a.y = 0.f;
                        b.y = 0.f;
                    }
                } else {
                    const int m = L - f;
                    a = make_float2(g0[m].x, -g0[m].y);
                    b = two ? make_float2(g0[gs + m].x, -g0[gs + m].y) : make_float2(0.f, 0.f);
                }
                return make_float2(a.x - b.y, a.y + b.x);  // a + i b
            };
            step_a<P, true>(get, n2, A + ((size_t)pr * Q + n2) * (P + 1), stw, Q);
        }
        __syncthreads();
        const int a_ph = (int)(ch % N), b_ph = (int)((ch / N) % N);
        float* dst = out + ch * (int64_t)Ly * Lx;
        for (int it = tid; it < npair * P; it += kFftThreads) {
            const int pr = it / P, k1 = it - pr * P;
            const int t0 = 2 * pr;
            const bool two = t0 + 1 < Ly;
            const bool y0 = (b_ph + (int64_t)N * t0) < Y, y1 = (b_ph + (int64_t)N * (t0 + 1)) < Y;
            step_c<P, QT, true>(A + (size_t)pr * Q * (P + 1), k1, stw, Q, Lx, [&](int k2, float2 v) {
                const int s = k1 + P * k2;
                const bool xin = (a_ph + (int64_t)N * s) < X;
                dst[t0 * Lx + s] = (xin && y0) ? v.x * inv : 0.f;
                if (two) dst[(t0 + 1) * Lx + s] = (xin && y1) ? v.y * inv : 0.f;
            });
        }
        // the half plane is consumed: stage the next channel's spectrum
        if (nx < nch) {
#pragma unroll
            for (int j = 0; j < kPfC; ++j) {
                const int i = tid + j * kFftThreads;
                if (i < nf) {
                    const int f2 = i / H1;
                    S[(size_t)f2 * gs + (i - f2 * H1)] = pf[j];
                }
            }
            for (int i = tid + kPfC * kFftThreads; i < nf; i += kFftThreads) {
                const int f2 = i / H1;
                S[(size_t)f2 * gs + (i - f2 * H1)] = nsrc[i];
            }
        }
    }
}

FftDims fft_dims(const sid_plan* p, int Q)
{
    FftDims d;
    d.Lx = (int)p->Lx;
    d.Ly = (int)p->Ly;
    d.L = (int)p->L;
    d.H1 = d.L / 2 + 1;
    d.Q = Q;
    d.npair = (d.Ly + 1) / 2;
    d.nseq = std::max(d.npair, d.H1);
    int qinv = 1;  // Q^-1 mod 16 (Q odd)
    while ((qinv * Q) % 16 != 1) ++qinv;
    d.gs = d.H1 + (((qinv - d.H1) % 16) + 16) % 16;
    return d;
}

size_t r2c_bytes(const FftDims& d, int P)
{
    const size_t u = std::max((size_t)d.Ly * d.gs * sizeof(float2), (size_t)d.Ly * d.Lx * sizeof(float));
    return ((size_t)d.L + (size_t)d.nseq * d.Q * (P + 1)) * sizeof(float2) + u;
}
size_t c2r_bytes(const FftDims& d, int P)
{
    return ((size_t)d.L + (size_t)d.nseq * d.Q * (P + 1) + (size_t)d.L * d.gs) * sizeof(float2);
}

// persistent grid: as many CTAs as fit on every SM at once
template <class K> int fft_grid(K kern, size_t smem, int64_t nch)
{
    int nb = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kFftThreads, smem) != cudaSuccess || nb < 1) nb = 1;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 152;
    return (int)std::min<int64_t>(nch, (int64_t)nb * sms);
}

}  // namespace

// L = P * Q with P a power of two in [4, 64] and Q odd, at most 15.
bool fft_factor(int64_t L, int* P, int* Q)
{
    int64_t p = 1;
    while (L % (p * 2) == 0 && p < 64) p *= 2;
    const int64_t q = L / p;
    if (p < 4 || q > 15 || (q % 2) == 0) return false;
    *P = (int)p;
    *Q = (int)q;
    return true;
}

template <int P, int QT>
static int launch_r2c(const float* in, float2* out, const float2* tw, const FftDims& d, int64_t nch, cudaStream_t st)
{
    const size_t sm = r2c_bytes(d, P);
    SID_REQUIRE(sm <= 200 * 1024, "spectral projector: lenslet grid too large for the FFT kernels");
    SID_TRY(smem_attr((const void*)k_fft_r2c<P, QT>, sm));
    k_fft_r2c<P, QT><<<fft_grid(k_fft_r2c<P, QT>, sm, nch), kFftThreads, sm, st>>>(in, out, tw, d, nch);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

template <int P, int QT>
static int launch_c2r(const float2* in, float* out, const float2* tw, const FftDims& d, int N, int64_t X, int64_t Y,
                      int64_t nch, cudaStream_t st)
{
    const size_t sm = c2r_bytes(d, P);
    SID_REQUIRE(sm <= 200 * 1024, "spectral projector: lenslet grid too large for the FFT kernels");
    SID_TRY(smem_attr((const void*)k_fft_c2r<P, QT>, sm));
    k_fft_c2r<P, QT><<<fft_grid(k_fft_c2r<P, QT>, sm, nch), kFftThreads, sm, st>>>(in, out, tw, d, N, X, Y, nch);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// (P, Q) dispatch: Q = 3 and 5 at compile time, other odd Q at run time
template <int P>
static int r2c_q(const float* in, float2* out, const float2* tw, const FftDims& d, int64_t nch, cudaStream_t st)
{
    if (d.Q == 5) return launch_r2c<P, 5>(in, out, tw, d, nch, st);
    if (d.Q == 3) return launch_r2c<P, 3>(in, out, tw, d, nch, st);
    return launch_r2c<P, 0>(in, out, tw, d, nch, st);
}

template <int P>
static int c2r_q(const float2* in, float* out, const float2* tw, const FftDims& d, int N, int64_t X, int64_t Y,
                 int64_t nch, cudaStream_t st)
{
    if (d.Q == 5) return launch_c2r<P, 5>(in, out, tw, d, N, X, Y, nch, st);
    if (d.Q == 3) return launch_c2r<P, 3>(in, out, tw, d, N, X, Y, nch, st);
    return launch_c2r<P, 0>(in, out, tw, d, N, X, Y, nch, st);
}

int fft_r2c(const sid_plan* p, const float* in, float2* out, int64_t nch, cudaStream_t st)
{
    int P = 0, Q = 0;
    SID_REQUIRE(fft_factor(p->L, &P, &Q), "fft_r2c: L = %lld does not factor as 2^a * odd (<= 15)", (long long)p->L);
    SID_REQUIRE(p->Lx <= p->L && p->Ly <= p->L, "fft_r2c: plane larger than the DFT length");
    const float2* tw = p->twiddle.as<float2>();
    const FftDims d = fft_dims(p, Q);
    switch (P) {
    case 4: return r2c_q<4>(in, out, tw, d, nch, st);
    case 8: return r2c_q<8>(in, out, tw, d, nch, st);
    case 16: return r2c_q<16>(in, out, tw, d, nch, st);
    case 32: return r2c_q<32>(in, out, tw, d, nch, st);
    default: return r2c_q<64>(in, out, tw, d, nch, st);
    }
}

int fft_c2r(const sid_plan* p, const float2* in, float* out, int64_t nch, cudaStream_t st)
{
    int P = 0, Q = 0;
    SID_REQUIRE(fft_factor(p->L, &P, &Q), "fft_c2r: L = %lld does not factor as 2^a * odd (<= 15)", (long long)p->L);
    SID_REQUIRE(p->Lx <= p->L && p->Ly <= p->L, "fft_c2r: plane larger than the DFT length");
    const float2* tw = p->twiddle.as<float2>();
    const FftDims d = fft_dims(p, Q);
    const int N = (int)p->N;
    switch (P) {
    case 4: return c2r_q<4>(in, out, tw, d, N, p->X, p->Y, nch, st);
    case 8: return c2r_q<8>(in, out, tw, d, N, p->X, p->Y, nch, st);
    case 16: return c2r_q<16>(in, out, tw, d, N, p->X, p->Y, nch, st);
    case 32: return c2r_q<32>(in, out, tw, d, N, p->X, p->Y, nch, st);
    default: return c2r_q<64>(in, out, tw, d, N, p->X, p->Y, nch, st);
    }
}

}  // namespace sid
