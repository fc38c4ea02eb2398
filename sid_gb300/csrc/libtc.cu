// libtc.cu -- library generation (generate_LFM_library_GPU.m:63-109) through
// the tensor-core spectral projector on per-neuron lenslet windows.
//
// A neuron's boxed volume covers at most `span` lattice points per axis and
// phase (3 for a 25-pixel box at Nnum 15), so its forward projection lives on
// Wo = span + D - 1 output lenslets per axis around the box.  In window
// coordinates (origin at the first output lenslet, umin + dlo) the box sits at
// lattice positions [-dlo, -dlo + span) and the output at [0, Wo); on a lenslet
// grid of L >= Wo points the circular convolution with the tap arrays never
// wraps, so one set of tap spectra on that small grid (nf = (L/2+1) L
// frequencies, 420 for L = 28 instead of 3280 for the 1005-pixel frame) serves
// every neuron:
//   Ihat_n[b'a'](f) = sum_abc Kw[f][b'a'][abc] Vhat_n[abc](f)
// which for up to 64 neurons at once is the batched tensor-core contraction of
// spec_tc.cu.  Per pass (neurons sorted by depth window, so a pass reduces only
// over the input channels of its depths):
//   1. k_lib_pack: each box channel's spectrum, a direct DFT of its <= span^2
//      lattice points, written straight into the contraction's B operand
//      (three BF16 parts, columns (Vr, -Vi) and (Vi, Vr) per neuron);
//   2. k_spec_tc over the window spectra (24-bit planes), the pass's K range;
//   3. k_lib_synth: per neuron and output phase, the inverse real DFT of the
//      window spectrum straight from the contraction's output, written into
//      the library row (pixels outside the frame dropped; the rest of each row
//      is zero), on a second stream beside the next pass's pack.
// Precision: 24-bit window spectra, box spectra split into two BF16 parts
// (16-17 bits), three MMA passes with FP32 accumulation -- about 1e-5 relative
// per row, against FP32 rounding for the tap kernels of library.cu.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda_bf16.h>

#include "library.cuh"

namespace sid {

bool fft_factor(int64_t L, int* P, int* Q);
int build_khat_f24(const sid_plan* p, int64_t L, const float2* tw, ushort2* h, uchar2* l);

struct LibWin {
    int64_t Wo = 0;      // window lenslets per axis
    int64_t L = 0, nf = 0;  // window grid length, frequencies (L/2+1) L
    DBuf tw;             // L float2: exp(2 pi i k / L)
    DBuf kh, kl;         // window tap spectra, 24-bit planes [f][b'a'][abc]
    DBuf bpl;            // B operand planes of one pass
    DBuf tco, cols;      // contraction outputs [2][f][neuron][b'a'] (alternate passes), neurons in pass order
    // the synthesis of pass k runs on `side` beside the pack of pass k + 1
    cudaStream_t side = nullptr;
    cudaEvent_t tc_done[2] = {nullptr, nullptr}, syn_done[2] = {nullptr, nullptr};
};

namespace {

constexpr int kLibPackThreads = 128;
constexpr int kLibMaxL = 64;  // window grid lengths handled by the pack and synthesis kernels
constexpr int kLibSynthWarps = 4;  // output phases per synthesis CTA
// B planes of the library contraction: two (hi, lo) and three MMA passes.  The
// window spectra carry 16 significant bits; B to 16-17 bits and the dropped
// A_lo B_lo product (below 2^-16 of each term) keep the rows within ~1e-5.
constexpr int kLibBPlanes = 2;

// x = hi + lo to 16-17 significant bits (hi: x rounded to BF16; lo: the remainder rounded)
__device__ __forceinline__ void split2(float x0, float x1, uint32_t& h, uint32_t& l)
{
    const __nv_bfloat162 hi = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(hi);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    h = *reinterpret_cast<const uint32_t*>(&hi);
    l = *reinterpret_cast<const uint32_t*>(&lo);
}

__device__ __forceinline__ void split3(float x0, float x1, uint32_t& h, uint32_t& m, uint32_t& l)
{
    // x = hi + mid + lo, each remainder exact in FP32 (24 significant bits in all)
    const __nv_bfloat162 hi = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(hi);
    const float r0 = x0 - hf.x, r1 = x1 - hf.y;
    const __nv_bfloat162 mi = __floats2bfloat162_rn(r0, r1);
    const float2 mf = __bfloat1622float2(mi);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
    h = *reinterpret_cast<const uint32_t*>(&hi);
    m = *reinterpret_cast<const uint32_t*>(&mi);
    l = *reinterpret_cast<const uint32_t*>(&lo);
}

// B planes [f][BN][kpb] for one pass: thread (channel cbase + cc, neuron slot j)
// evaluates the channel's spectrum at the H1 frequencies f1 of row f2 =
// blockIdx.y, separably over the box's lattice points (pu, pv: window
// coordinates mod L):
//   R(u) = sum_v V(u, v) exp(-2 pi i f2 pv / L),  Vhat(f1) = sum_u R(u) exp(-2 pi i f1 pu / L)
// and writes the two columns of slot j (zeros for empty slots and channels)
// as NBP BF16 planes (bmi unused for two).  MU bounds the lattice points per
// axis and phase.
template <int MU, int NBP>
__global__ void __launch_bounds__(kLibPackThreads)
k_lib_pack(const float* __restrict__ packed, const LibBox* __restrict__ boxes, const int* __restrict__ cols, int nb,
           int cbase, int nchb, int n_in, int N, int dlo, int L, int BN, const float2* __restrict__ tw,
           uint32_t* __restrict__ bhi, uint32_t* __restrict__ bmi, uint32_t* __restrict__ blo)
{
    __shared__ float2 stw[kLibMaxL];
    for (int i = threadIdx.x; i < L; i += blockDim.x) stw[i] = tw[i];
    __syncthreads();
    const int cc = blockIdx.x * blockDim.x + threadIdx.x;
    if (cc >= nchb) return;
    const int j = blockIdx.z, f2 = blockIdx.y, H1 = L / 2 + 1;
    const int c = cbase + cc;
    // empty slots and channels keep zero rows at phase 0
    float2 R[MU];
    int ph[MU], du[MU];
#pragma unroll
    for (int q = 0; q < MU; ++q) {
        R[q] = make_float2(0.f, 0.f);
        ph[q] = 0;
        du[q] = 0;
    }
    if (j < nb && c < n_in) {
        const LibBox b = boxes[cols[j]];
        const int a = c % N, bb = (c / N) % N, z = c / (N * N);
        if (z >= b.z0 && z < b.z1) {
            const int bw = b.x1 - b.x0, bh = b.y1 - b.y0;
            const int w0x = b.x0 / N + dlo, w0y = b.y0 / N + dlo;  // window origin (lattice)
            // lattice points of phase (a, bb) inside the box: x = a + N u in [x0, x1)
            const int ulo = (b.x0 - a + N - 1 + N) / N - 1, uhi = (b.x1 - 1 - a + N) / N - 1;
            const int vlo = (b.y0 - bb + N - 1 + N) / N - 1, vhi = (b.y1 - 1 - bb + N) / N - 1;
            const float* src = packed + b.off + (int64_t)bw * bh * (z - b.z0);
#pragma unroll
            for (int iv = 0; iv < MU; ++iv) {
                const int v = vlo + iv;
                if (v > vhi) break;
                const int pv = ((v - w0y) % L + L) % L;
                const float2 w = stw[(int)(((int64_t)f2 * pv) % L)];
#pragma unroll
                for (int iu = 0; iu < MU; ++iu) {
                    const int u = ulo + iu;
                    if (u <= uhi) {
                        const float val = src[(a + N * u - b.x0) + bw * (bb + N * v - b.y0)];
                        R[iu].x = fmaf(val, w.x, R[iu].x);  // val exp(-i theta)
                        R[iu].y = fmaf(-val, w.y, R[iu].y);
                    }
                }
            }
#pragma unroll
            for (int iu = 0; iu < MU; ++iu) du[iu] = ((ulo + iu - w0x) % L + L) % L;
        }
    }
    const int64_t kw = nchb;  // 32-bit words (complex parts as a BF16 pair) per B row
    for (int f1 = 0; f1 < H1; ++f1) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int q = 0; q < MU; ++q) {
            // R exp(-i theta) = (Rx cos + Ry sin) + i (Ry cos - Rx sin)
            const float2 w = stw[ph[q]];
            re = fmaf(R[q].x, w.x, fmaf(R[q].y, w.y, re));
            im = fmaf(R[q].y, w.x, fmaf(-R[q].x, w.y, im));
            const int nx = ph[q] + du[q];
            ph[q] = nx >= L ? nx - L : nx;
        }
        const int64_t f = (int64_t)f2 * H1 + f1;
        uint32_t h, m, l;
        // column 2j: (Vr, -Vi); column 2j + 1: (Vi, Vr)
        const int64_t o0 = (f * BN + 2 * j) * kw + cc, o1 = o0 + kw;
        if (NBP == 3) {
            split3(re, -im, h, m, l);
            bhi[o0] = h; bmi[o0] = m; blo[o0] = l;
            split3(im, re, h, m, l);
            bhi[o1] = h; bmi[o1] = m; blo[o1] = l;
        } else {
            split2(re, -im, h, l);
            bhi[o0] = h; blo[o0] = l;
            split2(im, re, h, l);
            bhi[o1] = h; blo[o1] = l;
        }
    }
}

// Inverse real DFT of the window spectra, one warp per (neuron slot j =
// blockIdx.y, output phase o = kLibSynthWarps blockIdx.x + warp), from the
// contraction output S = tco[f][j][o] (f = f1 + H1 f2) into the library row of
// the slot's neuron:
//   G(f1, t)   = sum_f2 S(f1, f2) w^(t f2)                            t < Wo
//   img(t, s)  = 1/L^2 sum_f1 c(f1) Re(G(f1, t) w^(s f1))            s < Wo
// with w = exp(2 pi i / L), c = 1 at f1 = 0 and at L/2 (even L), else 2;
// window lenslet (s, t) is pixel (a' + N (w0x + s), b' + N (w0y + t)).  The
// CTA's warps take consecutive output phases, so the spectra arrive in
// 32-byte pieces; shared memory: twiddles, then per warp S [H1][L], G [H1][Wo].
__global__ void __launch_bounds__(kLibSynthWarps * 32)
k_lib_synth(const float2* __restrict__ tco, const LibBox* __restrict__ boxes, const int* __restrict__ cols, int nb,
            int rows, int N, int L, int Wo, int dlo, int64_t X, int64_t Y, const float2* __restrict__ tw,
            float* __restrict__ out, int64_t ldn, int64_t ldp)
{
    extern __shared__ float2 syn_sm[];
    const int H1 = L / 2 + 1, nf = H1 * L, per = H1 * L + H1 * Wo;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = blockIdx.y, o0 = blockIdx.x * kLibSynthWarps;
    float2* stw = syn_sm;
    for (int i = threadIdx.x; i < L; i += blockDim.x) stw[i] = tw[i];
    for (int i = threadIdx.x; i < nf * kLibSynthWarps; i += blockDim.x) {
        const int f = i / kLibSynthWarps, q = i - f * kLibSynthWarps;
        if (o0 + q < rows) {
            const int f2 = f / H1;
            syn_sm[L + q * per + (f - f2 * H1) * L + f2] = tco[((int64_t)f * nb + j) * rows + o0 + q];
        }
    }
    __syncthreads();
    const int o = o0 + warp;
    if (o >= rows) return;
    const float2* S = syn_sm + L + warp * per;
    float2* G = syn_sm + L + warp * per + H1 * L;
    for (int i = lane; i < H1 * Wo; i += 32) {
        const int f1 = i / Wo, t = i - f1 * Wo;
        float gr = 0.f, gi = 0.f;
        int ph = 0;
        for (int f2 = 0; f2 < L; ++f2) {
            const float2 sv = S[f1 * L + f2], w = stw[ph];
            gr = fmaf(sv.x, w.x, fmaf(-sv.y, w.y, gr));
            gi = fmaf(sv.x, w.y, fmaf(sv.y, w.x, gi));
            ph += t;
            ph = ph >= L ? ph - L : ph;
        }
        G[f1 * Wo + t] = make_float2(gr, gi);
    }
    __syncwarp();
    const int n = cols[j];
    const LibBox b = boxes[n];
    const int64_t x0 = (o % N) + (int64_t)N * (b.x0 / N + dlo), y0 = (o / N) + (int64_t)N * (b.y0 / N + dlo);
    const float inv = 1.0f / ((float)L * (float)L);
    for (int i = lane; i < Wo * Wo; i += 32) {
        const int t = i / Wo, s = i - t * Wo;
        const int64_t x = x0 + (int64_t)N * s, y = y0 + (int64_t)N * t;
        if (x < 0 || x >= X || y < 0 || y >= Y) continue;
        float acc = 0.f;
        int ph = 0;
        for (int f1 = 0; f1 < H1; ++f1) {
            const float2 g = G[f1 * Wo + t], w = stw[ph];
            const float cf = (f1 == 0 || 2 * f1 == L) ? 1.f : 2.f;
            acc = fmaf(cf, fmaf(g.x, w.x, -g.y * w.y), acc);
            ph += s;
            ph = ph >= L ? ph - L : ph;
        }
        out[(int64_t)n * ldn + (x + X * y) * ldp] = acc * inv;
    }
}

}  // namespace

int64_t libwin_bytes(const sid_plan* p)
{
    if (!p->libwin) return 0;
    const LibWin* w = p->libwin;
    int64_t b = 0;
    for (const DBuf* d : {&w->tw, &w->kh, &w->kl, &w->bpl, &w->tco, &w->cols}) b += (int64_t)d->bytes;
    return b;
}

void libwin_release_workspaces(sid_plan* p)
{
    if (!p->libwin) return;
    LibWin* w = p->libwin;
    for (DBuf* b : {&w->bpl, &w->tco, &w->cols}) b->release();
}

void libwin_free(sid_plan* p)
{
    if (!p->libwin) return;
    libwin_release_workspaces(p);
    LibWin* w = p->libwin;
    w->kh.release();
    w->kl.release();
    w->tw.release();
    if (w->side) cudaStreamDestroy(w->side);
    for (int b = 0; b < 2; ++b) {
        if (w->tc_done[b]) cudaEventDestroy(w->tc_done[b]);
        if (w->syn_done[b]) cudaEventDestroy(w->syn_done[b]);
    }
    delete w;
    p->libwin = nullptr;
}

// Window spectra for windows of at least Wo lenslets (kept on the plan; a
// larger window serves smaller boxes too).
static int libwin_ensure(sid_plan* p, int64_t Wo)
{
    if (p->libwin && p->libwin->Wo >= Wo) return SID_OK;
    libwin_free(p);
    int64_t L = Wo;
    int P = 0, Q = 0;
    while (!fft_factor(L, &P, &Q)) ++L;
    SID_REQUIRE(L <= kLibMaxL, "sid_library_spectral: window of %lld lenslets exceeds the window grid limit",
                (long long)Wo);
    LibWin* w = new LibWin();
    p->libwin = w;
    w->Wo = Wo;
    w->L = L;
    w->nf = (L / 2 + 1) * L;
    std::vector<float2> tw((size_t)L);
    for (int64_t k = 0; k < L; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)L;
        tw[(size_t)k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    SID_TRY(w->tw.alloc((size_t)L * sizeof(float2)));
    SID_CUDA_TRY(cudaMemcpy(w->tw.p, tw.data(), (size_t)L * sizeof(float2), cudaMemcpyHostToDevice));
    const int64_t n_out = p->N * p->N, n_in_pad = cdiv(p->N * p->N * p->Z, 8) * 8;
    const size_t nent = (size_t)(w->nf * n_out * n_in_pad);
    SID_TRY(w->kh.alloc(nent * sizeof(ushort2)));
    SID_TRY(w->kl.alloc(nent * sizeof(uchar2)));
    SID_CUDA_TRY(cudaStreamCreateWithFlags(&w->side, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        SID_CUDA_TRY(cudaEventCreateWithFlags(&w->tc_done[b], cudaEventDisableTiming));
        SID_CUDA_TRY(cudaEventCreateWithFlags(&w->syn_done[b], cudaEventDisableTiming));
    }
    return build_khat_f24(p, L, w->tw.as<float2>(), w->kh.as<ushort2>(), w->kl.as<uchar2>());
}

template <int MU>
static int launch_pack(dim3 grid, const float* packed, const LibBox* boxes, const int* cols, int nb, int cbase,
                       int nchb, int n_in, int N, int dlo, int L, int BN, const float2* tw, uint32_t* h, uint32_t* m,
                       uint32_t* l, cudaStream_t st)
{
    k_lib_pack<MU, kLibBPlanes><<<grid, kLibPackThreads, 0, st>>>(packed, boxes, cols, nb, cbase, nchb, n_in, N, dlo,
                                                                   L, BN, tw, h, m, l);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Forward projections of the staged boxes (lib_stage: boxes in p->ws[3] and
// `boxes`, packed values in p->ws[2]) into the library rows, on the tensor
// cores; leaves `st` to be synchronised by the caller.
int lib_run_spectral(sid_plan* p, const char* who, const std::vector<LibBox>& boxes, float* out, int out_layout,
                     cudaStream_t st)
{
    SID_REQUIRE(!p->adj_separate, "%s: the spectral form needs odd PSF crop widths", who);
    const int64_t n_neur = (int64_t)boxes.size();
    if (n_neur == 0) return SID_OK;
    const int64_t N = p->N, D = p->g.D, n_out = N * N, n_in = N * N * p->Z, n_in_pad = cdiv(n_in, 8) * 8;
    int span = 1, mu = 1;
    for (const LibBox& b : boxes) {
        span = std::max(span, std::max((b.x1 - 1) / (int)N - b.x0 / (int)N, (b.y1 - 1) / (int)N - b.y0 / (int)N) + 1);
        mu = std::max(mu, (int)std::max(cdiv(b.x1 - b.x0, N), cdiv(b.y1 - b.y0, N)));
    }
    SID_REQUIRE(mu <= 6, "%s: boxes of more than 6 lattice points per phase (use the FP32 tap form)", who);
    SID_TRY(libwin_ensure(p, span + D - 1));
    LibWin* w = p->libwin;
    const int64_t L = w->L, nf = w->nf, Wo = w->Wo;
    // passes: up to 64 neurons in depth-window order
    std::vector<int> order((size_t)n_neur);
    for (int64_t n = 0; n < n_neur; ++n) order[(size_t)n] = (int)n;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return boxes[x].z0 != boxes[y].z0 ? boxes[x].z0 < boxes[y].z0 : boxes[x].z1 < boxes[y].z1;
    });
    const int G = spectral_tc_max_volumes();
    struct Pass { int first, nb, akb0, nkb; };
    std::vector<Pass> passes;
    int64_t max_kpb = 0;
    for (int i = 0; i < (int)n_neur; i += G) {
        Pass ps;
        ps.first = i;
        ps.nb = (int)std::min<int64_t>(G, n_neur - i);
        int zlo = INT32_MAX, zhi = 0;
        for (int k = i; k < i + ps.nb; ++k) {
            zlo = std::min(zlo, boxes[order[k]].z0);
            zhi = std::max(zhi, boxes[order[k]].z1);
        }
        // K elements (complex parts interleaved) of the depths [zlo, zhi), in 64-element blocks
        ps.akb0 = (int)((2 * n_out * zlo) / 64);
        ps.nkb = (int)(cdiv(2 * n_out * zhi, 64) - ps.akb0);
        max_kpb = std::max<int64_t>(max_kpb, 64 * ps.nkb);
        passes.push_back(ps);
    }
    const int64_t bn_max = n_neur > 32 ? 128 : 64;
    SID_TRY(w->bpl.alloc((size_t)(kLibBPlanes * nf * bn_max * max_kpb) * sizeof(uint16_t)));
    const int gmax = (int)std::min<int64_t>(n_neur, G);
    const size_t tco_elems = (size_t)(nf * gmax * n_out);
    SID_TRY(w->tco.alloc(2 * tco_elems * sizeof(float2)));
    SID_TRY(w->cols.alloc((size_t)n_neur * sizeof(int)));
    SID_CUDA_TRY(cudaMemcpyAsync(w->cols.p, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const int64_t P = p->X * p->Y;
    SID_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)(P * n_neur) * sizeof(float), st));
    const int64_t ldn = out_layout == 0 ? 1 : P, ldp = out_layout == 0 ? n_neur : 1;
    const LibBox* dbox = p->ws[3].as<LibBox>();
    const float* dpack = p->ws[2].as<float>();
    const int64_t H1 = L / 2 + 1;
    const size_t synth_smem = (size_t)(L + kLibSynthWarps * (H1 * L + H1 * Wo)) * sizeof(float2);
    SID_CUDA_TRY(cudaFuncSetAttribute(k_lib_synth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)synth_smem));
    for (size_t k = 0; k < passes.size(); ++k) {
        const Pass& ps = passes[k];
        const int bn = ps.nb <= 32 ? 64 : 128;
        const int buf = (int)(k & 1);
        float2* tco = w->tco.as<float2>() + buf * tco_elems;
        const int64_t kpb = 64 * (int64_t)ps.nkb, nchb = kpb / 2;
        const size_t plane = (size_t)(nf * bn * kpb);
        uint16_t* bh = w->bpl.as<uint16_t>();
        const int* cols = w->cols.as<int>() + ps.first;
        dim3 grid((unsigned)cdiv(nchb, kLibPackThreads), (unsigned)L, (unsigned)(bn / 2));
        uint32_t* h32 = reinterpret_cast<uint32_t*>(bh);
        uint32_t* m32 = reinterpret_cast<uint32_t*>(bh + plane);
        uint32_t* l32 = reinterpret_cast<uint32_t*>(bh + (kLibBPlanes - 1) * plane);
        const int cbase = 32 * ps.akb0;
        if (mu <= 3)
            SID_TRY(launch_pack<3>(grid, dpack, dbox, cols, ps.nb, cbase, (int)nchb, (int)n_in, (int)N, (int)p->g.dlo,
                                   (int)L, bn, w->tw.as<float2>(), h32, m32, l32, st));
        else
            SID_TRY(launch_pack<6>(grid, dpack, dbox, cols, ps.nb, cbase, (int)nchb, (int)n_in, (int)N, (int)p->g.dlo,
                                   (int)L, bn, w->tw.as<float2>(), h32, m32, l32, st));
        // the contraction output buffer is free once the synthesis two passes back has read it
        if (k >= 2) SID_CUDA_TRY(cudaStreamWaitEvent(st, w->syn_done[buf], 0));
        SID_TRY(spec_tc_forward_raw(w->kh.p, w->kl.p, n_out, 2 * n_in_pad, ps.akb0, bh, kLibBPlanes, kpb, nf, ps.nb,
                                    tco, p->errflag.as<int>(), st));
        SID_CUDA_TRY(cudaEventRecord(w->tc_done[buf], st));
        SID_CUDA_TRY(cudaStreamWaitEvent(w->side, w->tc_done[buf], 0));
        k_lib_synth<<<dim3((unsigned)cdiv(n_out, kLibSynthWarps), (unsigned)ps.nb), kLibSynthWarps * 32, synth_smem,
                      w->side>>>(tco, dbox, cols, ps.nb, (int)n_out, (int)N, (int)L, (int)Wo, (int)p->g.dlo, p->X, p->Y,
                                 w->tw.as<float2>(), out, ldn, ldp);
        SID_CHECK_LAUNCH();
        SID_CUDA_TRY(cudaEventRecord(w->syn_done[buf], w->side));
    }
    // join the synthesis stream (in order: its last event covers every pass)
    SID_CUDA_TRY(cudaStreamWaitEvent(st, w->syn_done[(passes.size() - 1) & 1], 0));
    return SID_OK;
}

}  // namespace sid

using namespace sid;

extern "C" int sid_library_spectral(sid_plan* p, const float* const* recon, int64_t n_comp, const double* centers,
                                    const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial,
                                    float* out, int out_layout, void* stream)
{
    SID_REQUIRE(p && recon && centers && neur_id && out, "sid_library_spectral: NULL argument");
    SID_REQUIRE(n_comp >= 1 && n_neur >= 1 && neur_rad >= 0 && axial > 0,
                "sid_library_spectral: need n_comp >= 1, n_neur >= 1, neur_rad >= 0, axial > 0");
    SID_REQUIRE(out_layout == 0 || out_layout == 1,
                "sid_library_spectral: out_layout must be 0 (n x P) or 1 (P x n)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<LibBox> boxes;
    SID_TRY(lib_stage(p, "sid_library_spectral", recon, n_comp, centers, neur_id, n_neur, neur_rad, axial, boxes,
                      st));
    SID_TRY(lib_run_spectral(p, "sid_library_spectral", boxes, out, out_layout, st));
    // the staging buffers are read by the kernels above until they finish
    return plan_sync(p, st);
}
