// sid_internal.cuh -- shared definitions of the libsid CUDA library.
//
// Geometry (MATLAB column-major, 0-based here):
//   H(i,j,a,b,c)  PSF, M x M x N x N x Z  (i,j sensor offsets, (a,b) lenslet phase, c depth)
//   V(x,y,c)      volume, X x Y x Z;  I(x,y) sensor image, X x Y.
// Lenslet (polyphase) decomposition used by every projector kernel:
//   x = a + N*u  (a = phase in [0,N), u = lenslet index in [0,Lx), Lx = ceil(X/N))
//   Vp[c][b][a][v][u] = V(a+N*u, b+N*v, c)      (zero where x >= X or y >= Y)
//   Ip[b'][a'][t][s]  = I(a'+N*s, b'+N*t)
// Forward projection (forwardProjectACC.m:14-29, conv2 'same' alignment):
//   Ip[b'a'](s,t) = sum_{abc} sum_{m1,m2} Vp[abc](s-m1-dlo, t-m2-dlo) * K[abc][b'a'](m1,m2)
//   K[abc][b'a'](m1,m2) = H(a'-a+cf_c+lo_c+N*(m1+dlo), b'-b+cf_c+lo_c+N*(m2+dlo), a, b, c)
// and the adjoint (backwardProjectACC_new.m:14-26) uses the same taps with cf
// replaced by cb = Mc-1-floor(Mc/2) (equal for odd Mc).
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/sid.h"

namespace sid {

void set_error(const char* fmt, ...);

#define SID_CUDA_TRY(expr)                                                      \
    do {                                                                        \
        cudaError_t _e = (expr);                                                \
        if (_e != cudaSuccess) {                                                \
            ::sid::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,         \
                             cudaGetErrorString(_e));                           \
            return (_e == cudaErrorMemoryAllocation) ? SID_ENOMEM : SID_ECUDA;  \
        }                                                                       \
    } while (0)

#define SID_CHECK_LAUNCH() SID_CUDA_TRY(cudaGetLastError())

#define SID_REQUIRE(cond, ...)                                                  \
    do {                                                                        \
        if (!(cond)) {                                                          \
            ::sid::set_error(__VA_ARGS__);                                      \
            return SID_EINVAL;                                                  \
        }                                                                       \
    } while (0)

#define SID_TRY(expr)                                                           \
    do {                                                                        \
        int _s = (expr);                                                        \
        if (_s != SID_OK) return _s;                                            \
    } while (0)

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// looked up once per device ordinal; 152 on GB300).
int sm_count();
// cudaFuncSetAttribute(func, MaxDynamicSharedMemorySize, bytes) for the launch
// that follows.  Set on every launch, not once per process: the setting
// belongs to the current context and device (a device reset, as MATLAB's
// reset(gpuDevice) does, or a second device starts from the default), and the
// size can grow with the plan (the direct kernels' tap tiles with Nnum).
int smem_attr(const void* func, size_t bytes);
// The power of two that brings a largest magnitude amax into [2^13, 2^14)
// (1 for a zero or non-finite amax): the scale of an FP16 hi/lo split.
__device__ __forceinline__ float pow2_for(float amax)
{
    if (!(amax > 0.f) || !isfinite(amax)) return 1.f;
    int ex;
    frexpf(amax, &ex);  // amax in [2^(ex-1), 2^ex)
    return ldexpf(1.f, max(-126, min(126, 14 - ex)));
}

// Device-resident operand scales (gemm_simt.cu): pow2_scale_dev writes
// pow2_for(max |x|) to dscale[0]; scale_ratio_dev writes num / (a[0] b[0]).
int pow2_scale_dev(const float* x, int64_t n, unsigned int* amax, float* dscale, cudaStream_t st);
int scale_ratio_dev(const float* a, const float* b, float num, float* out, cudaStream_t st);
int split16_ds(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
               float scale, const float* dscale, cudaStream_t st);
int split16_t_ds(const float* src, int64_t rows, int64_t k, int64_t ldr, uint16_t* hi, uint16_t* lo, bool bf16,
                 float scale, const float* dscale, cudaStream_t st);
// tensor-core GEMM (gemm_tc.cu) whose alpha is multiplied by dalpha[0] (device memory) when dalpha is given
int gemm_tn_ds(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
               float* C, int64_t ldc, float alpha, const float* dalpha, float beta, int bn, int splitk, float* ws,
               int64_t ws_elems, int* err, cudaStream_t st);
inline int64_t floordiv(int64_t a, int64_t b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }
inline int64_t ceildiv_signed(int64_t a, int64_t b) { return -floordiv(-a, b); }

// Device buffer owned by a plan.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int alloc(size_t n) {
        if (bytes >= n && p) return SID_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) return SID_OK;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc(%zu bytes) failed: %s", n, cudaGetErrorString(e));
            return SID_ENOMEM;
        }
        bytes = n;
        return SID_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// CUDA-event timing of the dominant kernel launches of a plan (opt-in).
struct KTimer {
    bool on = false;
    std::vector<cudaEvent_t> beg, end;
    size_t used = 0;
    void begin(cudaStream_t st) {
        if (!on) return;
        if (used == beg.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            beg.push_back(a);
            end.push_back(b);
        }
        cudaEventRecord(beg[used], st);
    }
    void finish(cudaStream_t st) {
        if (!on) return;
        cudaEventRecord(end[used], st);
        ++used;
    }
    void release() {
        for (auto e : beg) cudaEventDestroy(e);
        for (auto e : end) cudaEventDestroy(e);
        beg.clear();
        end.clear();
        used = 0;
    }
};

// A pixel-major P x k factor in the K-blocked 16-bit layout of the tensor-core
// GEMM (nmf.cu pix_operand / gemm_pix): hi (and lo for a split FP32 factor).
struct PixOperand {
    const void* hi;
    const void* lo;
    bool f16;             // FP16 operands (else BF16)
    const float* dscale;  // X was multiplied by the power of two dscale[0] (device memory; null: 1)
};

constexpr int kScaleWords = 16;

// Lenslet-tap geometry shared by the direct and spectral projectors.
struct TapGeom {
    int64_t N, Z, X, Y, Lx, Ly;
    int64_t dlo, dhi, D;  // tap range along each axis (lenslet units)
};

}  // namespace sid

namespace sid {
struct LibWin;  // library windows (libtc.cu)
}

// The opaque plan (declared in sid.h as struct sid_plan).
struct sid_plan {
    int64_t M, N, Z, X, Y, Lx, Ly;
    int flags;
    int device;
    bool adj_separate;          // adjoint taps differ from forward taps (even crop width)
    sid::TapGeom g;
    sid::DBuf taps_f;           // [c][b][a][b'][a'][m1][m2] float, forward taps
    sid::DBuf taps_b;           // same layout, adjoint taps (only if adj_separate)
    // spectral form
    int64_t L;                  // lenslet-grid DFT length (>= Lx + max(dhi,-dlo))
    int64_t nf;                 // number of r2c frequencies = (L/2+1) * L
    bool spec_f32, spec_i16;
    sid::DBuf khat_f32;         // [f][b'a'][abc] float2
    sid::DBuf khat_i16;         // [f][b'a'][abc] short2 mantissas
    sid::DBuf rstep;            // [f][b'a'] step (rowmax/32767) of each 16-bit row
    sid::DBuf khat_f24h;        // [f][b'a'][abc] 24-bit floats: high 16 bits of re, im
    sid::DBuf khat_f24l;        // [f][b'a'][abc] 24-bit floats: low 8 bits of re, im
    bool spec_f24;
    sid::DBuf khat_f24th;       // [f][abc][b'a' padded to 8] the 24-bit planes transposed (tensor-core adjoint)
    sid::DBuf khat_f24tl;
    bool spec_tc = false;
    sid::DBuf tcb, tco;         // tensor-core projections: B operand planes, contraction output
    sid::DBuf twiddle;          // L float2: exp(+2 pi i k / L)
    sid::DBuf weak;             // runs (column runs, then row runs) of the weakly observed voxels
    sid::DBuf weak_pad;         //   (recomputed exactly after each spectral back projection) and the
    int64_t nweak = 0;          //   zero-padded sensor-lattice copies their kernel reads
    sid::DBuf weak_part;        //   (partial sums when the tap arrays are split over several CTAs)
    std::vector<int> weak_cz, weak_rz;  // column / row runs of depths [0, z) (Z + 1 entries each)
    int64_t nweak_cols = 0, nweak_rows = 0;
    double weak_frac = 1e-2;    // ... those with column mass A'1 below this fraction of the largest
    // workspaces
    sid::DBuf vp, ip, bp, ipart, vhat, ihat, bhat, red;
    sid::DBuf ws[9];            // solver state (polyphase volumes); [6..8] component reconstruction
    sid::DBuf errflag;          // device int: nonzero after a bounded wait expired
    sid::KTimer timer;          // dominant-kernel timing (sid_plan_timing_*)
    int zsplit;
    // neuron-kernel composition (sid_plan_set_kernel): kernel kx x ky x kz, two volume
    // scratch buffers and a polyphase one
    sid::DBuf kern, kvol[3];
    int64_t kdims[3] = {0, 0, 0};
    // host-array calls: [0] work stream, [1] side stream (copies, higher priority);
    // events: [0] input volume converted, [1] Htf converted, [2] caller's stream 0
    cudaStream_t hstream[2] = {nullptr, nullptr};
    cudaEvent_t hevent[3] = {nullptr, nullptr, nullptr};
    // library generation on the tensor cores: tap spectra on a small lenslet
    // window and the per-pass workspaces (libtc.cu)
    sid::LibWin* libwin = nullptr;
};

namespace sid {
// projector building blocks (polyphase in, polyphase out)
int direct_forward(sid_plan* p, const float* vp, float* ip, int* err, cudaStream_t st);
int direct_adjoint(sid_plan* p, const float* ip, float* bp, int* err, cudaStream_t st);
int spectral_forward(sid_plan* p, bool i16, const float* vp, float* ip, cudaStream_t st);
// storage formats of the tap spectra
enum SpecFmt { FMT_F32 = 0, FMT_I16 = 1, FMT_F24 = 2 };
int spectral_adjoint(sid_plan* p, int fmt, const float* ip, float* bp, cudaStream_t st);
// the forward contraction over input channels [c0, c1) (c0 on a 4-channel
// boundary) from p->vhat into p->ihat, added to it when accum
int spectral_forward_part(sid_plan* p, bool i16, int64_t c0, int64_t c1, bool accum, cudaStream_t st);
int ensure_spec_ws(sid_plan* p);  // the channel spectra buffers p->vhat, p->ihat of one volume
// the back projection's contraction alone: sensor lattice ip -> channel spectra p->vhat
int spectral_adjoint_spectra(sid_plan* p, int fmt, const float* ip, cudaStream_t st);
// nb (<= 4) polyphase volumes / images back to back
int spectral_forward_batch(sid_plan* p, bool i16, const float* vp, float* ip, int nb, cudaStream_t st);
int spectral_adjoint_batch(sid_plan* p, int fmt, const float* ip, float* bp, int nb, cudaStream_t st);
// many volumes per pass on the tensor cores (spec_tc.cu; plan flag SID_PLAN_SPECTRAL_TC)
int build_spectra_tc(sid_plan* p);
int spectral_tc_max_volumes();
int spectral_tc_group(const sid_plan* p, int64_t nb);  // volumes per pass that fit the device memory
int64_t vol_group(const sid_plan* p, int method, int64_t nb);  // deconv.cu: volumes per batched pass
int spectral_forward_tc(sid_plan* p, const float* vp, float* ip, int nb, cudaStream_t st);
int spectral_adjoint_tc(sid_plan* p, const float* ip, float* bp, int nb, cudaStream_t st);
// the contraction alone: A = 24-bit planes (rows x kp per frequency, reduction
// from element 64 akb0), B = nbp (3: hi, mid, lo; 2: hi, lo) BF16 planes
// [f][BN][kpb] back to back, out [f][nb][rows]
int spec_tc_forward_raw(const void* ah, const void* al, int64_t rows, int64_t kp, int akb0, const uint16_t* bplanes,
                        int nbp, int64_t kpb, int64_t nf, int nb, float2* out, int* err, cudaStream_t st);
// dst[b][c][f] = src[f][b][c] for c < nch (rows >= nch per frequency and volume)
int spec_tc_unpack(const float2* src, int nb, int rows, int nch, int64_t nf, float2* dst, cudaStream_t st);
int plan_sync(sid_plan* p, cudaStream_t st);  // synchronise; an expired device wait -> SID_ETIMEOUT
void libwin_free(sid_plan* p);
void libwin_release_workspaces(sid_plan* p);
// lenslet-grid real DFTs of nch channels (spectral.cu): planes [ch][Ly][Lx] <-> half spectra [ch][nf]
int spec_r2c(sid_plan* p, const float* in, float2* out, int64_t nch, cudaStream_t st);
int spec_c2r(sid_plan* p, const float2* in, float* out, int64_t nch, cudaStream_t st);
int conv_poly(sid_plan* p, const float* in_vp, float* out_vp, cudaStream_t st);
int weak_build(sid_plan* p);
int weak_fix(sid_plan* p, const float* ip, float* bp, cudaStream_t st);
int weak_fix_n(sid_plan* p, const float* ip, float* bp, int nb, cudaStream_t st);  // nb back to back
int weak_qsplit(const sid_plan* p, int64_t nb);  // CTAs per weak run (> 1: a finishing launch adds the parts)
bool weak_runs_path(const sid_plan* p);          // the weak voxels go through the run kernels
int weak_pad(sid_plan* p, const float* ip, int nb, cudaStream_t st);                   // lattice copies
int weak_runs(sid_plan* p, float* bp, int nb, int64_t z0, int64_t z1, cudaStream_t st);  // depths [z0, z1)
int64_t libwin_bytes(const sid_plan* p);         // device bytes of the library windows
int v_to_vp(const sid_plan* p, const float* V, float* vp, int64_t Z, cudaStream_t st);
int vp_to_v(const sid_plan* p, const float* vp, float* V, int64_t Z, cudaStream_t st);
int mask_vp(const sid_plan* p, float* vp, int64_t Z, cudaStream_t st);
inline int64_t vol_plane_elems(const sid_plan* p) { return p->N * p->N * p->Lx * p->Ly; }
}  // namespace sid

// NNLS / contraction context (declared in sid.h as struct sid_ctx).
struct sid_ctx {
    int device;
    sid::DBuf a_hi, a_lo, b_hi, b_lo, ws, scal, errflag;
    // Power-of-two operand scales that stay on the device (kScaleWords words,
    // allocated with the context so its address never changes): words 4s and
    // 4s+1 hold the absmax bits and scale of pixel-operand slot s (s = 0, 1),
    // 8..10 the right operand's absmax, scale and the product's alpha, 12..14
    // the same for the FP16-movie contraction.
    sid::DBuf scales;
    sid::DBuf nn[16];  // NNLS iteration state
    sid::DBuf mf[8];   // NMF step workspaces (T_update / S_update)
    sid::DBuf bg[6];   // movie scans (rank-1 background, standard-deviation image)
    sid::DBuf pix[6];  // K-blocked 16-bit copies of pixel-major factors and their right operands
    sid::KTimer timer; // tensor-core GEMM launches of sid_gram / sid_cross (sid_ctx_timing_*)
};
