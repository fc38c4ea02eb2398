// recon.cu -- MATLAB quantiles on the GPU and the per-component driver of
// reconstruct_S (reconstruct_S.m:130-148 CPU branch, :169-205 GPU branch).
//
// Quantile (MATLAB `quantile` of a vector): with the n non-NaN values sorted,
// x(k) sits at probability (k - 0.5)/n; p maps to position pos = n*p + 0.5,
// clamped to [1, n], and the result interpolates linearly between x(floor(pos))
// and x(floor(pos) + 1).  Both order statistics come from one radix select
// over the order-preserving 32-bit keys of the floats: three histogram passes
// (11, 11 and 10 bits), each followed by a one-block kernel that picks the
// digit holding the wanted rank.  Every count and rank stays in device memory,
// so the selection needs no host round trip.
//
// Component reconstruction, all on the plan's stream:
//   img = max(img - quantile(img(microlenses == 0), q), 0); img = img / max(img)
//   nrm = ||img||_2; Htf = A'(img / nrm)
//   lamb_L1 = min(quantile(Htf, 1 - 1e-4), lamb_L1)
//   X = nrm * LS_deconv(A, A', Htf)   or   nrm * deconvRL(A, A', Htf, maxIter, Htf)
#include <cmath>
#include <cstring>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

namespace {

constexpr int kQBins = 2048;
// digits of the three passes: bits 31..21, 20..10, 9..0
__host__ __device__ __forceinline__ int qbits(int pass) { return pass == 2 ? 10 : 11; }
__host__ __device__ __forceinline__ int qshift(int pass) { return pass == 0 ? 21 : (pass == 1 ? 10 : 0); }

// Selection state for two ranks (the two neighbours of one quantile).
struct QState {
    unsigned prefix[2];
    unsigned mask[2];
    long long rank[2];
    long long n;       // valid (non-NaN, not excluded) values
    double frac;       // interpolation weight of the upper neighbour
    double p;
    unsigned hist[2][kQBins];
};

__device__ __forceinline__ unsigned float_key(float f)
{
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_float(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Histogram of the current digit of the values whose key matches each
// target's prefix.  Warp-aggregated shared-memory counts; the loop is
// warp-uniform so that __match_any_sync sees every lane.
__global__ void __launch_bounds__(512) k_qhist(const float* __restrict__ x, int64_t n,
                                               const uint8_t* __restrict__ excl, QState* __restrict__ s, int pass)
{
    __shared__ unsigned h[2][kQBins];
    for (int i = threadIdx.x; i < 2 * kQBins; i += blockDim.x) (&h[0][0])[i] = 0u;
    __syncthreads();
    const unsigned p0 = s->prefix[0], m0 = s->mask[0], p1 = s->prefix[1], m1 = s->mask[1];
    const int shift = qshift(pass);
    const unsigned dmask = (1u << qbits(pass)) - 1u;
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp0 * 32; base < n; base += nwarps * 32) {
        const int64_t i = base + lane;
        bool ok = i < n;
        float v = 0.f;
        if (ok) {
            v = x[i];
            ok = !isnan(v) && !(excl && excl[i]);
        }
        const unsigned key = float_key(v);
        const unsigned d = (key >> shift) & dmask;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const unsigned pf = t ? p1 : p0, mk = t ? m1 : m0;
            const int bin = (ok && (key & mk) == pf) ? (int)d : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            if (bin >= 0 && lane == __ffs(peers) - 1) atomicAdd(&h[t][bin], (unsigned)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * kQBins; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c) atomicAdd(&(&s->hist[0][0])[i], c);
    }
}

// Pick the digit of each target (one block).  Pass 0 also counts the valid
// values and turns p into the two ranks.
__global__ void k_qselect(QState* __restrict__ s, int pass)
{
    const int shift = qshift(pass);
    const unsigned dmask = (1u << qbits(pass)) - 1u;
    const int nbins = 1 << qbits(pass);
    if (threadIdx.x == 0) {
        if (pass == 0) {
            long long n = 0;
            for (int b = 0; b < nbins; ++b) n += s->hist[0][b];
            s->n = n;
            double pos = (double)n * s->p + 0.5;  // 1-based
            long long lo;
            double frac;
            if (n == 0) {
                lo = 0;
                frac = 0.0;
            } else if (pos < 1.0) {
                lo = 1;
                frac = 0.0;
            } else if (pos >= (double)n) {
                lo = n;
                frac = 0.0;
            } else {
                lo = (long long)floor(pos);
                frac = pos - (double)lo;
            }
            s->frac = frac;
            s->rank[0] = lo > 0 ? lo - 1 : 0;
            s->rank[1] = (lo < n) ? lo : (lo > 0 ? lo - 1 : 0);
        }
        for (int t = 0; t < 2; ++t) {
            long long cum = 0, r = s->rank[t];
            int pick = nbins - 1;
            for (int b = 0; b < nbins; ++b) {
                const long long c = s->hist[t][b];
                if (cum + c > r) {
                    pick = b;
                    break;
                }
                cum += c;
            }
            s->rank[t] = r - cum;
            s->prefix[t] |= (unsigned)pick << shift;
            s->mask[t] |= dmask << shift;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * kQBins; i += blockDim.x) (&s->hist[0][0])[i] = 0u;
}

__global__ void k_qinit(QState* __restrict__ s, double p)
{
    for (int i = threadIdx.x; i < 2 * kQBins; i += blockDim.x) (&s->hist[0][0])[i] = 0u;
    if (threadIdx.x == 0) {
        s->prefix[0] = s->prefix[1] = 0u;
        s->mask[0] = s->mask[1] = 0u;
        s->rank[0] = s->rank[1] = 0;
        s->n = 0;
        s->frac = 0.0;
        s->p = p;
    }
}

__global__ void k_qfinish(const QState* __restrict__ s, double* __restrict__ out)
{
    if (s->n == 0) {
        *out = nan("");
        return;
    }
    const double a = (double)key_float(s->prefix[0]), b = (double)key_float(s->prefix[1]);
    // a + frac*(b - a) with separate roundings (no FMA): the value NumPy computes
    *out = __dadd_rn(a, __dmul_rn(s->frac, __dsub_rn(b, a)));
}

// img2 = max(img - q, 0); *mx = max over img2 (non-negative floats: uint ordering)
__global__ void k_clip_max(const float* __restrict__ img, int64_t n, const double* __restrict__ q,
                           float* __restrict__ out, unsigned* __restrict__ mx)
{
    const double qv = *q;
    float m = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = (float)fmax((double)img[i] - qv, 0.0);
        out[i] = v;
        m = fmaxf(m, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

// img2 /= max; *ss += sum(img2.^2)
__global__ void k_div_sumsq(float* __restrict__ v, int64_t n, const unsigned* __restrict__ mx, double* __restrict__ ss)
{
    const float m = __uint_as_float(*mx);
    double a = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float w = v[i] / m;
        v[i] = w;
        a += (double)w * (double)w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(ss, a);
}

// v = v / sqrt(*ss)  (inverse = 0) or v = v * sqrt(*ss)  (inverse = 1)
__global__ void k_scale_norm(float* __restrict__ v, int64_t n, const double* __restrict__ ss, int inverse)
{
    const float nrm = (float)sqrt(*ss);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = inverse ? v[i] * nrm : v[i] / nrm;
}

inline unsigned qgrid(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 512), 152 * 4)); }

}  // namespace

// MATLAB quantile p of x (n values, NaN ignored, entries with excl != 0
// skipped); the result lands in d_out (device double).  work: sizeof(QState).
int quantile_dev(const float* x, int64_t n, const uint8_t* excl, double p, double* d_out, void* work,
                 cudaStream_t st)
{
    QState* s = static_cast<QState*>(work);
    k_qinit<<<1, 256, 0, st>>>(s, p);
    for (int pass = 0; pass < 3; ++pass) {
        if (n > 0) k_qhist<<<qgrid(n), 512, 0, st>>>(x, n, excl, s, pass);
        k_qselect<<<1, 256, 0, st>>>(s, pass);
    }
    k_qfinish<<<1, 1, 0, st>>>(s, d_out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

size_t quantile_work_bytes() { return sizeof(QState); }

}  // namespace sid

using namespace sid;

extern "C" int sid_quantile(sid_ctx* c, const float* x, int64_t n, const uint8_t* exclude, const double* p, int np,
                            double* out, void* stream)
{
    SID_REQUIRE(c && out && p, "sid_quantile: NULL argument");
    SID_REQUIRE(n >= 0 && (n == 0 || x), "sid_quantile: bad input");
    SID_REQUIRE(np >= 1 && np <= 64, "sid_quantile: 1..64 probabilities");
    for (int i = 0; i < np; ++i) SID_REQUIRE(p[i] >= 0.0 && p[i] <= 1.0, "sid_quantile: p[%d] outside [0, 1]", i);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SID_TRY(c->scal.alloc(quantile_work_bytes() + 64 * sizeof(double)));
    void* work = c->scal.p;
    double* d_out = reinterpret_cast<double*>(static_cast<char*>(c->scal.p) + quantile_work_bytes());
    for (int i = 0; i < np; ++i) SID_TRY(quantile_dev(x, n, exclude, p[i], d_out + i, work, st));
    SID_CUDA_TRY(cudaMemcpyAsync(out, d_out, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    return SID_OK;
}

extern "C" void sid_recon_defaults(sid_recon_opts* o)
{
    std::memset(o, 0, sizeof(*o));
    o->q = 0.8;          // reconstruct_S.m:93-95
    o->lamb_L1 = 0.0;    // :66-68
    o->lamb_L2 = 0.0;    // :69-71
    o->solver = 0;       // 'fast_nnls' -> LS_deconv (:79-81)
    o->max_iter = 8;     // :72-74 (LS_deconv) and :87-89 (maxIter, ISRA)
}

extern "C" int sid_reconstruct_component(sid_plan* p, int method, const float* img, const uint8_t* microlenses,
                                         const sid_recon_opts* o, float* X, double* lamb_used, void* stream)
{
    SID_REQUIRE(p && img && o && X, "sid_reconstruct_component: NULL argument");
    SID_REQUIRE(o->q >= 0.0 && o->q <= 1.0, "sid_reconstruct_component: q outside [0, 1]");
    SID_REQUIRE(o->solver == 0 || o->solver == 1,
                "sid_reconstruct_component: solver must be 0 ('fast_nnls') or 1 ('ISRA'); 'fast_ls' is not supported");
    SID_REQUIRE(o->max_iter >= 0, "sid_reconstruct_component: negative max_iter");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t nI = p->X * p->Y, nV = nI * p->Z;
    SID_TRY(p->ws[6].alloc((size_t)nI * sizeof(float)));
    SID_TRY(p->ws[8].alloc(quantile_work_bytes() + 64));
    float* im = p->ws[6].as<float>();
    void* qw = p->ws[8].p;
    double* dsc = reinterpret_cast<double*>(static_cast<char*>(p->ws[8].p) + quantile_work_bytes());
    // dsc[0] background quantile, dsc[1] sum of squares, dsc[2] Htf quantile, dsc[3] (uint) max
    unsigned* dmax = reinterpret_cast<unsigned*>(dsc + 3);
    SID_CUDA_TRY(cudaMemsetAsync(dsc + 1, 0, sizeof(double), st));
    SID_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned), st));
    // background clip and normalisation (:168-170, 190-191)
    SID_TRY(quantile_dev(img, nI, microlenses, o->q, dsc, qw, st));
    const unsigned g = (unsigned)std::min<int64_t>(cdiv(nI, 256), 152 * 8);
    k_clip_max<<<g, 256, 0, st>>>(img, nI, dsc, im, dmax);
    k_div_sumsq<<<g, 256, 0, st>>>(im, nI, dmax, dsc + 1);
    k_scale_norm<<<g, 256, 0, st>>>(im, nI, dsc + 1, 0);
    SID_CHECK_LAUNCH();
    // Htf = A'(img / nrm)  (:192)
    SID_TRY(sid_adjoint(p, method, im, X, stream));
    // lamb_L1 = min(quantile(Htf, 1 - 1e-4), lamb_L1)  (:193)
    SID_TRY(quantile_dev(X, nV, nullptr, 1.0 - 1e-4, dsc + 2, qw, st));
    double hq = 0.0;
    SID_CUDA_TRY(cudaMemcpyAsync(&hq, dsc + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    const double lamb = std::fmin(hq, o->lamb_L1);
    if (lamb_used) *lamb_used = lamb;
    if (o->solver == 0) {
        // X holds df = Htf on entry (:197)
        SID_TRY(sid_deconv_ls(p, method, X, o->max_iter, (float)lamb, (float)o->lamb_L2, stream));
    } else {
        // deconvRL(fwd, bwd, Htf, maxIter, Htf, opts) (:195)
        SID_TRY(p->ws[7].alloc((size_t)nV * sizeof(float)));
        float* htf = p->ws[7].as<float>();
        SID_CUDA_TRY(cudaMemcpyAsync(htf, X, (size_t)nV * sizeof(float), cudaMemcpyDeviceToDevice, st));
        SID_TRY(sid_deconv_isra(p, method, htf, X, o->max_iter, 0.f, stream));
    }
    // X = nrm * X  (:205)
    k_scale_norm<<<(unsigned)std::min<int64_t>(cdiv(nV, 256), 152 * 8), 256, 0, st>>>(X, nV, dsc + 1, 1);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Several components (reconstruct_S.m:162-212 reconstructs them side by side):
// the background clip, normalisation and lamb_L1 quantile per component, the
// back projection Htf and the solver for all components of a group together
// (sid_adjoint_batched, sid_deconv_ls_batched / sid_deconv_isra_batched), so
// the tap spectra stream once per group.
extern "C" int sid_reconstruct_components(sid_plan* p, int method, int64_t nc, const float* const* imgs,
                                          const uint8_t* microlenses, const sid_recon_opts* o, float* const* X,
                                          double* lamb_used, void* stream)
{
    SID_REQUIRE(p && imgs && o && X, "sid_reconstruct_components: NULL argument");
    SID_REQUIRE(nc >= 1, "sid_reconstruct_components: no components");
    for (int64_t c = 0; c < nc; ++c)
        SID_REQUIRE(imgs[c] && X[c], "sid_reconstruct_components: component %lld is NULL", (long long)c);
    SID_REQUIRE(o->q >= 0.0 && o->q <= 1.0, "sid_reconstruct_components: q outside [0, 1]");
    SID_REQUIRE(o->solver == 0 || o->solver == 1,
                "sid_reconstruct_components: solver must be 0 ('fast_nnls') or 1 ('ISRA'); 'fast_ls' is not "
                "supported");
    SID_REQUIRE(o->max_iter >= 0, "sid_reconstruct_components: negative max_iter");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t nI = p->X * p->Y, nV = nI * p->Z;
    const int64_t g = (p->spec_tc && method == SID_METHOD_SPECTRAL_MIXED) ? vol_group(p, method, nc)
                                                                          : std::min<int64_t>(nc, 32);
    SID_TRY(p->ws[6].alloc((size_t)(g * nI) * sizeof(float)));
    SID_TRY(p->ws[8].alloc(quantile_work_bytes() + (size_t)(4 * g + 8) * sizeof(double)));
    if (o->solver == 1) SID_TRY(p->ws[7].alloc((size_t)(g * nV) * sizeof(float)));
    void* qw = p->ws[8].p;
    double* dscs = reinterpret_cast<double*>(static_cast<char*>(p->ws[8].p) + quantile_work_bytes());
    std::vector<const float*> ims(g), hs(g);
    std::vector<float*> xs(g);
    std::vector<float> lamb(g);
    for (int64_t c0 = 0; c0 < nc; c0 += g) {
        const int m = (int)std::min<int64_t>(g, nc - c0);
        for (int b = 0; b < m; ++b) {
            // per component: dsc[0] background quantile, dsc[1] sum of squares, dsc[2] Htf quantile, dsc[3] max
            double* dsc = dscs + 4 * b;
            unsigned* dmax = reinterpret_cast<unsigned*>(dsc + 3);
            float* im = p->ws[6].as<float>() + b * nI;
            SID_CUDA_TRY(cudaMemsetAsync(dsc + 1, 0, sizeof(double), st));
            SID_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned), st));
            SID_TRY(quantile_dev(imgs[c0 + b], nI, microlenses, o->q, dsc, qw, st));
            const unsigned gr = (unsigned)std::min<int64_t>(cdiv(nI, 256), 152 * 8);
            k_clip_max<<<gr, 256, 0, st>>>(imgs[c0 + b], nI, dsc, im, dmax);
            k_div_sumsq<<<gr, 256, 0, st>>>(im, nI, dmax, dsc + 1);
            k_scale_norm<<<gr, 256, 0, st>>>(im, nI, dsc + 1, 0);
            SID_CHECK_LAUNCH();
            ims[b] = im;
            xs[b] = X[c0 + b];
        }
        // Htf = A'(img / nrm) for the group
        SID_TRY(sid_adjoint_batched(p, method, m, ims.data(), xs.data(), stream));
        for (int b = 0; b < m; ++b) {
            double* dsc = dscs + 4 * b;
            SID_TRY(quantile_dev(X[c0 + b], nV, nullptr, 1.0 - 1e-4, dsc + 2, qw, st));
        }
        std::vector<double> hq(4 * m);
        SID_CUDA_TRY(cudaMemcpyAsync(hq.data(), dscs, (size_t)(4 * m) * sizeof(double), cudaMemcpyDeviceToHost, st));
        SID_CUDA_TRY(cudaStreamSynchronize(st));
        for (int b = 0; b < m; ++b) {
            const double l = std::fmin(hq[4 * b + 2], o->lamb_L1);
            lamb[b] = (float)l;
            if (lamb_used) lamb_used[c0 + b] = l;
        }
        if (o->solver == 0) {
            SID_TRY(sid_deconv_ls_batched(p, method, m, xs.data(), o->max_iter, lamb.data(), (float)o->lamb_L2,
                                          stream));
        } else {
            for (int b = 0; b < m; ++b) {
                float* h = p->ws[7].as<float>() + b * nV;
                SID_CUDA_TRY(cudaMemcpyAsync(h, X[c0 + b], (size_t)nV * sizeof(float), cudaMemcpyDeviceToDevice, st));
                hs[b] = h;
            }
            SID_TRY(sid_deconv_isra_batched(p, method, m, hs.data(), xs.data(), o->max_iter, 0.f, stream));
        }
        for (int b = 0; b < m; ++b) {
            k_scale_norm<<<(unsigned)std::min<int64_t>(cdiv(nV, 256), 152 * 8), 256, 0, st>>>(X[c0 + b], nV,
                                                                                           dscs + 4 * b + 1, 1);
            SID_CHECK_LAUNCH();
        }
    }
    return SID_OK;
}
