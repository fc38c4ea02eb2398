// plan.cu -- projector plan: PSF upload, lenslet-tap construction, error state.
//
// The reference re-uploads and re-transforms every PSF slice on every call
// (forwardProjectGPU.m:19 gpuArray(squeeze(H(:,:,aa,bb,cc))); conv2FFT_.m:14
// recomputes fft2 of the padded PSF).  Here the PSF is uploaded once and
// rearranged into lenslet taps K[abc][b'a'](m1,m2), the only form the kernels
// read (see sid_internal.cuh for the index algebra).
#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int build_spectra(sid_plan* p);  // spectral.cu

int sm_count()
{
    static std::mutex mu;
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    std::lock_guard<std::mutex> lk(mu);
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

// Tap builder.  One thread per tap; `adj_layout` selects [c][b][b'][a'][a]
// block order (adjoint kernels) instead of [c][b][a][b'][a'] (forward kernels).
// Each (block of N tap arrays) starts on a 32-float boundary: stride tbs.
__global__ void k_build_taps(const float* __restrict__ H, float* __restrict__ taps,
                             const int* __restrict__ lo_c, const int* __restrict__ mc_c,
                             const int* __restrict__ off_c, int64_t M, int N, int Z,
                             int dlo, int D, int64_t tbs, int adj_layout)
{
    const int64_t D2 = (int64_t)D * D;
    const int64_t per_block = (int64_t)N * D2;
    const int64_t nblocks = (int64_t)Z * N * N * N;
    const int64_t total = nblocks * per_block;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int64_t blk = idx / per_block;
        int64_t rem = idx - blk * per_block;
        int inner = (int)(rem / D2);  // a' (forward layout) or a (adjoint layout)
        int64_t m = rem - (int64_t)inner * D2;
        int m1 = (int)(m / D), m2 = (int)(m - (int64_t)m1 * D);
        // decode blk = ((c*N + b)*N + o1)*N + o2
        int o2 = (int)(blk % N);
        int64_t t = blk / N;
        int o1 = (int)(t % N);
        t /= N;
        int b = (int)(t % N);
        int c = (int)(t / N);
        int a, bp, ap;
        if (adj_layout) { bp = o1; ap = o2; a = inner; }
        else            { a = o1; bp = o2; ap = inner; }
        const int lo = lo_c[c], mc = mc_c[c], off = off_c[c];
        const int i = ap - a + off + N * (m1 + dlo);
        const int j = bp - b + off + N * (m2 + dlo);
        float v = 0.f;
        if (i >= 0 && i < mc && j >= 0 && j < mc)
            v = H[(int64_t)(lo + i) + M * ((int64_t)(lo + j) + M * (a + (int64_t)N * (b + (int64_t)N * c)))];
        taps[blk * tbs + rem] = v;
    }
}

static int build_taps(sid_plan* p, const float* dH, const std::vector<int>& lo,
                      const std::vector<int>& mc, const std::vector<int>& off,
                      DBuf& out, int adj_layout)
{
    const int64_t N = p->N, Z = p->Z, D = p->g.D;
    const int64_t tbs = cdiv(N * D * D, 32) * 32;
    const int64_t nblocks = Z * N * N * N;
    SID_TRY(out.alloc((size_t)(nblocks * tbs) * sizeof(float)));
    SID_CUDA_TRY(cudaMemset(out.p, 0, (size_t)(nblocks * tbs) * sizeof(float)));
    DBuf meta;
    SID_TRY(meta.alloc(3 * Z * sizeof(int)));
    std::vector<int> h(3 * Z);
    for (int64_t c = 0; c < Z; ++c) { h[c] = lo[c]; h[Z + c] = mc[c]; h[2 * Z + c] = off[c]; }
    cudaError_t e = cudaMemcpy(meta.p, h.data(), 3 * Z * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { meta.release(); SID_CUDA_TRY(e); }
    const int* dm = meta.as<int>();
    k_build_taps<<<4096, 256>>>(dH, out.as<float>(), dm, dm + Z, dm + 2 * Z, p->M, (int)N, (int)Z,
                                (int)p->g.dlo, (int)D, tbs, adj_layout);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    meta.release();
    SID_CUDA_TRY(e);
    return SID_OK;
}

int smem_attr(const void* func, size_t bytes)
{
    SID_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SID_OK;
}

}  // namespace sid

using namespace sid;

extern "C" const char* sid_last_error(void) { return sid::g_err; }
extern "C" int sid_version(void) { return 10000; }

extern "C" int sid_plan_create(const float* H, int64_t M, int64_t Nnum, int64_t Z,
                               const int32_t* CAindex, int64_t X, int64_t Y, int flags,
                               sid_plan** out)
{
    SID_REQUIRE(out != nullptr, "sid_plan_create: plan output pointer is NULL");
    *out = nullptr;
    SID_REQUIRE(H != nullptr, "sid_plan_create: H is NULL");
    SID_REQUIRE(M >= 1 && Nnum >= 1 && Z >= 1 && X >= 1 && Y >= 1,
                "sid_plan_create: sizes must be positive (M=%lld Nnum=%lld Z=%lld X=%lld Y=%lld)",
                (long long)M, (long long)Nnum, (long long)Z, (long long)X, (long long)Y);
    SID_REQUIRE(Nnum <= 32, "sid_plan_create: Nnum=%lld exceeds 32", (long long)Nnum);
    SID_REQUIRE((flags & (SID_PLAN_DIRECT | SID_PLAN_SPECTRAL_F32 | SID_PLAN_SPECTRAL_I16 | SID_PLAN_SPECTRAL_F24)) != 0,
                "sid_plan_create: flags select no operator form");
    std::vector<int> lo(Z), mc(Z), cf(Z), cb(Z);
    for (int64_t c = 0; c < Z; ++c) {
        int64_t l = 1, h = M;
        if (CAindex) { l = CAindex[c]; h = CAindex[Z + c]; }
        SID_REQUIRE(l >= 1 && h <= M && l <= h,
                    "sid_plan_create: CAindex(%lld,:) = [%lld %lld] outside [1, %lld]",
                    (long long)(c + 1), (long long)l, (long long)h, (long long)M);
        lo[c] = (int)(l - 1);
        mc[c] = (int)(h - l + 1);
        cf[c] = mc[c] / 2;               // conv2 'same' centre
        cb[c] = mc[c] - 1 - mc[c] / 2;   // centre after imrotate(., 180)
    }
    sid_plan* p = new sid_plan();
    p->M = M; p->N = Nnum; p->Z = Z; p->X = X; p->Y = Y;
    p->Lx = cdiv(X, Nnum); p->Ly = cdiv(Y, Nnum);
    p->flags = flags;
    cudaGetDevice(&p->device);
    p->adj_separate = false;
    int64_t dlo = INT64_MAX, dhi = INT64_MIN;
    for (int64_t c = 0; c < Z; ++c) {
        if (cb[c] != cf[c]) p->adj_separate = true;
        for (int which = 0; which < 2; ++which) {
            int64_t off = which ? cb[c] : cf[c];
            // need 0 <= (a'-a) + off + N d <= mc-1 for some a'-a in [-(N-1), N-1]
            int64_t l = ceildiv_signed(-off - (Nnum - 1), Nnum);
            int64_t h = floordiv(mc[c] - 1 - off + (Nnum - 1), Nnum);
            dlo = std::min(dlo, l);
            dhi = std::max(dhi, h);
        }
    }
    p->g = TapGeom{Nnum, Z, X, Y, p->Lx, p->Ly, dlo, dhi, dhi - dlo + 1};
    p->zsplit = 1;
    p->L = 0; p->nf = 0; p->spec_f32 = p->spec_i16 = p->spec_f24 = false;

    if (p->errflag.alloc(sizeof(int)) != SID_OK || cudaMemset(p->errflag.p, 0, sizeof(int)) != cudaSuccess) {
        sid_plan_destroy(p);
        return SID_ENOMEM;
    }
    // Upload H once.
    DBuf dH;
    const size_t hbytes = (size_t)(M * M * Nnum * Nnum * Z) * sizeof(float);
    int st = dH.alloc(hbytes);
    if (st != SID_OK) { delete p; return st; }
    cudaError_t e = cudaMemcpy(dH.p, H, hbytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        dH.release(); delete p;
        set_error("sid_plan_create: H upload failed: %s", cudaGetErrorString(e));
        return SID_ECUDA;
    }
    // Forward taps are always built: the spectral form is computed from them.
    st = build_taps(p, dH.as<float>(), lo, mc, cf, p->taps_f, 0);
    if (st == SID_OK && (flags & SID_PLAN_DIRECT))
        st = build_taps(p, dH.as<float>(), lo, mc, p->adj_separate ? cb : cf, p->taps_b, 1);
    dH.release();
    if (st == SID_OK && (flags & (SID_PLAN_SPECTRAL_F32 | SID_PLAN_SPECTRAL_I16 | SID_PLAN_SPECTRAL_F24))) {
        if (p->adj_separate) {
            set_error("sid_plan_create: the spectral form needs odd PSF crop widths "
                      "(even widths shift the reference's back projection by one pixel); "
                      "use SID_PLAN_DIRECT");
            st = SID_EINVAL;
        } else {
            st = build_spectra(p);
        }
    }
    if (st == SID_OK && (flags & SID_PLAN_SPECTRAL_TC)) {
        if (!(flags & SID_PLAN_SPECTRAL_F24)) {
            set_error("sid_plan_create: SID_PLAN_SPECTRAL_TC needs SID_PLAN_SPECTRAL_F24");
            st = SID_EINVAL;
        } else {
            st = build_spectra_tc(p);
        }
    }
    if (st != SID_OK) { sid_plan_destroy(p); return st; }
    *out = p;
    return SID_OK;
}

extern "C" int sid_plan_destroy(sid_plan* p)
{
    if (!p) return SID_OK;
    libwin_free(p);
    DBuf* bufs[] = {&p->taps_f, &p->taps_b, &p->khat_f32, &p->khat_i16, &p->rstep, &p->khat_f24h, &p->khat_f24l,
                    &p->khat_f24th, &p->khat_f24tl, &p->tcb, &p->tco, &p->twiddle, &p->weak, &p->weak_pad, &p->weak_part,
                    &p->kern, &p->kvol[0], &p->kvol[1], &p->kvol[2],
                    &p->vp, &p->ip, &p->bp, &p->ipart, &p->vhat, &p->ihat, &p->bhat, &p->red, &p->errflag};
    for (DBuf* b : bufs) b->release();
    for (DBuf& b : p->ws) b.release();
    p->timer.release();
    for (cudaStream_t& s : p->hstream)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t& e : p->hevent)
        if (e) cudaEventDestroy(e);
    delete p;
    return SID_OK;
}

extern "C" int sid_plan_release_workspaces(sid_plan* p)
{
    SID_REQUIRE(p, "sid_plan_release_workspaces: NULL plan");
    SID_CUDA_TRY(cudaDeviceSynchronize());
    DBuf* bufs[] = {&p->vp, &p->ip, &p->bp, &p->ipart, &p->vhat, &p->ihat, &p->bhat, &p->red, &p->tcb, &p->tco,
                    &p->kvol[0], &p->kvol[1], &p->kvol[2], &p->weak_part};
    for (DBuf* b : bufs) b->release();
    for (DBuf& b : p->ws) b.release();
    libwin_release_workspaces(p);
    return SID_OK;
}

extern "C" int sid_plan_info(const sid_plan* p, int64_t* info)
{
    SID_REQUIRE(p && info, "sid_plan_info: NULL argument");
    const DBuf* bufs[] = {&p->taps_f, &p->taps_b, &p->khat_f32, &p->khat_i16, &p->rstep, &p->khat_f24h,
                          &p->khat_f24l, &p->khat_f24th, &p->khat_f24tl, &p->tcb, &p->tco, &p->twiddle,
                          &p->weak, &p->weak_pad, &p->kern, &p->kvol[0],
                          &p->kvol[1], &p->kvol[2], &p->vp, &p->ip, &p->bp, &p->ipart, &p->vhat, &p->ihat,
                          &p->bhat, &p->red, &p->weak_part};
    int64_t bytes = libwin_bytes(p);
    for (const DBuf* b : bufs) bytes += (int64_t)b->bytes;
    for (const DBuf& b : p->ws) bytes += (int64_t)b.bytes;
    // launches of one volume's weak-voxel fix: lattice copy, column and row runs, the split's sum
    const int64_t weak_launches =
        p->nweak == 0 ? 0
                      : (p->weak_pad.p ? 1 + (p->nweak_cols > 0) + (p->nweak_rows > 0) + (weak_qsplit(p, 1) > 1) : 1);
    int64_t v[14] = {p->M, p->N, p->Z, p->X, p->Y, p->Lx, p->Ly, p->g.D, p->L, bytes,
                     p->flags, p->adj_separate ? 1 : 0, p->nweak, weak_launches};
    std::memcpy(info, v, sizeof(v));
    return SID_OK;
}

extern "C" int sid_plan_timing_enable(sid_plan* p, int on)
{
    SID_REQUIRE(p, "sid_plan_timing_enable: NULL plan");
    if (on && !p->timer.on) p->timer.used = 0;
    p->timer.on = on != 0;
    return SID_OK;
}

extern "C" int sid_plan_timing_read(sid_plan* p, double* total_ms, int64_t* launches)
{
    SID_REQUIRE(p && total_ms && launches, "sid_plan_timing_read: NULL argument");
    double t = 0.0;
    for (size_t i = 0; i < p->timer.used; ++i) {
        SID_CUDA_TRY(cudaEventSynchronize(p->timer.end[i]));
        float ms = 0.f;
        SID_CUDA_TRY(cudaEventElapsedTime(&ms, p->timer.beg[i], p->timer.end[i]));
        t += ms;
    }
    *total_ms = t;
    *launches = (int64_t)p->timer.used;
    p->timer.used = 0;
    return SID_OK;
}
