// deconv.cu -- C-ABI projector entry points and the deconvolution solvers.
//
// Solvers keep their state in the polyphase layout of the projector kernels
// (Vp[c][b][a][v][u]), so an iteration is: forward (polyphase in/out),
// adjoint, and one fused elementwise pass; the V <-> Vp transposes run only at
// entry and exit.
#include <algorithm>
#include <cmath>

#include <utility>

#include "sid_internal.cuh"

namespace sid {

static cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Projection in the polyphase layout; with a neuron kernel set, the volume is
// convolved with it first (reconstruct_S.m:126) and back projections are
// convolved after (:127).
int fwd_poly(sid_plan* p, int method, const float* vp, float* ip, cudaStream_t st)
{
    if (p->kdims[0]) {
        SID_TRY(p->kvol[2].alloc((size_t)(vol_plane_elems(p) * p->Z) * sizeof(float)));
        SID_TRY(conv_poly(p, vp, p->kvol[2].as<float>(), st));
        vp = p->kvol[2].as<float>();
    }
    switch (method) {
    case SID_METHOD_DIRECT: return direct_forward(p, vp, ip, p->errflag.as<int>(), st);
    case SID_METHOD_SPECTRAL_F32: return spectral_forward(p, false, vp, ip, st);
    case SID_METHOD_SPECTRAL_I16: return spectral_forward(p, true, vp, ip, st);
    case SID_METHOD_SPECTRAL_MIXED: return spectral_forward(p, true, vp, ip, st);
    case SID_METHOD_SPECTRAL_MIXED_F32: return spectral_forward(p, true, vp, ip, st);
    default: set_error("unknown projection method %d", method); return SID_EINVAL;
    }
}

// Spectral back projections are followed by the exact recomputation of the
// weakly observed voxels (weak.cu), then by the neuron kernel if one is set.
static int adj_raw(sid_plan* p, int method, const float* ip, float* bp, cudaStream_t st);

int adj_poly(sid_plan* p, int method, const float* ip, float* bp, cudaStream_t st)
{
    SID_TRY(adj_raw(p, method, ip, bp, st));
    return p->kdims[0] ? conv_poly(p, bp, bp, st) : SID_OK;
}

static int adj_raw(sid_plan* p, int method, const float* ip, float* bp, cudaStream_t st)
{
    int fmt = FMT_F32;
    switch (method) {
    case SID_METHOD_DIRECT: return direct_adjoint(p, ip, bp, p->errflag.as<int>(), st);
    case SID_METHOD_SPECTRAL_F32: fmt = FMT_F32; break;
    case SID_METHOD_SPECTRAL_I16: fmt = FMT_I16; break;
    case SID_METHOD_SPECTRAL_MIXED: fmt = FMT_F24; break;
    case SID_METHOD_SPECTRAL_MIXED_F32: fmt = FMT_F32; break;
    default: set_error("unknown projection method %d", method); return SID_EINVAL;
    }
    SID_TRY(spectral_adjoint(p, fmt, ip, bp, st));
    return weak_fix(p, ip, bp, st);
}

int ensure_proj_ws(sid_plan* p)
{
    SID_TRY(p->vp.alloc((size_t)(vol_plane_elems(p) * p->Z) * sizeof(float)));
    SID_TRY(p->bp.alloc((size_t)(vol_plane_elems(p) * p->Z) * sizeof(float)));
    SID_TRY(p->ip.alloc((size_t)vol_plane_elems(p) * sizeof(float)));
    SID_TRY(p->red.alloc(4096 * sizeof(double)));
    return SID_OK;
}

// Synchronise `st` and turn an expired device wait into SID_ETIMEOUT.
int plan_sync(sid_plan* p, cudaStream_t st)
{
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    int flag = 0;
    SID_CUDA_TRY(cudaMemcpy(&flag, p->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        cudaMemset(p->errflag.p, 0, sizeof(int));
        set_error("a device-side wait exceeded its budget (code %d)", flag);
        return SID_ETIMEOUT;
    }
    return SID_OK;
}

// ------------------------------------------------------ elementwise + sums --
constexpr int kRedBlocks = 1024;

// Sums on the FP32 pipes: exact products (fmaf two-product) added as
// unevaluated pairs hi + lo (two-sum), as accurate as FP64 accumulation.
// GB300's FP64 rate is about 1/64 of its FP32 rate: an FP64 product and add
// per voxel made the dot products of a 31-million-voxel volume FP64-bound at
// about four times their memory time.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    const float l = (a.y + b.y) + e;
    const float hi = s + l;
    return make_float2(hi, l - (hi - s));
}

// partial[block] = sum over the block's grid-stride range of a[i]*b[i]
__global__ void __launch_bounds__(256) k_dot_partial(const float* __restrict__ a, const float* __restrict__ b,
                                                     int64_t n, double* __restrict__ partial)
{
    __shared__ float2 red[8];
    float2 s = make_float2(0.f, 0.f);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = a[i], y = b[i];
        const float p = x * y;
        s = ff_add(s, make_float2(p, fmaf(x, y, -p)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s = ff_add(s, make_float2(__shfl_xor_sync(0xffffffffu, s.x, o), __shfl_xor_sync(0xffffffffu, s.y, o)));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 t = red[0];
        for (int w = 1; w < 8; ++w) t = ff_add(t, red[w]);
        partial[blockIdx.x] = (double)t.x + (double)t.y;
    }
}

// *out = sum of the partials (one CTA); with `alpha`, also the LS step size
// *num / *out as FP32, 0 where not finite (LS_deconv.m:86-88)
__global__ void k_sum_partials(const double* __restrict__ partial, int n, double* __restrict__ out,
                               const double* __restrict__ num, float* __restrict__ alpha)
{
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *out = red[0];
        if (alpha) {
            const float a = (float)(*num / red[0]);
            *alpha = isfinite(a) ? a : 0.f;
        }
    }
}

// out = sum a.*b, deterministic two-stage reduction into `out` (device double)
static int dot(const float* a, const float* b, int64_t n, double* scratch, double* out, cudaStream_t st,
               const double* num = nullptr, float* alpha = nullptr)
{
    k_dot_partial<<<kRedBlocks, 256, 0, st>>>(a, b, n, scratch);
    SID_CHECK_LAUNCH();
    k_sum_partials<<<1, 256, 0, st>>>(scratch, kRedBlocks, out, num, alpha);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// ISRA update, deconvRL.m:52,55,85-87:
//   e = Htf ./ (B + lambda); e(isinf(e)) = 0; X = X .* e; X(isnan(X)) = 0
__device__ __forceinline__ float isra_one(float x, float h, float b, float lambda)
{
    const float den = (lambda != 0.f) ? b + lambda : b;
    float e = __fdiv_rn(h, den);
    if (isinf(e)) e = 0.f;
    const float v = x * e;
    return isnan(v) ? 0.f : v;
}

__global__ void k_isra_update(float* __restrict__ x, const float* __restrict__ htf, const float* __restrict__ b,
                              float lambda, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = isra_one(x[i], htf[i], b[i], lambda);
}

// the same on 16-byte-aligned arrays, four elements per load (the tail n % 4 by the first threads)
__global__ void k_isra_update4(float* __restrict__ x, const float* __restrict__ htf, const float* __restrict__ b,
                               float lambda, int64_t n)
{
    const int64_t n4 = n >> 2;
    float4* x4 = reinterpret_cast<float4*>(x);
    const float4* h4 = reinterpret_cast<const float4*>(htf);
    const float4* b4 = reinterpret_cast<const float4*>(b);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 xv = x4[i], hv = h4[i], bv = b4[i];
        x4[i] = make_float4(isra_one(xv.x, hv.x, bv.x, lambda), isra_one(xv.y, hv.y, bv.y, lambda),
                            isra_one(xv.z, hv.z, bv.z, lambda), isra_one(xv.w, hv.w, bv.w, lambda));
    }
    const int64_t t = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) x[t] = isra_one(x[t], htf[t], b[t], lambda);
}

static void launch_isra_update(float* x, const float* htf, const float* b, float lambda, int64_t n, cudaStream_t st)
{
    const bool al = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(htf) |
                      reinterpret_cast<uintptr_t>(b)) & 15u) == 0;
    if (al) k_isra_update4<<<1216, 256, 0, st>>>(x, htf, b, lambda, n);
    else k_isra_update<<<2048, 256, 0, st>>>(x, htf, b, lambda, n);
}

// Poisson RL ratio in sensor space: r = y / AX, 0 where not finite (AX = 0,
// and the lattice positions outside the sensor, where both are 0).
__global__ void k_rl_ratio(float* __restrict__ ax, const float* __restrict__ y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float r = __fdiv_rn(y[i], ax[i]);
        ax[i] = isfinite(r) ? r : 0.f;
    }
}

__global__ void k_fill(float* __restrict__ x, float v, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}

// d = B + l2*x - x + l1  (LS_deconv.m:73-75: df = Q(df) - df + lamb_L1 with x = df)
__global__ void k_ls_init(float* __restrict__ d, const float* __restrict__ b, const float* __restrict__ x,
                          float l1, float l2, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = b[i] + l2 * x[i] - x[i] + l1;
}

// d_ = ((x > 0) | (d < 0)) .* d   (LS_deconv.m:80-81)
__global__ void k_ls_passive(const float* __restrict__ x, const float* __restrict__ d, float* __restrict__ dm,
                             int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float di = d[i];
        dm[i] = (x[i] > 0.f || di < 0.f) ? di : 0.f;
    }
}

// xn = max(x - alpha*d_, 0); dm <- xn - x; x <- xn  (LS_deconv.m:89-91; alpha
// = s1/s2 with nan/inf -> 0, formed once by the reduction)
__global__ void k_ls_step(float* __restrict__ x, float* __restrict__ dm, const float* __restrict__ alpha_p,
                          int64_t n)
{
    const float alpha = *alpha_p;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float xo = x[i];
        float xn = xo - alpha * dm[i];
        if (xn < 0.f) xn = 0.f;
        dm[i] = xn - xo;
        x[i] = xn;
    }
}

// d += B + l2 * step   (LS_deconv.m:92: df = df + Q(df_ - Xguess))
__global__ void k_ls_grad(float* __restrict__ d, const float* __restrict__ b, const float* __restrict__ step,
                          float l2, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] += b[i] + l2 * step[i];
}

// ---------------------------------------------------------------- TV terms --
// Neighbours along x, y and z of a polyphase volume entry: Vp index
// i = u + Lx (v + Ly (a + N (b + N c))) holds V(a + N u, b + N v, c).  Entries
// past the volume (x >= X, y >= Y, or off the lattice) read 0, as convn's
// zero padding does (the polyphase padding itself holds zeros).
struct PolyGeom {
    int N, Lx, Ly, Z;
    int X, Y;
};

struct PolyPos {
    int u, v, a, b, c;
};

__device__ __forceinline__ float pv_at(const float* __restrict__ x, const PolyGeom& g, int u, int v, int a, int b,
                                       int c)
{
    if (c < 0 || c >= g.Z) return 0.f;
    if (a < 0) { a += g.N; --u; } else if (a >= g.N) { a -= g.N; ++u; }
    if (b < 0) { b += g.N; --v; } else if (b >= g.N) { b -= g.N; ++v; }
    if (u < 0 || u >= g.Lx || v < 0 || v >= g.Ly) return 0.f;
    if (a + g.N * u >= g.X || b + g.N * v >= g.Y) return 0.f;
    return x[u + (int64_t)g.Lx * (v + (int64_t)g.Ly * (a + g.N * (b + (int64_t)g.N * c)))];
}

// grid: x over the Lx*Ly lattice of one plane, y over the N*N*Z planes
__device__ __forceinline__ bool poly_pos(const PolyGeom& g, PolyPos& p, int64_t& i)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Lx * g.Ly) return false;
    const int pl = blockIdx.y;  // a + N (b + N c)
    p.u = e % g.Lx;
    p.v = e / g.Lx;
    p.a = pl % g.N;
    p.b = (pl / g.N) % g.N;
    p.c = pl / (g.N * g.N);
    i = e + (int64_t)g.Lx * g.Ly * pl;
    return true;
}

__device__ __forceinline__ float sgnf(float v) { return v > 0.f ? 1.f : (v < 0.f ? -1.f : 0.f); }

// deconvRL.m:61-87 (mode 'TV'), out-of-place (the stencil reads the old X):
//   p = 1: dx = sign(convn(X, center-left)) = sign(X(x) - X(x+1)) (y, z alike),
//          den = A'AX + l1 dx + l2 dy + l3 dz + sum(l),
//          num = Htf + l1 dx(x-1) + l2 dy(y-1) + l3 dz(z-1) + sum(l);
//   p = 2: den = A'AX + 2 sum(l) X, num = Htf + convn(X, filt) = Htf + l1 (X(x+1) + X(x-1)) + ...;
//   e = num ./ den, e(isinf(e)) = 0, X = X .* e, X(isnan(X)) = 0.
__global__ void k_isra_tv(float* __restrict__ xn, const float* __restrict__ x, const float* __restrict__ htf,
                          const float* __restrict__ b, PolyGeom g, int pnorm, float l1, float l2, float l3)
{
    PolyPos q;
    int64_t i;
    if (!poly_pos(g, q, i)) return;
    const float xi = x[i];
    const float lsum = (float)((double)l1 + (double)l2 + (double)l3);
    float den, num;
    if (pnorm == 1) {
        const float dxp = sgnf(xi - pv_at(x, g, q.u, q.v, q.a + 1, q.b, q.c));
        const float dyp = sgnf(xi - pv_at(x, g, q.u, q.v, q.a, q.b + 1, q.c));
        const float dzp = sgnf(xi - pv_at(x, g, q.u, q.v, q.a, q.b, q.c + 1));
        // dx at x - 1 (0 at the first plane: convn(dx, right) reads dx(0) = 0)
        const bool hx = (q.a + g.N * q.u) > 0, hy = (q.b + g.N * q.v) > 0, hz = q.c > 0;
        const float dxm = hx ? sgnf(pv_at(x, g, q.u, q.v, q.a - 1, q.b, q.c) - xi) : 0.f;
        const float dym = hy ? sgnf(pv_at(x, g, q.u, q.v, q.a, q.b - 1, q.c) - xi) : 0.f;
        const float dzm = hz ? sgnf(pv_at(x, g, q.u, q.v, q.a, q.b, q.c - 1) - xi) : 0.f;
        den = (((b[i] + l1 * dxp) + l2 * dyp) + l3 * dzp) + lsum;
        num = (((htf[i] + l1 * dxm) + l2 * dym) + l3 * dzm) + lsum;
    } else {
        den = b[i] + (2.f * lsum) * xi;
        const float cx = pv_at(x, g, q.u, q.v, q.a + 1, q.b, q.c) + pv_at(x, g, q.u, q.v, q.a - 1, q.b, q.c);
        const float cy = pv_at(x, g, q.u, q.v, q.a, q.b + 1, q.c) + pv_at(x, g, q.u, q.v, q.a, q.b - 1, q.c);
        const float cz = pv_at(x, g, q.u, q.v, q.a, q.b, q.c + 1) + pv_at(x, g, q.u, q.v, q.a, q.b, q.c - 1);
        num = htf[i] + (l1 * cx + l2 * cy + l3 * cz);
    }
    float e = __fdiv_rn(num, den);
    if (isinf(e)) e = 0.f;
    float v = xi * e;
    if (isnan(v)) v = 0.f;
    xn[i] = v;
}

// LS_deconv.m:53-59: lb_TV_L2(X) = convn(X, filter, 'same') with filter
// l1 at (+-1,0,0), l2 at (0,+-1,0), l3 at (0,0,+-1) and -sum(l) at the centre.
__device__ __forceinline__ float tv_l2_at(const float* __restrict__ x, const PolyGeom& g, const PolyPos& q, float xi,
                                          float l1, float l2, float l3)
{
    const float cx = pv_at(x, g, q.u, q.v, q.a + 1, q.b, q.c) + pv_at(x, g, q.u, q.v, q.a - 1, q.b, q.c);
    const float cy = pv_at(x, g, q.u, q.v, q.a, q.b + 1, q.c) + pv_at(x, g, q.u, q.v, q.a, q.b - 1, q.c);
    const float cz = pv_at(x, g, q.u, q.v, q.a, q.b, q.c + 1) + pv_at(x, g, q.u, q.v, q.a, q.b, q.c - 1);
    return (l1 * cx + l2 * cy + l3 * cz) - (float)((double)l1 + (double)l2 + (double)l3) * xi;
}

// d = B + lb_TV_L2(x) + l2 x - x + l1   (LS_deconv.m:73-75 with x = df)
__global__ void k_ls_init_tv(float* __restrict__ d, const float* __restrict__ b, const float* __restrict__ x,
                             PolyGeom g, float l1, float l2, float t1, float t2, float t3)
{
    PolyPos q;
    int64_t i;
    if (!poly_pos(g, q, i)) return;
    const float xi = x[i];
    d[i] = (((b[i] + tv_l2_at(x, g, q, xi, t1, t2, t3)) + l2 * xi) - xi) + l1;
}

// d += B + lb_TV_L2(step) + l2 step   (LS_deconv.m:92)
__global__ void k_ls_grad_tv(float* __restrict__ d, const float* __restrict__ b, const float* __restrict__ step,
                             PolyGeom g, float l2, float t1, float t2, float t3)
{
    PolyPos q;
    int64_t i;
    if (!poly_pos(g, q, i)) return;
    const float si = step[i];
    d[i] += (b[i] + tv_l2_at(step, g, q, si, t1, t2, t3)) + l2 * si;
}

// qd = B + lb_TV_L2(d) + l2 d   (Q(df_) of LS_deconv.m:83)
__global__ void k_ls_qd(float* __restrict__ qd, const float* __restrict__ b, const float* __restrict__ d, PolyGeom g,
                        float l2, float t1, float t2, float t3)
{
    PolyPos q;
    int64_t i;
    if (!poly_pos(g, q, i)) return;
    const float di = d[i];
    qd[i] = (b[i] + tv_l2_at(d, g, q, di, t1, t2, t3)) + l2 * di;
}

// Xguess_history(it, :, :, :) = X  (deconvRL.m:90-92): history is maxIter x X x Y x Z
__global__ void k_history(float* __restrict__ hist, const float* __restrict__ xp, PolyGeom g, int it, int maxIter)
{
    PolyPos q;
    int64_t i;
    if (!poly_pos(g, q, i)) return;
    const int xx = q.a + g.N * q.u, yy = q.b + g.N * q.v;
    if (xx >= g.X || yy >= g.Y) return;
    hist[it + (int64_t)maxIter * (xx + (int64_t)g.X * (yy + (int64_t)g.Y * q.c))] = xp[i];
}

static PolyGeom poly_geom(const sid_plan* p)
{
    return PolyGeom{(int)p->N, (int)p->Lx, (int)p->Ly, (int)p->Z, (int)p->X, (int)p->Y};
}

static dim3 poly_grid(const sid_plan* p) { return dim3((unsigned)cdiv(p->Lx * p->Ly, 256), (unsigned)(p->N * p->N * p->Z)); }

static int isra_update(sid_plan* p, float* xp, const float* hp, float lambda, cudaStream_t st)
{
    launch_isra_update(xp, hp, p->bp.as<float>(), lambda, vol_plane_elems(p) * p->Z, st);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Device address of a caller's host array, or nullptr (stage through copies):
// pinned or registered memory has one; pageable memory is device-accessible
// where the GPU walks the host's page tables (Grace-class systems).
static void* host_device_view(const void* h)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void*>(h);
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && pageable)
        return const_cast<void*>(h);
    return nullptr;
}

// The plan's streams for host-array calls, ordered after the caller's work on
// the legacy default stream.
static int host_streams(sid_plan* p, cudaStream_t* work, cudaStream_t* side)
{
    if (!p->hstream[0]) {
        int least = 0, greatest = 0;
        SID_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SID_CUDA_TRY(cudaStreamCreateWithPriority(&p->hstream[0], cudaStreamNonBlocking, least));
        SID_CUDA_TRY(cudaStreamCreateWithPriority(&p->hstream[1], cudaStreamNonBlocking, greatest));
        for (cudaEvent_t& e : p->hevent) SID_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    SID_CUDA_TRY(cudaEventRecord(p->hevent[2], 0));
    SID_CUDA_TRY(cudaStreamWaitEvent(p->hstream[0], p->hevent[2], 0));
    *work = p->hstream[0];
    *side = p->hstream[1];
    return SID_OK;
}

}  // namespace sid

using namespace sid;

extern "C" int sid_forward(sid_plan* p, int method, const float* V, float* I, void* stream)
{
    SID_REQUIRE(p && V && I, "sid_forward: NULL argument");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    SID_TRY(v_to_vp(p, V, p->vp.as<float>(), p->Z, st));
    SID_TRY(fwd_poly(p, method, p->vp.as<float>(), p->ip.as<float>(), st));
    SID_TRY(vp_to_v(p, p->ip.as<float>(), I, 1, st));
    return SID_OK;
}

extern "C" int sid_adjoint(sid_plan* p, int method, const float* I, float* V, void* stream)
{
    SID_REQUIRE(p && V && I, "sid_adjoint: NULL argument");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    SID_TRY(v_to_vp(p, I, p->ip.as<float>(), 1, st));
    SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
    SID_TRY(vp_to_v(p, p->bp.as<float>(), V, p->Z, st));
    return SID_OK;
}

// Host-array calls: where the device can address the caller's arrays, the
// layout kernels read the input and write the result over the host link
// directly (no staging pass); otherwise they stage through two plan-owned
// device buffers (ws[4], ws[5]) that persist across calls.
template <class F>
static int with_device_copies(sid_plan* p, const float* in_h, size_t in_n, float* out_h, size_t out_n, F fn)
{
    const float* iv = static_cast<const float*>(host_device_view(in_h));
    float* ov = static_cast<float*>(host_device_view(out_h));
    if (iv && ov) {
        cudaStream_t st, side;
        SID_TRY(host_streams(p, &st, &side));
        SID_TRY(fn(iv, ov, st));
        return plan_sync(p, st);
    }
    DBuf& din = p->ws[4];
    DBuf& dout = p->ws[5];
    SID_TRY(din.alloc(in_n * sizeof(float)));
    SID_TRY(dout.alloc(out_n * sizeof(float)));
    SID_CUDA_TRY(cudaMemcpy(din.p, in_h, in_n * sizeof(float), cudaMemcpyHostToDevice));
    SID_TRY(fn(din.as<float>(), dout.as<float>(), (cudaStream_t)0));
    SID_TRY(plan_sync(p, 0));
    SID_CUDA_TRY(cudaMemcpy(out_h, dout.p, out_n * sizeof(float), cudaMemcpyDeviceToHost));
    return SID_OK;
}

extern "C" int sid_forward_host(sid_plan* p, int method, const float* V, float* I)
{
    SID_REQUIRE(p && V && I, "sid_forward_host: NULL argument");
    return with_device_copies(p, V, (size_t)(p->X * p->Y * p->Z), I, (size_t)(p->X * p->Y),
                              [&](const float* dv, float* di, cudaStream_t st) { return sid_forward(p, method, dv, di, st); });
}

extern "C" int sid_adjoint_host(sid_plan* p, int method, const float* I, float* V)
{
    SID_REQUIRE(p && V && I, "sid_adjoint_host: NULL argument");
    return with_device_copies(p, I, (size_t)(p->X * p->Y), V, (size_t)(p->X * p->Y * p->Z),
                              [&](const float* di, float* dv, cudaStream_t st) { return sid_adjoint(p, method, di, dv, st); });
}

extern "C" int sid_deconv_isra(sid_plan* p, int method, const float* Htf, float* X, int maxIter, float lambda,
                               void* stream)
{
    SID_REQUIRE(p && Htf && X, "sid_deconv_isra: NULL argument");
    SID_REQUIRE(maxIter >= 0, "sid_deconv_isra: maxIter < 0");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z;
    SID_TRY(p->ws[0].alloc((size_t)n * sizeof(float)));
    SID_TRY(p->ws[1].alloc((size_t)n * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* hp = p->ws[1].as<float>();
    SID_TRY(v_to_vp(p, Htf, hp, p->Z, st));
    SID_TRY(v_to_vp(p, X, xp, p->Z, st));
    for (int it = 0; it < maxIter; ++it) {
        SID_TRY(fwd_poly(p, method, xp, p->ip.as<float>(), st));
        SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
        SID_TRY(isra_update(p, xp, hp, lambda, st));
    }
    SID_TRY(vp_to_v(p, xp, X, p->Z, st));
    return SID_OK;
}

extern "C" int sid_deconv_rl_poisson(sid_plan* p, int method, const float* y, float* X, int maxIter,
                                     void* stream)
{
    SID_REQUIRE(p && y && X, "sid_deconv_rl_poisson: NULL argument");
    SID_REQUIRE(maxIter >= 0, "sid_deconv_rl_poisson: maxIter < 0");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z;
    const int64_t ni = vol_plane_elems(p);
    SID_TRY(p->ws[0].alloc((size_t)n * sizeof(float)));
    SID_TRY(p->ws[1].alloc((size_t)n * sizeof(float)));
    SID_TRY(p->ws[2].alloc((size_t)ni * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* np_ = p->ws[1].as<float>();  // A'1
    float* yp = p->ws[2].as<float>();
    float* ip = p->ip.as<float>();
    float* bp = p->bp.as<float>();
    SID_TRY(v_to_vp(p, y, yp, 1, st));
    SID_TRY(v_to_vp(p, X, xp, p->Z, st));
    // normaliser A'1: ones on the sensor, zero at lattice positions outside it
    k_fill<<<1024, 256, 0, st>>>(ip, 1.f, ni);
    SID_CHECK_LAUNCH();
    SID_TRY(mask_vp(p, ip, 1, st));
    SID_TRY(adj_poly(p, method, ip, np_, st));
    for (int it = 0; it < maxIter; ++it) {
        SID_TRY(fwd_poly(p, method, xp, ip, st));
        k_rl_ratio<<<1024, 256, 0, st>>>(ip, yp, ni);
        SID_CHECK_LAUNCH();
        SID_TRY(adj_poly(p, method, ip, bp, st));
        // X <- X .* (A'r ./ A'1): the ISRA update with numerator A'r, denominator A'1
        launch_isra_update(xp, bp, np_, 0.f, n, st);
        SID_CHECK_LAUNCH();
    }
    SID_TRY(vp_to_v(p, xp, X, p->Z, st));
    return SID_OK;
}

extern "C" int sid_deconv_ls(sid_plan* p, int method, float* X, int max_iter, float lamb_L1, float lamb_L2,
                             void* stream)
{
    SID_REQUIRE(p && X, "sid_deconv_ls: NULL argument");
    SID_REQUIRE(max_iter >= 0, "sid_deconv_ls: max_iter < 0");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z;
    const int64_t ni = vol_plane_elems(p);
    for (int k = 0; k < 3; ++k) SID_TRY(p->ws[k].alloc((size_t)n * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* dp = p->ws[1].as<float>();
    float* tp = p->ws[2].as<float>();
    double* red = p->red.as<double>();
    double* s12 = red + kRedBlocks;  // two scalars after the partials, then alpha
    float* alpha = reinterpret_cast<float*>(s12 + 2);
    SID_TRY(v_to_vp(p, X, xp, p->Z, st));
    // df = Q(x0) - x0 + lamb_L1 with x0 = df
    SID_TRY(fwd_poly(p, method, xp, p->ip.as<float>(), st));
    SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
    k_ls_init<<<2048, 256, 0, st>>>(dp, p->bp.as<float>(), xp, lamb_L1, lamb_L2, n);
    SID_CHECK_LAUNCH();
    SID_TRY(mask_vp(p, dp, p->Z, st));
    for (int it = 0; it < max_iter; ++it) {
        k_ls_passive<<<2048, 256, 0, st>>>(xp, dp, tp, n);
        SID_CHECK_LAUNCH();
        SID_TRY(dot(tp, tp, n, red, s12, st));
        SID_TRY(fwd_poly(p, method, tp, p->ip.as<float>(), st));
        SID_TRY(dot(p->ip.as<float>(), p->ip.as<float>(), ni, red, s12 + 1, st, s12, alpha));
        k_ls_step<<<2048, 256, 0, st>>>(xp, tp, alpha, n);
        SID_CHECK_LAUNCH();
        SID_TRY(fwd_poly(p, method, tp, p->ip.as<float>(), st));
        SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
        k_ls_grad<<<2048, 256, 0, st>>>(dp, p->bp.as<float>(), tp, lamb_L2, n);
        SID_CHECK_LAUNCH();
    }
    SID_TRY(vp_to_v(p, xp, X, p->Z, st));
    return SID_OK;
}

extern "C" int sid_deconv_isra_ex(sid_plan* p, int method, const float* Htf, float* X, int maxIter, int mode,
                                  int pnorm, const float* lambda3, float* history, void* stream)
{
    SID_REQUIRE(p && Htf && X && lambda3, "sid_deconv_isra_ex: NULL argument");
    SID_REQUIRE(maxIter >= 0, "sid_deconv_isra_ex: maxIter < 0");
    SID_REQUIRE(mode == 0 || mode == 1, "sid_deconv_isra_ex: mode must be 0 ('basic') or 1 ('TV')");
    const float l1 = lambda3[0], l2 = mode ? lambda3[1] : 0.f, l3 = mode ? lambda3[2] : 0.f;
    const bool lam_on = mode ? (l1 != 0.f || l2 != 0.f || l3 != 0.f) : (l1 != 0.f);
    SID_REQUIRE(mode == 1 || !lam_on || pnorm == 1,
                "deconvRL: mode 'basic' with lambda ~= 0 and p ~= 1 uses the undefined Filter (deconvRL.m:57)");
    SID_REQUIRE(!p->X || p->X * p->Y < INT32_MAX, "sid_deconv_isra_ex: volume too large");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z;
    SID_TRY(p->ws[0].alloc((size_t)n * sizeof(float)));
    SID_TRY(p->ws[1].alloc((size_t)n * sizeof(float)));
    if (mode && lam_on) SID_TRY(p->ws[2].alloc((size_t)n * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* hp = p->ws[1].as<float>();
    SID_TRY(v_to_vp(p, Htf, hp, p->Z, st));
    SID_TRY(v_to_vp(p, X, xp, p->Z, st));
    const PolyGeom g = poly_geom(p);
    // mode 'TV' with p > 2 prints 'p>2 not supported' and returns X (deconvRL.m:79-81)
    const bool tv_stop = mode && lam_on && pnorm != 1 && pnorm != 2;
    for (int it = 0; it < maxIter && !tv_stop; ++it) {
        SID_TRY(fwd_poly(p, method, xp, p->ip.as<float>(), st));
        SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
        if (mode && lam_on) {
            float* xn = p->ws[2].as<float>();
            k_isra_tv<<<poly_grid(p), 256, 0, st>>>(xn, xp, hp, p->bp.as<float>(), g, pnorm, l1, l2, l3);
            SID_CHECK_LAUNCH();
            std::swap(p->ws[0], p->ws[2]);
            xp = p->ws[0].as<float>();
        } else {
            SID_TRY(isra_update(p, xp, hp, l1, st));
        }
        if (history) {
            k_history<<<poly_grid(p), 256, 0, st>>>(history, xp, g, it, maxIter);
            SID_CHECK_LAUNCH();
        }
    }
    SID_TRY(vp_to_v(p, xp, X, p->Z, st));
    return SID_OK;
}

extern "C" int sid_deconv_ls_ex(sid_plan* p, int method, float* X, int max_iter, float lamb_L1, float lamb_L2,
                                const float* lamb_TV_L2, float lamb_TV_L1, void* stream)
{
    SID_REQUIRE(p && X && lamb_TV_L2, "sid_deconv_ls_ex: NULL argument");
    SID_REQUIRE(max_iter >= 0, "sid_deconv_ls_ex: max_iter < 0");
    const float t1 = lamb_TV_L2[0], t2 = lamb_TV_L2[1], t3 = lamb_TV_L2[2];
    const bool tv = t1 != 0.f || t2 != 0.f || t3 != 0.f;  // max(opts.lamb_TV_L2) ~= 0 (LS_deconv.m:49)
    // alpha from Q itself only when lamb_TV_L1 * lamb_TV_L2 * lamb_L2 is nonzero in every component (LS_deconv.m:82)
    const bool qalpha = lamb_TV_L1 != 0.f && t1 != 0.f && t2 != 0.f && t3 != 0.f && lamb_L2 != 0.f;
    if (!tv && !qalpha) return sid_deconv_ls(p, method, X, max_iter, lamb_L1, lamb_L2, stream);
    SID_REQUIRE(p->X * p->Y < INT32_MAX, "sid_deconv_ls_ex: volume too large");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z;
    const int64_t ni = vol_plane_elems(p);
    for (int k = 0; k < 4; ++k) SID_TRY(p->ws[k].alloc((size_t)n * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* dp = p->ws[1].as<float>();
    float* tp = p->ws[2].as<float>();
    float* qp = p->ws[3].as<float>();
    double* red = p->red.as<double>();
    double* s12 = red + kRedBlocks;
    float* alpha = reinterpret_cast<float*>(s12 + 2);
    const PolyGeom g = poly_geom(p);
    const dim3 pg = poly_grid(p);
    SID_TRY(v_to_vp(p, X, xp, p->Z, st));
    // df = Q(x0) - x0 + lamb_L1 with x0 = df, Q = A'A + lb_TV_L2 + lamb_L2 I
    SID_TRY(fwd_poly(p, method, xp, p->ip.as<float>(), st));
    SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
    k_ls_init_tv<<<pg, 256, 0, st>>>(dp, p->bp.as<float>(), xp, g, lamb_L1, lamb_L2, t1, t2, t3);
    SID_CHECK_LAUNCH();
    SID_TRY(mask_vp(p, dp, p->Z, st));
    for (int it = 0; it < max_iter; ++it) {
        k_ls_passive<<<2048, 256, 0, st>>>(xp, dp, tp, n);
        SID_CHECK_LAUNCH();
        SID_TRY(dot(tp, tp, n, red, s12, st));
        if (qalpha) {
            // alpha = (df_' df_) / sum(df_ .* Q(df_))
            SID_TRY(fwd_poly(p, method, tp, p->ip.as<float>(), st));
            SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
            k_ls_qd<<<pg, 256, 0, st>>>(qp, p->bp.as<float>(), tp, g, lamb_L2, t1, t2, t3);
            SID_CHECK_LAUNCH();
            SID_TRY(dot(tp, qp, n, red, s12 + 1, st, s12, alpha));
        } else {
            // alpha = (df_' df_) / (v' v), v = A df_
            SID_TRY(fwd_poly(p, method, tp, p->ip.as<float>(), st));
            SID_TRY(dot(p->ip.as<float>(), p->ip.as<float>(), ni, red, s12 + 1, st, s12, alpha));
        }
        k_ls_step<<<2048, 256, 0, st>>>(xp, tp, alpha, n);
        SID_CHECK_LAUNCH();
        SID_TRY(fwd_poly(p, method, tp, p->ip.as<float>(), st));
        SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
        k_ls_grad_tv<<<pg, 256, 0, st>>>(dp, p->bp.as<float>(), tp, g, lamb_L2, t1, t2, t3);
        SID_CHECK_LAUNCH();
    }
    SID_TRY(vp_to_v(p, xp, X, p->Z, st));
    return SID_OK;
}

// --------------------------------------------------- several volumes at once --
// Projections of nb volumes (polyphase, back to back): on a plan built with
// SID_PLAN_SPECTRAL_TC the mixed form contracts up to 64 volumes per pass on
// the tensor cores (spec_tc.cu, the 24-bit spectra both ways); otherwise the
// spectral forms run up to four volumes per tap-spectrum pass on the FP32
// pipes (spectral_forward_batch).  The direct form and the per-volume steps
// (neuron kernel, weak-voxel recomputation) go volume by volume.
static bool use_tc(const sid_plan* p, int method, int nb)
{
    return p->spec_tc && method == SID_METHOD_SPECTRAL_MIXED && nb >= 2;
}
static int spectral_fmt_fwd(int method, bool* i16)
{
    switch (method) {
    case SID_METHOD_SPECTRAL_F32: *i16 = false; return 1;
    case SID_METHOD_SPECTRAL_I16:
    case SID_METHOD_SPECTRAL_MIXED:
    case SID_METHOD_SPECTRAL_MIXED_F32: *i16 = true; return 1;
    default: return 0;
    }
}

static int spectral_fmt_adj(int method)
{
    switch (method) {
    case SID_METHOD_SPECTRAL_F32: return FMT_F32;
    case SID_METHOD_SPECTRAL_I16: return FMT_I16;
    case SID_METHOD_SPECTRAL_MIXED: return FMT_F24;
    case SID_METHOD_SPECTRAL_MIXED_F32: return FMT_F32;
    default: return -1;
    }
}

int fwd_poly_batch(sid_plan* p, int method, const float* vp, float* ip, int nb, cudaStream_t st)
{
    const int64_t nv = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    bool i16 = false;
    if (nb == 1 || p->kdims[0] || !spectral_fmt_fwd(method, &i16)) {
        for (int b = 0; b < nb; ++b) SID_TRY(fwd_poly(p, method, vp + b * nv, ip + b * ni, st));
        return SID_OK;
    }
    if (use_tc(p, method, nb)) return spectral_forward_tc(p, vp, ip, nb, st);
    return spectral_forward_batch(p, i16, vp, ip, nb, st);
}

int adj_poly_batch(sid_plan* p, int method, const float* ip, float* bp, int nb, cudaStream_t st)
{
    const int64_t nv = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    const int fmt = spectral_fmt_adj(method);
    if (nb == 1 || fmt < 0) {
        for (int b = 0; b < nb; ++b) SID_TRY(adj_poly(p, method, ip + b * ni, bp + b * nv, st));
        return SID_OK;
    }
    if (use_tc(p, method, nb)) SID_TRY(spectral_adjoint_tc(p, ip, bp, nb, st));
    else SID_TRY(spectral_adjoint_batch(p, fmt, ip, bp, nb, st));
    SID_TRY(weak_fix_n(p, ip, bp, nb, st));
    if (p->kdims[0])
        for (int b = 0; b < nb; ++b) SID_TRY(conv_poly(p, bp + b * nv, bp + b * nv, st));
    return SID_OK;
}

// volumes per pass over the tap spectra
// (the tensor-core form takes up to 64 volumes per pass -- 1.4x less time per
// volume in the contraction than 32 -- where the device has room for the
// group's workspaces; spectral_tc_group)
int64_t sid::vol_group(const sid_plan* p, int method, int64_t nb)
{
    if (p->spec_tc && method == SID_METHOD_SPECTRAL_MIXED) return std::min<int64_t>(nb, spectral_tc_group(p, nb));
    return std::min<int64_t>(nb, 4);
}

extern "C" int sid_deconv_isra_batched(sid_plan* p, int method, int64_t nb, const float* const* Htf, float* const* X,
                                       int maxIter, float lambda, void* stream)
{
    SID_REQUIRE(p && Htf && X, "sid_deconv_isra_batched: NULL argument");
    SID_REQUIRE(nb >= 1 && maxIter >= 0, "sid_deconv_isra_batched: need nb >= 1 and maxIter >= 0");
    for (int64_t b = 0; b < nb; ++b)
        SID_REQUIRE(Htf[b] && X[b], "sid_deconv_isra_batched: volume %lld is NULL", (long long)b);
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t nv = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    const int64_t g = vol_group(p, method, nb);
    SID_TRY(p->ws[0].alloc((size_t)(g * nv) * sizeof(float)));  // iterates
    SID_TRY(p->ws[1].alloc((size_t)(g * nv) * sizeof(float)));  // Htf
    SID_TRY(p->ws[4].alloc((size_t)(g * nv) * sizeof(float)));  // back projections
    SID_TRY(p->ws[5].alloc((size_t)(g * ni) * sizeof(float)));  // images
    float* xp = p->ws[0].as<float>();
    float* hp = p->ws[1].as<float>();
    float* bp = p->ws[4].as<float>();
    float* ip = p->ws[5].as<float>();
    for (int64_t b0 = 0; b0 < nb; b0 += g) {
        const int n = (int)std::min<int64_t>(g, nb - b0);
        for (int b = 0; b < n; ++b) {
            SID_TRY(v_to_vp(p, Htf[b0 + b], hp + b * nv, p->Z, st));
            SID_TRY(v_to_vp(p, X[b0 + b], xp + b * nv, p->Z, st));
        }
        for (int it = 0; it < maxIter; ++it) {
            SID_TRY(fwd_poly_batch(p, method, xp, ip, n, st));
            SID_TRY(adj_poly_batch(p, method, ip, bp, n, st));
            launch_isra_update(xp, hp, bp, lambda, n * nv, st);
            SID_CHECK_LAUNCH();
        }
        for (int b = 0; b < n; ++b) SID_TRY(vp_to_v(p, xp + b * nv, X[b0 + b], p->Z, st));
    }
    return SID_OK;
}

// LS_deconv (plain mode, LS_deconv.m:72-93) for nb volumes: the projections
// go through the batched forms, the per-volume scalars (step sizes) through
// one reduction per volume.  lamb_L1: nb values (host), one per volume.
extern "C" int sid_deconv_ls_batched(sid_plan* p, int method, int64_t nb, float* const* X, int max_iter,
                                     const float* lamb_L1, float lamb_L2, void* stream)
{
    SID_REQUIRE(p && X && lamb_L1, "sid_deconv_ls_batched: NULL argument");
    SID_REQUIRE(nb >= 1 && max_iter >= 0, "sid_deconv_ls_batched: need nb >= 1 and max_iter >= 0");
    for (int64_t b = 0; b < nb; ++b) SID_REQUIRE(X[b], "sid_deconv_ls_batched: volume %lld is NULL", (long long)b);
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t n = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    const int64_t g = vol_group(p, method, nb);
    for (int k = 0; k < 3; ++k) SID_TRY(p->ws[k].alloc((size_t)(g * n) * sizeof(float)));
    SID_TRY(p->ws[4].alloc((size_t)(g * n) * sizeof(float)));   // back projections
    SID_TRY(p->ws[5].alloc((size_t)(g * ni) * sizeof(float)));  // images
    SID_TRY(p->red.alloc((size_t)(kRedBlocks + 4 * g + 8) * sizeof(double)));
    float* xp = p->ws[0].as<float>();
    float* dp = p->ws[1].as<float>();
    float* tp = p->ws[2].as<float>();
    float* bp = p->ws[4].as<float>();
    float* ip = p->ws[5].as<float>();
    double* red = p->red.as<double>();
    double* s12 = red + kRedBlocks;                            // two scalars per volume
    float* alpha = reinterpret_cast<float*>(s12 + 2 * g);      // one step size per volume
    for (int64_t b0 = 0; b0 < nb; b0 += g) {
        const int m = (int)std::min<int64_t>(g, nb - b0);
        for (int b = 0; b < m; ++b) SID_TRY(v_to_vp(p, X[b0 + b], xp + b * n, p->Z, st));
        // df = Q(x0) - x0 + lamb_L1 with x0 = df
        SID_TRY(fwd_poly_batch(p, method, xp, ip, m, st));
        SID_TRY(adj_poly_batch(p, method, ip, bp, m, st));
        for (int b = 0; b < m; ++b)
            k_ls_init<<<2048, 256, 0, st>>>(dp + b * n, bp + b * n, xp + b * n, lamb_L1[b0 + b], lamb_L2, n);
        SID_CHECK_LAUNCH();
        SID_TRY(mask_vp(p, dp, m * p->Z, st));
        for (int it = 0; it < max_iter; ++it) {
            k_ls_passive<<<2048, 256, 0, st>>>(xp, dp, tp, m * n);
            SID_CHECK_LAUNCH();
            for (int b = 0; b < m; ++b) SID_TRY(dot(tp + b * n, tp + b * n, n, red, s12 + 2 * b, st));
            SID_TRY(fwd_poly_batch(p, method, tp, ip, m, st));
            for (int b = 0; b < m; ++b)
                SID_TRY(dot(ip + b * ni, ip + b * ni, ni, red, s12 + 2 * b + 1, st, s12 + 2 * b, alpha + b));
            for (int b = 0; b < m; ++b) k_ls_step<<<2048, 256, 0, st>>>(xp + b * n, tp + b * n, alpha + b, n);
            SID_CHECK_LAUNCH();
            SID_TRY(fwd_poly_batch(p, method, tp, ip, m, st));
            SID_TRY(adj_poly_batch(p, method, ip, bp, m, st));
            k_ls_grad<<<2048, 256, 0, st>>>(dp, bp, tp, lamb_L2, m * n);
            SID_CHECK_LAUNCH();
        }
        for (int b = 0; b < m; ++b) SID_TRY(vp_to_v(p, xp + b * n, X[b0 + b], p->Z, st));
    }
    return SID_OK;
}

extern "C" int sid_forward_batched(sid_plan* p, int method, int64_t nb, const float* const* V, float* const* I,
                                   void* stream)
{
    SID_REQUIRE(p && V && I && nb >= 1, "sid_forward_batched: NULL argument or empty batch");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t nv = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    const int64_t g = vol_group(p, method, nb);
    SID_TRY(p->ws[0].alloc((size_t)(g * nv) * sizeof(float)));
    SID_TRY(p->ws[5].alloc((size_t)(g * ni) * sizeof(float)));
    for (int64_t b0 = 0; b0 < nb; b0 += g) {
        const int n = (int)std::min<int64_t>(g, nb - b0);
        for (int b = 0; b < n; ++b) SID_TRY(v_to_vp(p, V[b0 + b], p->ws[0].as<float>() + b * nv, p->Z, st));
        SID_TRY(fwd_poly_batch(p, method, p->ws[0].as<float>(), p->ws[5].as<float>(), n, st));
        for (int b = 0; b < n; ++b) SID_TRY(vp_to_v(p, p->ws[5].as<float>() + b * ni, I[b0 + b], 1, st));
    }
    return SID_OK;
}

extern "C" int sid_adjoint_batched(sid_plan* p, int method, int64_t nb, const float* const* I, float* const* V,
                                   void* stream)
{
    SID_REQUIRE(p && V && I && nb >= 1, "sid_adjoint_batched: NULL argument or empty batch");
    cudaStream_t st = as_stream(stream);
    SID_TRY(ensure_proj_ws(p));
    const int64_t nv = vol_plane_elems(p) * p->Z, ni = vol_plane_elems(p);
    const int64_t g = vol_group(p, method, nb);
    SID_TRY(p->ws[4].alloc((size_t)(g * nv) * sizeof(float)));
    SID_TRY(p->ws[5].alloc((size_t)(g * ni) * sizeof(float)));
    for (int64_t b0 = 0; b0 < nb; b0 += g) {
        const int n = (int)std::min<int64_t>(g, nb - b0);
        for (int b = 0; b < n; ++b) SID_TRY(v_to_vp(p, I[b0 + b], p->ws[5].as<float>() + b * ni, 1, st));
        SID_TRY(adj_poly_batch(p, method, p->ws[5].as<float>(), p->ws[4].as<float>(), n, st));
        for (int b = 0; b < n; ++b) SID_TRY(vp_to_v(p, p->ws[4].as<float>() + b * nv, V[b0 + b], p->Z, st));
    }
    return SID_OK;
}

extern "C" int sid_plan_sync(sid_plan* p, void* stream)
{
    SID_REQUIRE(p, "sid_plan_sync: NULL plan");
    return plan_sync(p, as_stream(stream));
}

extern "C" int sid_deconv_isra_host(sid_plan* p, int method, const float* Htf, float* X, int maxIter,
                                    float lambda)
{
    SID_REQUIRE(p && Htf && X, "sid_deconv_isra_host: NULL argument");
    SID_REQUIRE(maxIter >= 0, "sid_deconv_isra_host: maxIter < 0");
    const size_t n = (size_t)(p->X * p->Y * p->Z);
    DBuf& dh = p->ws[4];
    SID_TRY(dh.alloc(n * sizeof(float)));
    float* xv = static_cast<float*>(host_device_view(X));
    if (!xv) {
        DBuf& dx = p->ws[5];
        SID_TRY(dx.alloc(n * sizeof(float)));
        SID_CUDA_TRY(cudaMemcpy(dh.p, Htf, n * sizeof(float), cudaMemcpyHostToDevice));
        SID_CUDA_TRY(cudaMemcpy(dx.p, X, n * sizeof(float), cudaMemcpyHostToDevice));
        SID_TRY(sid_deconv_isra(p, method, dh.as<float>(), dx.as<float>(), maxIter, lambda, nullptr));
        SID_TRY(plan_sync(p, 0));
        SID_CUDA_TRY(cudaMemcpy(X, dx.p, n * sizeof(float), cudaMemcpyDeviceToHost));
        return SID_OK;
    }
    // X crosses the host link inside its layout conversion; Htf (needed first by
    // the update) crosses on a copy engine while the first projections run; the
    // result is written back by the inverse conversion.
    cudaStream_t st, side;
    SID_TRY(host_streams(p, &st, &side));
    SID_TRY(ensure_proj_ws(p));
    const int64_t nv = vol_plane_elems(p) * p->Z;
    SID_TRY(p->ws[0].alloc((size_t)nv * sizeof(float)));
    SID_TRY(p->ws[1].alloc((size_t)nv * sizeof(float)));
    float* xp = p->ws[0].as<float>();
    float* hp = p->ws[1].as<float>();
    SID_TRY(v_to_vp(p, xv, xp, p->Z, st));
    SID_CUDA_TRY(cudaEventRecord(p->hevent[0], st));
    for (int it = 0; it < maxIter; ++it) {
        SID_TRY(fwd_poly(p, method, xp, p->ip.as<float>(), st));
        SID_TRY(adj_poly(p, method, p->ip.as<float>(), p->bp.as<float>(), st));
        if (it == 0) {
            SID_CUDA_TRY(cudaStreamWaitEvent(side, p->hevent[0], 0));
            SID_CUDA_TRY(cudaMemcpyAsync(dh.p, Htf, n * sizeof(float), cudaMemcpyHostToDevice, side));
            SID_TRY(v_to_vp(p, dh.as<float>(), hp, p->Z, side));
            SID_CUDA_TRY(cudaEventRecord(p->hevent[1], side));
            SID_CUDA_TRY(cudaStreamWaitEvent(st, p->hevent[1], 0));
        }
        SID_TRY(isra_update(p, xp, hp, lambda, st));
    }
    SID_TRY(vp_to_v(p, xp, xv, p->Z, st));
    return plan_sync(p, st);
}
