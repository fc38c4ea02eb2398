// direct.cu -- FP32 direct lenslet-structured projector (the plain path).
//
// forwardProjectACC.m:14-29 writes the projection as N*N*Z full-frame 2-D
// convolutions of a zero-filled lattice image.  Only every N-th voxel of each
// lattice image is non-zero, so the same sum is a multichannel convolution on
// the lenslet grid (channels abc = N*N*Z, outputs b'a' = N*N, D x D taps):
//   Ip[b'a'](s,t) = sum_abc sum_m Vp[abc](s-m1-dlo, t-m2-dlo) K[abc][b'a'](m1,m2)
// Kernel design (one CTA = one output phase row b', all N phases a' (one warp
// each), a 32 x R tile of lenslets, one depth range):
//   * per slice (c,b,a) the N tap arrays of that slice are staged into shared
//     memory by one TMA bulk copy (cp.async.bulk + mbarrier), the lattice
//     window of the input channel by cp.async with zero fill; two stages are
//     in flight so the copies of slice i+1 overlap the FMAs of slice i;
//   * lanes own 32 consecutive lenslets along u, registers own R consecutive
//     lenslets along v; a window column of R+D-1 values is held in registers
//     and swept against the D taps of one tap row (R FMAs per tap load).
// The adjoint (backwardProjectACC_new.m:14-26) is the transposed sum with the
// roles of (abc) and (b'a') exchanged and the window sliding the other way.
#include <algorithm>

#include "ptx.cuh"
#include "sid_internal.cuh"

namespace sid {

// ---------------------------------------------------------------- layouts --
// Vp[c][b][a][v][u] <- V(a+N*u, b+N*v, c); zero outside X x Y.  V may be a
// caller's host array (device view).  One CTA per (kLayoutRows lattice rows v,
// input row phase b, depth c): it reads the rows y = b + N v (contiguous) into
// shared memory and writes, per column phase a, the rows' lattice points as
// one contiguous run of kLayoutRows x Lx values.
constexpr int kLayoutRows = 8;
constexpr int kLayoutBatch = 4;  // loads per row and thread kept in flight

__global__ void __launch_bounds__(256)
k_v_to_vp(const float* __restrict__ V, float* __restrict__ Vp, int64_t X, int64_t Y, int N, int Lx, int Ly)
{
    extern __shared__ float s[];  // [kLayoutRows][N * Lx]
    const int v0 = blockIdx.x * kLayoutRows, b = blockIdx.y, c = blockIdx.z;
    const int W = N * Lx;
    const int nr = min(kLayoutRows, Ly - v0);
    // all rows' loads of a column block are issued before any is stored (the
    // source may sit across the host link: many requests in flight per thread)
    for (int x0 = 0; x0 < W; x0 += kLayoutBatch * blockDim.x) {
        float t[kLayoutRows][kLayoutBatch];
#pragma unroll
        for (int r = 0; r < kLayoutRows; ++r) {
            const int64_t y = b + (int64_t)N * (v0 + r);
            const float* row = V + X * (y + Y * c);
#pragma unroll
            for (int k = 0; k < kLayoutBatch; ++k) {
                const int x = x0 + threadIdx.x + k * blockDim.x;
                t[r][k] = (r < nr && y < Y && x < X) ? row[x] : 0.f;
            }
        }
#pragma unroll
        for (int r = 0; r < kLayoutRows; ++r)
#pragma unroll
            for (int k = 0; k < kLayoutBatch; ++k) {
                const int x = x0 + threadIdx.x + k * blockDim.x;
                if (r < nr && x < W) s[r * W + x] = t[r][k];
            }
    }
    __syncthreads();
    const int64_t plane = (int64_t)Ly * Lx;
    const int run = nr * Lx;
    for (int a = 0; a < N; ++a) {
        float* dst = Vp + (((int64_t)c * N + b) * N + a) * plane + (int64_t)v0 * Lx;
        for (int e = threadIdx.x; e < run; e += blockDim.x) {
            const int r = e / Lx, u = e - r * Lx;
            dst[e] = s[r * W + a + N * u];
        }
    }
}

// V(x,y,c) <- Vp (x < X, y < Y).  V may be a caller's host array (device
// view): each CTA writes one contiguous row.
__global__ void k_vp_to_v(const float* __restrict__ Vp, float* __restrict__ V, int64_t X, int64_t Y,
                          int N, int Lx, int Ly)
{
    extern __shared__ float s[];
    const int y = blockIdx.x;  // 0 .. Y-1
    const int c = blockIdx.y;
    const int b = y % N, v = y / N;
    const int W = N * Lx;
    const int64_t plane = (int64_t)Ly * Lx;
    for (int idx = threadIdx.x; idx < W; idx += blockDim.x) {
        const int a = idx / Lx, u = idx - a * Lx;
        s[a + N * u] = Vp[(((int64_t)c * N + b) * N + a) * plane + (int64_t)v * Lx + u];
    }
    __syncthreads();
    for (int x = threadIdx.x; x < X; x += blockDim.x) V[x + X * ((int64_t)y + Y * c)] = s[x];
}

// Sum the depth-split partial images and zero the lattice positions that fall
// outside the X x Y sensor (x = a'+N*s >= X or y = b'+N*t >= Y).
__global__ void k_reduce_parts(const float* __restrict__ parts, float* __restrict__ Ip, int nparts,
                               int64_t part_stride, int N, int Lx, int Ly, int64_t X, int64_t Y)
{
    const int64_t n = (int64_t)N * N * Ly * Lx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(i % Lx);
        int64_t r = i / Lx;
        const int t = (int)(r % Ly);
        r /= Ly;
        const int ap = (int)(r % N), bp = (int)(r / N);
        float acc = 0.f;
        if (ap + (int64_t)N * s < X && bp + (int64_t)N * t < Y)
            for (int z = 0; z < nparts; ++z) acc += parts[z * part_stride + i];
        Ip[i] = acc;
    }
}

// Zero the padded lattice positions of a polyphase volume (x >= X or y >= Y).
__global__ void k_mask_vp(float* __restrict__ Vp, int N, int Z, int Lx, int Ly, int64_t X, int64_t Y)
{
    const int64_t n = (int64_t)Z * N * N * Ly * Lx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int u = (int)(i % Lx);
        int64_t r = i / Lx;
        const int v = (int)(r % Ly);
        r /= Ly;
        const int a = (int)(r % N);
        const int b = (int)((r / N) % N);
        if (a + (int64_t)N * u >= X || b + (int64_t)N * v >= Y) Vp[i] = 0.f;
    }
}

// --------------------------------------------------------- direct forward --
template <int R, int D>
__global__ void __launch_bounds__(480, 2)
k_fwd_direct(const float* __restrict__ Vp, const float* __restrict__ taps, float* __restrict__ parts,
             int N, int Z, int Lx, int Ly, int dhi, int64_t tbs, int zper, int64_t part_stride,
             int* __restrict__ err)
{
    constexpr int WR = 32 + D - 1;  // window extent along u (lanes)
    constexpr int WQ = R + D - 1;   // window extent along v (registers)
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) uint64_t bar[2];
    const int TB = (int)tbs;
    float* Tb = smem;            // [2][TB]
    float* Wb = smem + 2 * TB;   // [2][WQ*WR]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // warp = a'
    const int bp = blockIdx.z % N, zs = blockIdx.z / N;
    const int s0 = blockIdx.x * 32, t0 = blockIdx.y * R;
    const int c0 = zs * zper, c1 = min(Z, c0 + zper);
    const int nsl = (c1 - c0) * N * N;
    const int64_t plane = (int64_t)Ly * Lx;
    const uint32_t tbytes = (uint32_t)(N * D * D) * 4u;
    const uint32_t tbytes16 = (tbytes + 15u) & ~15u;

    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int i, int buf) {
        const int c = c0 + i / (N * N);
        const int rem = i - (c - c0) * N * N;
        const int b = rem / N, a = rem - (rem / N) * N;
        const int64_t ch = ((int64_t)c * N + b) * N + a;
        if (threadIdx.x == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf], tbytes16);
            bulk_g2s(Tb + buf * TB, taps + (ch * N + bp) * tbs, tbytes16, &bar[buf]);
        }
        const float* src = Vp + ch * plane;
        float* dst = Wb + buf * (WQ * WR);
        for (int e = threadIdx.x; e < WQ * WR; e += blockDim.x) {
            const int q = e / WR, r = e - (e / WR) * WR;
            const int u = s0 - dhi + r, v = t0 - dhi + q;
            const bool ok = (u >= 0) && (u < Lx) && (v >= 0) && (v < Ly);
            cp_async4(dst + e, ok ? (src + (int64_t)v * Lx + u) : src, ok);
        }
        cp_async_commit();
    };

    float acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0.f;

    bool alive = true;
    if (nsl > 0) issue(0, 0);
    for (int i = 0; i < nsl && alive; ++i) {
        const int buf = i & 1;
        if (i + 1 < nsl) issue(i + 1, buf ^ 1);
        else cp_async_commit();
        cp_async_wait<1>();
        // every thread waits; the CTA agrees on the outcome before going on
        alive = !__syncthreads_or(!mbar_wait(&bar[buf], (uint32_t)((i >> 1) & 1), err));
        if (alive) {
            const float* T = Tb + buf * TB + warp * D * D;
            const float* W = Wb + buf * (WQ * WR);
            // two-level sum: a slice's D*D taps into `part`, slices into `acc`
            float part[R];
#pragma unroll
            for (int k = 0; k < R; ++k) part[k] = 0.f;
#pragma unroll 1
            for (int m1 = 0; m1 < D; ++m1) {
                const int r = lane + (D - 1 - m1);
                float col[WQ];
#pragma unroll
                for (int q = 0; q < WQ; ++q) col[q] = W[q * WR + r];
#pragma unroll
                for (int m2 = 0; m2 < D; ++m2) {
                    const float h = T[m1 * D + m2];
#pragma unroll
                    for (int k = 0; k < R; ++k) part[k] = fmaf(h, col[k + D - 1 - m2], part[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < R; ++k) acc[k] += part[k];
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    const int s = s0 + lane;
    if (s < Lx) {
        float* out = parts + zs * part_stride + ((int64_t)bp * N + warp) * plane + s;
#pragma unroll
        for (int k = 0; k < R; ++k)
            if (t0 + k < Ly) out[(int64_t)(t0 + k) * Lx] = acc[k];
    }
}

// --------------------------------------------------------- direct adjoint --
template <int R, int D>
__global__ void __launch_bounds__(480, 2)
k_adj_direct(const float* __restrict__ Ip, const float* __restrict__ taps, float* __restrict__ Bp,
             int N, int Lx, int Ly, int dlo, int64_t tbs, int64_t X, int64_t Y, int* __restrict__ err)
{
    constexpr int WR = 32 + D - 1;
    constexpr int WQ = R + D - 1;
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) uint64_t bar[2];
    const int TB = (int)tbs;
    float* Tb = smem;
    float* Wb = smem + 2 * TB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // warp = a
    const int u0 = blockIdx.x * 32, v0 = blockIdx.y * R;
    const int b = blockIdx.z % N, c = blockIdx.z / N;
    const int nsl = N * N;
    const int64_t plane = (int64_t)Ly * Lx;
    const uint32_t tbytes = (uint32_t)(N * D * D) * 4u;
    const uint32_t tbytes16 = (tbytes + 15u) & ~15u;

    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int i, int buf) {
        const int bpi = i / N, api = i - (i / N) * N;  // input phase (b', a')
        if (threadIdx.x == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf], tbytes16);
            const int64_t blk = (((int64_t)c * N + b) * N + bpi) * N + api;
            bulk_g2s(Tb + buf * TB, taps + blk * tbs, tbytes16, &bar[buf]);
        }
        const float* src = Ip + ((int64_t)bpi * N + api) * plane;
        float* dst = Wb + buf * (WQ * WR);
        for (int e = threadIdx.x; e < WQ * WR; e += blockDim.x) {
            const int q = e / WR, r = e - (e / WR) * WR;
            const int s = u0 + dlo + r, t = v0 + dlo + q;
            const bool ok = (s >= 0) && (s < Lx) && (t >= 0) && (t < Ly);
            cp_async4(dst + e, ok ? (src + (int64_t)t * Lx + s) : src, ok);
        }
        cp_async_commit();
    };

    float acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0.f;
    bool alive = true;
    issue(0, 0);
    for (int i = 0; i < nsl && alive; ++i) {
        const int buf = i & 1;
        if (i + 1 < nsl) issue(i + 1, buf ^ 1);
        else cp_async_commit();
        cp_async_wait<1>();
        // every thread waits; the CTA agrees on the outcome before going on
        alive = !__syncthreads_or(!mbar_wait(&bar[buf], (uint32_t)((i >> 1) & 1), err));
        if (alive) {
            const float* T = Tb + buf * TB + warp * D * D;
            const float* W = Wb + buf * (WQ * WR);
            float part[R];
#pragma unroll
            for (int k = 0; k < R; ++k) part[k] = 0.f;
#pragma unroll 1
            for (int m1 = 0; m1 < D; ++m1) {
                const int r = lane + m1;
                float col[WQ];
#pragma unroll
                for (int q = 0; q < WQ; ++q) col[q] = W[q * WR + r];
#pragma unroll
                for (int m2 = 0; m2 < D; ++m2) {
                    const float h = T[m1 * D + m2];
#pragma unroll
                    for (int k = 0; k < R; ++k) part[k] = fmaf(h, col[k + m2], part[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < R; ++k) acc[k] += part[k];
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    const int u = u0 + lane;
    if (u < Lx) {
        const bool xin = (warp + (int64_t)N * u) < X;
        float* out = Bp + (((int64_t)c * N + b) * N + warp) * plane + u;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int v = v0 + k;
            if (v < Ly) out[(int64_t)v * Lx] = (xin && (b + (int64_t)N * v) < Y) ? acc[k] : 0.f;
        }
    }
}

// ------------------------------------------- generic-D kernels (any size) --
// One output per thread, taps and inputs read through the cache.  Used when
// the tap count D has no specialised instantiation.
__global__ void k_fwd_generic(const float* __restrict__ Vp, const float* __restrict__ taps,
                              float* __restrict__ Ip, int N, int Z, int Lx, int Ly, int dlo, int D,
                              int64_t tbs, int64_t X, int64_t Y)
{
    const int64_t n = (int64_t)N * N * Ly * Lx;
    const int64_t plane = (int64_t)Ly * Lx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(i % Lx);
        int64_t r = i / Lx;
        const int t = (int)(r % Ly);
        r /= Ly;
        const int ap = (int)(r % N), bp = (int)(r / N);
        float acc = 0.f;
        if (ap + (int64_t)N * s < X && bp + (int64_t)N * t < Y) {
            for (int c = 0; c < Z; ++c)
                for (int b = 0; b < N; ++b)
                    for (int a = 0; a < N; ++a) {
                        const int64_t ch = ((int64_t)c * N + b) * N + a;
                        const float* T = taps + (ch * N + bp) * tbs + (int64_t)ap * D * D;
                        const float* src = Vp + ch * plane;
                        for (int m1 = 0; m1 < D; ++m1) {
                            const int u = s - m1 - dlo;
                            if (u < 0 || u >= Lx) continue;
                            for (int m2 = 0; m2 < D; ++m2) {
                                const int v = t - m2 - dlo;
                                if (v < 0 || v >= Ly) continue;
                                acc = fmaf(T[m1 * D + m2], src[(int64_t)v * Lx + u], acc);
                            }
                        }
                    }
        }
        Ip[i] = acc;
    }
}

__global__ void k_adj_generic(const float* __restrict__ Ip, const float* __restrict__ taps,
                              float* __restrict__ Bp, int N, int Z, int Lx, int Ly, int dlo, int D,
                              int64_t tbs, int64_t X, int64_t Y)
{
    const int64_t plane = (int64_t)Ly * Lx;
    const int64_t n = (int64_t)Z * N * N * plane;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int u = (int)(i % Lx);
        int64_t r = i / Lx;
        const int v = (int)(r % Ly);
        r /= Ly;
        const int a = (int)(r % N);
        r /= N;
        const int b = (int)(r % N), c = (int)(r / N);
        float acc = 0.f;
        if (a + (int64_t)N * u < X && b + (int64_t)N * v < Y) {
            for (int bp = 0; bp < N; ++bp)
                for (int ap = 0; ap < N; ++ap) {
                    const int64_t blk = (((int64_t)c * N + b) * N + bp) * N + ap;
                    const float* T = taps + blk * tbs + (int64_t)a * D * D;
                    const float* src = Ip + ((int64_t)bp * N + ap) * plane;
                    for (int m1 = 0; m1 < D; ++m1) {
                        const int s = u + m1 + dlo;
                        if (s < 0 || s >= Lx) continue;
                        for (int m2 = 0; m2 < D; ++m2) {
                            const int t = v + m2 + dlo;
                            if (t < 0 || t >= Ly) continue;
                            acc = fmaf(T[m1 * D + m2], src[(int64_t)t * Lx + s], acc);
                        }
                    }
                }
        }
        Bp[i] = acc;
    }
}

// ------------------------------------------------------------ dispatchers --
static int pick_R(int64_t Ly)
{
    const int cand[3] = {16, 12, 8};
    int best = 8;
    int64_t bestw = INT64_MAX;
    for (int R : cand) {
        const int64_t w = cdiv(Ly, R) * R;
        if (w < bestw) { bestw = w; best = R; }
    }
    return best;
}

template <int R, int D>
static int launch_fwd(sid_plan* p, const float* vp, float* parts, int zsplit, int zper, int64_t tbs,
                      int* err, cudaStream_t st)
{
    constexpr int WQ = R + D - 1, WR = 32 + D - 1;
    const size_t smem = (size_t)(2 * tbs + 2 * WQ * WR) * sizeof(float);
    SID_TRY(smem_attr((const void*)k_fwd_direct<R, D>, smem));  // smem depends on the plan's Nnum
    dim3 grid((unsigned)cdiv(p->Lx, 32), (unsigned)cdiv(p->Ly, R), (unsigned)(p->N * zsplit));
    const int64_t part_stride = p->N * p->N * p->Ly * p->Lx;
    p->timer.begin(st);
    k_fwd_direct<R, D><<<grid, (unsigned)(32 * p->N), smem, st>>>(
        vp, p->taps_f.as<float>(), parts, (int)p->N, (int)p->Z, (int)p->Lx, (int)p->Ly, (int)p->g.dhi,
        tbs, zper, part_stride, err);
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

template <int R, int D>
static int launch_adj(sid_plan* p, const float* ip, float* bp, int64_t tbs, int* err, cudaStream_t st)
{
    constexpr int WQ = R + D - 1, WR = 32 + D - 1;
    const size_t smem = (size_t)(2 * tbs + 2 * WQ * WR) * sizeof(float);
    SID_TRY(smem_attr((const void*)k_adj_direct<R, D>, smem));
    dim3 grid((unsigned)cdiv(p->Lx, 32), (unsigned)cdiv(p->Ly, R), (unsigned)(p->N * p->Z));
    p->timer.begin(st);
    k_adj_direct<R, D><<<grid, (unsigned)(32 * p->N), smem, st>>>(
        ip, p->taps_b.as<float>(), bp, (int)p->N, (int)p->Lx, (int)p->Ly, (int)p->g.dlo, tbs, p->X, p->Y,
        err);
    p->timer.finish(st);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Specialised kernels: tap count 15 or 25 and at most 15 warps (Nnum <= 15),
// the block size their launch bounds were compiled for.
static bool specialised(const sid_plan* p) { return (p->g.D == 15 || p->g.D == 25) && p->N <= 15; }

// Polyphase volume -> polyphase (masked) image.
int direct_forward(sid_plan* p, const float* vp, float* ip, int* err, cudaStream_t st)
{
    SID_REQUIRE(p->taps_f.p, "direct projector: plan has no FP32 taps (build with SID_PLAN_DIRECT)");
    const int64_t tbs = cdiv(p->N * p->g.D * p->g.D, 32) * 32;
    const int64_t plane = p->N * p->N * p->Ly * p->Lx;
    if (!specialised(p)) {
        k_fwd_generic<<<1024, 256, 0, st>>>(vp, p->taps_f.as<float>(), ip, (int)p->N, (int)p->Z, (int)p->Lx,
                                            (int)p->Ly, (int)p->g.dlo, (int)p->g.D, tbs, p->X, p->Y);
        SID_CHECK_LAUNCH();
        return SID_OK;
    }
    const int R = pick_R(p->Ly);
    // depth split: enough CTAs for ~8 waves of 2 CTAs per SM on 152 SMs
    const int64_t base = cdiv(p->Lx, 32) * cdiv(p->Ly, R) * p->N;
    int zsplit = (int)std::min<int64_t>(p->Z, std::max<int64_t>(1, cdiv(152 * 2 * 8, base)));
    const int zper = (int)cdiv(p->Z, zsplit);
    zsplit = (int)cdiv(p->Z, zper);
    SID_TRY(p->ipart.alloc((size_t)(zsplit * plane) * sizeof(float)));
    int rc = SID_EINVAL;
    switch (p->g.D * 100 + R) {
    case 1516: rc = launch_fwd<16, 15>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    case 1512: rc = launch_fwd<12, 15>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    case 1508: rc = launch_fwd<8, 15>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    case 2516: rc = launch_fwd<16, 25>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    case 2512: rc = launch_fwd<12, 25>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    case 2508: rc = launch_fwd<8, 25>(p, vp, p->ipart.as<float>(), zsplit, zper, tbs, err, st); break;
    default: set_error("direct projector: no kernel for D=%lld R=%d", (long long)p->g.D, R); return SID_EINVAL;
    }
    SID_TRY(rc);
    k_reduce_parts<<<1024, 256, 0, st>>>(p->ipart.as<float>(), ip, zsplit, plane, (int)p->N, (int)p->Lx,
                                         (int)p->Ly, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// Polyphase image -> polyphase volume (zero at padded lattice positions).
int direct_adjoint(sid_plan* p, const float* ip, float* bp, int* err, cudaStream_t st)
{
    SID_REQUIRE(p->taps_b.p, "direct projector: plan has no FP32 adjoint taps (build with SID_PLAN_DIRECT)");
    const int64_t tbs = cdiv(p->N * p->g.D * p->g.D, 32) * 32;
    if (!specialised(p)) {
        k_adj_generic<<<2048, 256, 0, st>>>(ip, p->taps_b.as<float>(), bp, (int)p->N, (int)p->Z, (int)p->Lx,
                                            (int)p->Ly, (int)p->g.dlo, (int)p->g.D, tbs, p->X, p->Y);
        SID_CHECK_LAUNCH();
        return SID_OK;
    }
    const int R = pick_R(p->Ly);
    switch (p->g.D * 100 + R) {
    case 1516: return launch_adj<16, 15>(p, ip, bp, tbs, err, st);
    case 1512: return launch_adj<12, 15>(p, ip, bp, tbs, err, st);
    case 1508: return launch_adj<8, 15>(p, ip, bp, tbs, err, st);
    case 2516: return launch_adj<16, 25>(p, ip, bp, tbs, err, st);
    case 2512: return launch_adj<12, 25>(p, ip, bp, tbs, err, st);
    case 2508: return launch_adj<8, 25>(p, ip, bp, tbs, err, st);
    default: break;
    }
    set_error("direct projector: no kernel for D=%lld R=%d", (long long)p->g.D, R);
    return SID_EINVAL;
}

// Layout launchers.
static int layout_launch_check(const sid_plan* p, int64_t Z, size_t* smem)
{
    *smem = (size_t)(kLayoutRows * p->N * p->Lx) * sizeof(float);
    SID_REQUIRE(*smem <= 200 * 1024, "volume layout: rows of %lld lenslets x %lld too long", (long long)p->Lx,
                (long long)p->N);
    SID_REQUIRE(Z <= 65535, "volume layout: %lld depths above the grid limit", (long long)Z);
    return SID_OK;
}

int v_to_vp(const sid_plan* p, const float* V, float* vp, int64_t Z, cudaStream_t st)
{
    size_t sm = 0;
    SID_TRY(layout_launch_check(p, Z, &sm));
    SID_TRY(smem_attr((const void*)k_v_to_vp, sm));
    dim3 grid((unsigned)cdiv(p->Ly, kLayoutRows), (unsigned)p->N, (unsigned)Z);
    k_v_to_vp<<<grid, 256, sm, st>>>(V, vp, p->X, p->Y, (int)p->N, (int)p->Lx, (int)p->Ly);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int vp_to_v(const sid_plan* p, const float* vp, float* V, int64_t Z, cudaStream_t st)
{
    SID_REQUIRE(Z <= 65535, "volume layout: %lld depths above the grid limit", (long long)Z);
    dim3 grid((unsigned)p->Y, (unsigned)Z);
    k_vp_to_v<<<grid, 256, (size_t)(p->N * p->Lx) * sizeof(float), st>>>(vp, V, p->X, p->Y, (int)p->N,
                                                                          (int)p->Lx, (int)p->Ly);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

int mask_vp(const sid_plan* p, float* vp, int64_t Z, cudaStream_t st)
{
    k_mask_vp<<<1024, 256, 0, st>>>(vp, (int)p->N, (int)Z, (int)p->Lx, (int)p->Ly, p->X, p->Y);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace sid
