// library.cu -- batched LFM library generation (generate_LFM_library_GPU.m).
//
// For neuron n the reference builds a volume that is zero except for a box
// around the neuron's centre, filled with the mean of the reconstructions of
// the components it was found in, and forward-projects it with the PSF sliced
// to the box's depth window (generate_LFM_library_GPU.m:63-109).  Zero depths
// contribute nothing, so the row equals the full-depth forward projection of
// the boxed volume.  Here every neuron is one batch entry of one launch:
//   1. k_lib_average: the boxed, averaged sub-volumes (packed, one per neuron);
//   2. k_lib_project: one CTA per (group of neurons sharing a depth window,
//      output phase a'b'); threads own the output lenslets around each box; per
//      box channel (a,b,c) the D x D tap array K[abc][b'a'] is staged in shared
//      memory once for the whole group and applied to every box's lattice
//      points of that phase (the same lenslet-tap algebra as direct.cu), so
//      only the boxes' own channels are visited;
//   3. the rest of each row is zero (one memset of the output).
// Box and window arithmetic (MATLAB round, clipping at 1 and the volume size,
// ceil(neur_rad/axial)) is done on the host, bit-exact with the reference.
#include <algorithm>
#include <cmath>
#include <vector>

#include "library.cuh"

namespace sid {


// packed[b.off + (x-x0) + bw*((y-y0) + bh*(z-z0))] = mean_k recon_k(x, y, z)
__global__ void k_lib_average(const float* const* __restrict__ recon, const uint8_t* __restrict__ neur_id,
                              int64_t n_neur, const LibBox* __restrict__ boxes, int n_comp, int64_t X, int64_t Y,
                              float* __restrict__ packed)
{
    const int n = blockIdx.x;
    const LibBox b = boxes[n];
    const int bw = b.x1 - b.x0, bh = b.y1 - b.y0, bd = b.z1 - b.z0;
    const int total = bw * bh * bd;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int dx = i % bw, r = i / bw, dy = r % bh, dz = r / bh;
        const int64_t idx = (b.x0 + dx) + X * ((int64_t)(b.y0 + dy) + Y * (int64_t)(b.z0 + dz));
        float s = 0.f;
        for (int k = 0; k < n_comp; ++k)
            if (neur_id[n + n_neur * (int64_t)k]) s += recon[k][idx];
        packed[b.off + i] = s / (float)b.ncomp;
    }
}

// One CTA per (group of up to G neurons with the same depth window, output
// phase a'b'); output written to out[n * ldn + pixel * ldp] with pixel = x + X*y.
// Per depth c and input row phase b the D x D tap arrays of all N input column
// phases a are staged in shared memory once, inside a zero border of R taps
// (R = the boxes' lattice span), and applied to every neuron of the group: the
// tap arrays are the whole of the kernel's memory traffic, so grouping divides
// it by the group size.  Each thread owns four consecutive output lenslets
// (s, t..t+3) at the same place in every neuron's output window, so for every
// box lattice point (u, v) a neuron's four taps sit at one offset from the
// thread's base: one address, four shared loads and four FMAs per point, no
// range checks.  The lattice ranges of every neuron and phase are computed once
// per CTA.
constexpr int kLibT = 4;  // consecutive output lenslets per thread
constexpr int kLibG = 16;  // neurons per CTA

template <int G>
__global__ void __launch_bounds__(256)
k_lib_project(const float* __restrict__ taps, const float* __restrict__ packed, const LibBox* __restrict__ boxes,
              const int* __restrict__ groups, int N, int D, int dlo, int R, int ntgM, int64_t tbs, int Lx, int Ly,
              int64_t X, int64_t Y, float* __restrict__ out, int64_t ldn, int64_t ldp)
{
    extern __shared__ float tile[];  // [N][Dp][Dp + 4], then DD ints (padded tap offsets), then G * 4N ints (ranges)
    const int Dp = D + 2 * R, Dq = Dp + kLibT, tsz = Dp * Dq, DD = D * D;
    int* padoff = reinterpret_cast<int*>(tile + N * tsz);
    int* rng = padoff + DD;  // per neuron k: ulo[a], uhi[a], vlo[b], vhi[b] at rng + 4N k
    const int* grp = groups + blockIdx.x * (G + 1);
    const int cnt = grp[0];
    const int o = blockIdx.y;  // b'*N + a'
    const int bp = o / N, ap = o - (o / N) * N;
    for (int i = threadIdx.x; i < N * tsz; i += blockDim.x) tile[i] = 0.f;
    for (int r = threadIdx.x; r < DD; r += blockDim.x) padoff[r] = (r / D + R) * Dq + (r - (r / D) * D) + R;
    for (int e = threadIdx.x; e < cnt * N; e += blockDim.x) {
        // lattice columns u of phase ph in box k: x = ph + N u in [x0, x1); rows likewise
        const int k = e / N, ph = e - k * N;
        const LibBox b = boxes[grp[1 + k]];
        int* rk = rng + 4 * N * k;
        rk[ph] = (b.x0 - ph) > 0 ? (b.x0 - ph + N - 1) / N : 0;
        rk[N + ph] = (b.x1 - 1 - ph) >= 0 ? (b.x1 - 1 - ph) / N : -1;
        rk[2 * N + ph] = (b.y0 - ph) > 0 ? (b.y0 - ph + N - 1) / N : 0;
        rk[3 * N + ph] = (b.y1 - 1 - ph) >= 0 ? (b.y1 - 1 - ph) / N : -1;
    }
    const int g = threadIdx.x;
    const int ls = g / ntgM, lt = (g - (g / ntgM) * ntgM) * kLibT;
    const int base = (ls + R) * Dq + (lt + R);
    float acc[G][kLibT];
#pragma unroll
    for (int k = 0; k < G; ++k)
#pragma unroll
        for (int q = 0; q < kLibT; ++q) acc[k][q] = 0.f;
    const LibBox b0 = boxes[grp[1]];  // every neuron of the group has this depth window
    __syncthreads();
    for (int c = b0.z0; c < b0.z1; ++c) {
        for (int bb = 0; bb < N; ++bb) {
            __syncthreads();  // the previous row's taps are no longer read
            const int64_t rowblk = ((int64_t)c * N + bb) * N;
            for (int a = 0; a < N; ++a) {
                const float* src = taps + ((rowblk + a) * N + bp) * tbs + (int64_t)ap * DD;
                float* dst = tile + a * tsz;
                for (int r = threadIdx.x; r < DD; r += blockDim.x) dst[padoff[r]] = src[r];
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < G; ++k) {
                if (k >= cnt) break;
                const LibBox b = boxes[grp[1 + k]];
                const int* rk = rng + 4 * N * k;
                const int vlo = rk[2 * N + bb], vhi = rk[3 * N + bb];
                if (vhi < vlo || ls >= b.s1 - b.s0 || lt >= b.t1 - b.t0) continue;
                const int bw = b.x1 - b.x0, bh = b.y1 - b.y0;
                for (int a = 0; a < N; ++a) {
                    const int ulo = rk[a], uhi = rk[N + a];
                    if (uhi < ulo) continue;
                    const float* ta = tile + a * tsz + base;
                    for (int v = vlo; v <= vhi; ++v) {
                        const int e2 = b.t0 - v - dlo;
                        const float* prow = packed + b.off + bw * ((bb + N * v - b.y0) + bh * (c - b.z0)) - b.x0 + a;
                        for (int u = ulo; u <= uhi; ++u) {
                            const float val = prow[N * u];
                            const float* tp = ta + (b.s0 - u - dlo) * Dq + e2;
#pragma unroll
                            for (int q = 0; q < kLibT; ++q) acc[k][q] = fmaf(val, tp[q], acc[k][q]);
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
        if (k >= cnt) break;
        const int n = grp[1 + k];
        const LibBox b = boxes[n];
        if (ls >= b.s1 - b.s0 || lt >= b.t1 - b.t0) continue;
        const int s = b.s0 + ls;
#pragma unroll
        for (int q = 0; q < kLibT; ++q) {
            const int t = b.t0 + lt + q;
            if (lt + q >= b.t1 - b.t0) break;
            const int64_t x = ap + (int64_t)N * s, y = bp + (int64_t)N * t;
            if (s < Lx && t < Ly && x < X && y < Y) out[(int64_t)n * ldn + (x + X * y) * ldp] = acc[k][q];
        }
    }
}

// Tiled form (the default).  One CTA per (group of up to G neurons with the
// same depth window, output phase a'b').  Every neuron's output window has the
// same shape, W rows (s) x NTB*TB columns (t) of output lenslets starting at
// (umin + dlo, vmin + dlo) with (umin, vmin) the first lenslet its box touches,
// so a box lattice point (u, v) lands at a relative offset (ru, rv) = (u -
// umin, v - vmin) in [0, span]^2 and the tap it meets at relative output (ds,
// dt) is K(ds - ru, dt - rv).  Per depth c and input row phase b the N tap
// arrays K[abc][b'a'] of all input column phases a are copied (cp.async,
// double-buffered: the next (c, b) row is in flight while this one is used)
// into zero-bordered shared tiles with an odd row pitch.  Lane = output row ds,
// so the 32 lanes of a warp read 32 different tile rows (distinct banks); each
// warp owns (neuron, block of TB output columns) pairs.  For each lattice row
// ru of a box phase, a lane loads TB + NRV - 1 consecutive taps of its tile row
// into registers once and applies them to the NRV lattice columns rv of that
// row: TB + NRV - 1 shared loads for NRV * TB FMAs, and only the boxes' own
// lattice points are visited.  TB (the template's column count, >= the
// window's width) is the whole row, so one (warp, neuron) pair covers a
// neuron's window and the per-phase bookkeeping is paid once per row.

__device__ __forceinline__ void cp_async4_lib(float* dst, const float* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

struct LibTileArgs {
    int N, D, dlo, span, W, Wt, rows, pitch, cb, tsz;
    int bwm;  // widest box (x extent) of any neuron: the staged lattice rows hold bwm floats
    int64_t tbs;
    int Lx, Ly;
    int64_t X, Y, ldn, ldp;
};

template <int G, int TB, int NRV>
__global__ void __launch_bounds__(32 * G, 16 / G)
k_lib_tile(const float* __restrict__ taps, const float* __restrict__ packed, const LibBox* __restrict__ boxes,
           const int* __restrict__ groups, const LibTileArgs a, float* __restrict__ out)
{
    constexpr int NTB = 1;
    constexpr int NWARP = G;                // one warp per neuron of the group
    constexpr int NT = 32 * NWARP;
    constexpr int PPW = (G * NTB + NWARP - 1) / NWARP;  // (neuron, column block) pairs per warp
    constexpr int RI = (768 + NT - 1) / NT;             // tap copies per thread and tile (D*D <= 768)
    constexpr int NW = TB + NRV - 1;        // taps held per lattice row
    extern __shared__ float sm[];           // 2 x N tiles of rows x pitch, 2 x G x NRV box rows, neuron tables
    const int N = a.N, D = a.D, tsz = a.tsz;
    float* vrows = sm + 2 * N * tsz;        // [buf][k][e][x - x0]: the box rows of lattice row vlo + e at (c, b)
    const int vstride = NRV * a.bwm;
    int* tab = reinterpret_cast<int*>(vrows + 2 * G * vstride);
    // per neuron k: [0] x0 [1] y0 [2] z0 [3] bw [4] bh [5] off [6] umin [7] vmin, then ulo[N], nu[N], vlo[N], nv[N]
    const int tstride = 8 + 4 * N;
    const int* grp = groups + blockIdx.x * (G + 1);
    const int cnt = grp[0];
    const int o = blockIdx.y;
    const int bp = o / N, ap = o - bp * N;
    for (int i = threadIdx.x; i < 2 * N * tsz + 2 * G * vstride; i += blockDim.x) sm[i] = 0.f;
    for (int e = threadIdx.x; e < cnt * N; e += blockDim.x) {
        const int k = e / N, ph = e - k * N;
        const LibBox b = boxes[grp[1 + k]];
        int* t = tab + k * tstride;
        if (ph == 0) {
            t[0] = b.x0; t[1] = b.y0; t[2] = b.z0; t[3] = b.x1 - b.x0; t[4] = b.y1 - b.y0; t[5] = b.off;
            t[6] = b.x0 / N; t[7] = b.y0 / N;
        }
        // lattice u of column phase ph inside [x0, x1): x = ph + N u
        const int ulo = b.x0 > ph ? (b.x0 - ph + N - 1) / N : 0;
        const int uhi = (b.x1 - 1 - ph) >= 0 ? (b.x1 - 1 - ph) / N : -1;
        const int vlo = b.y0 > ph ? (b.y0 - ph + N - 1) / N : 0;
        const int vhi = (b.y1 - 1 - ph) >= 0 ? (b.y1 - 1 - ph) / N : -1;
        t[8 + ph] = ulo;
        t[8 + N + ph] = uhi - ulo + 1;
        t[8 + 2 * N + ph] = vlo;
        t[8 + 3 * N + ph] = vhi - vlo + 1;
    }
    const int z0 = boxes[grp[1]].z0, z1 = boxes[grp[1]].z1;
    const int nst = (z1 - z0) * N;
    const int DD = D * D;
    // this thread's tap copies: r = tid + NT i, i < RI covers D*D <= 768
    int roff[RI];
#pragma unroll
    for (int i = 0; i < RI; ++i) {
        const int r = threadIdx.x + NT * i;
        roff[i] = r < DD ? (r / D + a.span) * a.pitch + (r % D) + a.cb : -1;
    }
    auto issue = [&](int st, int buf) {
        const int c = z0 + st / N, bb = st - (st / N) * N;
        const int64_t rowblk = ((int64_t)c * N + bb) * N;
        float* dst0 = sm + buf * N * tsz;
        for (int aa = 0; aa < N; ++aa) {
            const float* src = taps + ((rowblk + aa) * N + bp) * a.tbs + (int64_t)ap * DD;
#pragma unroll
            for (int i = 0; i < RI; ++i)
                if (roff[i] >= 0) cp_async4_lib(dst0 + aa * tsz + roff[i], src + threadIdx.x + NT * i);
        }
        // each neuron's box rows y = bb + N (vlo + e), e < nv, at depth c (bw contiguous floats each)
        float* vdst = vrows + buf * G * vstride;
        for (int e2 = threadIdx.x; e2 < cnt * vstride; e2 += blockDim.x) {
            const int k = e2 / vstride, r = e2 - k * vstride;
            const int e = r / a.bwm, x = r - e * a.bwm;
            const int* t = tab + k * tstride;
            if (e < t[8 + 3 * N + bb] && x < t[3]) {
                const int y = bb + N * (t[8 + 2 * N + bb] + e);
                cp_async4_lib(vdst + e2, packed + t[5] + t[3] * ((y - t[1]) + t[4] * (c - t[2])) + x);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    const int warp = threadIdx.x >> 5, ds = threadIdx.x & 31;
    float acc[PPW][TB];
#pragma unroll
    for (int q = 0; q < PPW; ++q)
#pragma unroll
        for (int j = 0; j < TB; ++j) acc[q][j] = 0.f;
    __syncthreads();  // zeroed tiles and tables before the first copies land
    issue(0, 0);
    for (int st = 0; st < nst; ++st) {
        if (st + 1 < nst) {
            issue(st + 1, (st + 1) & 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const int bb = st - (st / N) * N;  // input row phase of this stage (depth z0 + st / N)
        const float* tb0 = sm + (st & 1) * N * tsz;
        if (ds < a.W) {
#pragma unroll
            for (int q = 0; q < PPW; ++q) {
                const int pr = warp + NWARP * q;
                const int k = pr / NTB, tbk = pr - (pr / NTB) * NTB;
                if (k >= cnt) continue;
                const int* t = tab + k * tstride;
                const int nv = t[8 + 3 * N + bb];
                if (nv <= 0) continue;
                const int vlo = t[8 + 2 * N + bb], rvlo = vlo - t[7];
                // the staged box rows of this neuron: V(x, bb + N (vlo + e), c) at vk[e * bwm + x - x0]
                const float* vk = vrows + ((st & 1) * G + k) * vstride - t[0];
                const int colb = tbk * TB - rvlo - (NRV - 1) + a.cb;
                for (int aa = 0; aa < N; ++aa) {
                    const int nu = t[8 + N + aa];
                    if (nu <= 0) continue;
                    const int ulo = t[8 + aa];
                    const float* tile = tb0 + aa * tsz;
                    for (int iu = 0; iu < nu; ++iu) {
                        const int u = ulo + iu;
                        const int row = ds - (u - t[6]) + a.span;
                        const float* wp = tile + row * a.pitch + colb;
                        float w[NW];
#pragma unroll
                        for (int i = 0; i < NW; ++i) w[i] = wp[i];
                        const float* vp = vk + aa + N * u;
#pragma unroll
                        for (int e = 0; e < NRV; ++e) {
                            if (e < nv) {
                                const float val = vp[e * a.bwm];
#pragma unroll
                                for (int j = 0; j < TB; ++j) acc[q][j] = fmaf(val, w[j - e + NRV - 1], acc[q][j]);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();  // this buffer is refilled by the next-but-one copy
    }
    if (ds < a.W) {
#pragma unroll
        for (int q = 0; q < PPW; ++q) {
            const int pr = warp + NWARP * q;
            const int k = pr / NTB, tbk = pr - (pr / NTB) * NTB;
            if (k >= cnt) continue;
            const int n = grp[1 + k];
            const int* t = tab + k * tstride;
            const int s = t[6] + a.dlo + ds;
            if (s < 0 || s >= a.Lx) continue;
            const int64_t x = ap + (int64_t)N * s;
            if (x >= a.X) continue;
#pragma unroll
            for (int j = 0; j < TB; ++j) {
                const int dt = tbk * TB + j;
                const int tt = t[7] + a.dlo + dt;
                if (dt >= a.Wt || tt < 0 || tt >= a.Ly) continue;
                const int64_t y = bp + (int64_t)N * tt;
                if (y < a.Y) out[(int64_t)n * a.ldn + (x + a.X * y) * a.ldp] = acc[q][j];
            }
        }
    }
}

template <int TB, int NRV>
static int launch_lib_tile_t(dim3 grid, size_t smem, const float* taps, const float* packed, const LibBox* boxes,
                             const int* groups, const LibTileArgs& a, float* out, cudaStream_t st)
{
    SID_CUDA_TRY(cudaFuncSetAttribute(k_lib_tile<kLibG, TB, NRV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    k_lib_tile<kLibG, TB, NRV><<<grid, 32 * kLibG, smem, st>>>(taps, packed, boxes, groups, a, out);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// output window columns per lane row, as a template: the smallest of 16, 24, 28, 32 that holds Wt
static int tile_tb(int Wt) { return Wt <= 16 ? 16 : (Wt <= 24 ? 24 : (Wt <= 28 ? 28 : 32)); }

static int launch_lib_tile(int tb, int nrv, dim3 grid, size_t smem, const float* taps, const float* packed,
                           const LibBox* boxes, const int* groups, const LibTileArgs& a, float* out, cudaStream_t st)
{
#define SID_LIB_CASE(T, R) \
    if (tb == T && nrv == R) return launch_lib_tile_t<T, R>(grid, smem, taps, packed, boxes, groups, a, out, st);
    SID_LIB_CASE(16, 1) SID_LIB_CASE(16, 2) SID_LIB_CASE(16, 3)
    SID_LIB_CASE(24, 1) SID_LIB_CASE(24, 2) SID_LIB_CASE(24, 3)
    SID_LIB_CASE(28, 1) SID_LIB_CASE(28, 2) SID_LIB_CASE(28, 3)
    SID_LIB_CASE(32, 1) SID_LIB_CASE(32, 2) SID_LIB_CASE(32, 3)
#undef SID_LIB_CASE
    set_error("sid_library: no tiled kernel for %d columns x %d lattice points", tb, nrv);
    return SID_EINVAL;
}

static int mround(double v) { return (int)(v < 0 ? -std::floor(-v + 0.5) : std::floor(v + 0.5)); }

// Box of neuron n: x = round(centre), [max(x-r,1), min(x+r,size)] laterally,
// [max(z-ceil(r/axial),1), min(z+ceil(r/axial),Z)] axially (1-based), returned
// 0-based half-open.  generate_LFM_library_GPU.m:68-88.
static void neuron_box(const double* centers, int64_t n_neur, int64_t n, int64_t neur_rad, double axial, int64_t X,
                       int64_t Y, int64_t Z, int* box6)
{
    const int64_t zr = (int64_t)std::ceil((double)neur_rad / axial);
    const int x = mround(centers[n]), y = mround(centers[n + n_neur]), z = mround(centers[n + 2 * n_neur]);
    box6[0] = (int)std::max<int64_t>(x - neur_rad, 1) - 1;
    box6[1] = (int)std::min<int64_t>(x + neur_rad, X);
    box6[2] = (int)std::max<int64_t>(y - neur_rad, 1) - 1;
    box6[3] = (int)std::min<int64_t>(y + neur_rad, Y);
    box6[4] = (int)std::max<int64_t>(z - zr, 1) - 1;
    box6[5] = (int)std::min<int64_t>(z + zr, Z);
}

void lib_box_window(const sid_plan* p, LibBox& b)
{
    // output lenslets reached from the box: s = u + m + dlo
    const int N = (int)p->N;
    const int umin = b.x0 / N, umax = (b.x1 - 1) / N;
    const int vmin = b.y0 / N, vmax = (b.y1 - 1) / N;
    b.s0 = (int)std::max<int64_t>(0, umin + p->g.dlo);
    b.s1 = (int)std::min<int64_t>(p->Lx, umax + p->g.dhi + 1);
    b.t0 = (int)std::max<int64_t>(0, vmin + p->g.dlo);
    b.t1 = (int)std::min<int64_t>(p->Ly, vmax + p->g.dhi + 1);
}

int lib_stage(sid_plan* p, const char* who, const float* const* recon, int64_t n_comp, const double* centers,
              const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial, std::vector<LibBox>& boxes,
              cudaStream_t st)
{
    boxes.resize((size_t)n_neur);
    int64_t off = 0;
    for (int64_t n = 0; n < n_neur; ++n) {
        int bx[6];
        neuron_box(centers, n_neur, n, neur_rad, axial, p->X, p->Y, p->Z, bx);
        LibBox b;
        b.x0 = bx[0]; b.x1 = bx[1]; b.y0 = bx[2]; b.y1 = bx[3]; b.z0 = bx[4]; b.z1 = bx[5];
        int nc = 0;
        for (int64_t k = 0; k < n_comp; ++k) nc += neur_id[n + n_neur * k] ? 1 : 0;
        SID_REQUIRE(nc > 0, "%s: neuron %lld is in no component (neur_id row is empty)", who, (long long)(n + 1));
        SID_REQUIRE(b.x1 > b.x0 && b.y1 > b.y0 && b.z1 > b.z0,
                    "%s: neuron %lld has an empty box (centre outside the volume)", who, (long long)(n + 1));
        b.ncomp = nc;
        b.off = (int)off;
        off += (int64_t)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
        lib_box_window(p, b);
        boxes[(size_t)n] = b;
        SID_REQUIRE(off < INT32_MAX, "%s: boxes too large", who);
    }
    DBuf& dbox = p->ws[3];
    DBuf& dpack = p->ws[2];
    DBuf& dmeta = p->ws[1];
    SID_TRY(dbox.alloc(boxes.size() * sizeof(LibBox)));
    SID_TRY(dpack.alloc((size_t)off * sizeof(float)));
    SID_TRY(dmeta.alloc((size_t)(n_comp * sizeof(float*) + n_neur * n_comp)));
    SID_CUDA_TRY(cudaMemcpyAsync(dbox.p, boxes.data(), boxes.size() * sizeof(LibBox), cudaMemcpyHostToDevice, st));
    SID_CUDA_TRY(cudaMemcpyAsync(dmeta.p, recon, (size_t)n_comp * sizeof(float*), cudaMemcpyHostToDevice, st));
    uint8_t* did = dmeta.as<uint8_t>() + n_comp * sizeof(float*);
    SID_CUDA_TRY(cudaMemcpyAsync(did, neur_id, (size_t)(n_neur * n_comp), cudaMemcpyHostToDevice, st));
    k_lib_average<<<(unsigned)n_neur, 256, 0, st>>>(dmeta.as<const float*>(), did, n_neur, dbox.as<LibBox>(),
                                                    (int)n_comp, p->X, p->Y, dpack.as<float>());
    SID_CHECK_LAUNCH();
    return SID_OK;
}

}  // namespace sid

using namespace sid;

extern "C" int sid_library_boxes(const double* centers, int64_t n_neur, int64_t neur_rad, double axial, int64_t X,
                                 int64_t Y, int64_t Z, int32_t* boxes)
{
    SID_REQUIRE(centers && boxes && n_neur >= 0 && neur_rad >= 0 && axial > 0, "sid_library_boxes: bad argument");
    for (int64_t n = 0; n < n_neur; ++n) neuron_box(centers, n_neur, n, neur_rad, axial, X, Y, Z, boxes + 6 * n);
    return SID_OK;
}

namespace sid {

// Forward projections of the staged boxes (lib_stage) into the library rows
// through the FP32 lenslet taps; leaves `st` to be synchronised by the caller
// (the host tables are uploaded by pageable copies, so they may go out of scope).
int lib_run_direct(sid_plan* p, const char* who, const std::vector<LibBox>& boxes, float* out, int out_layout,
                   cudaStream_t st)
{
    SID_REQUIRE(p->taps_f.p, "%s: the plan has no lenslet taps", who);
    const int64_t n_neur = (int64_t)boxes.size();
    const int64_t N = p->N, D = p->g.D;
    int max_ns = 0, ntgM = 0, span = 0, nrv = 0, bwm = 0;
    for (const LibBox& b : boxes) {
        const int umin = b.x0 / (int)N, umax = (b.x1 - 1) / (int)N;
        const int vmin = b.y0 / (int)N, vmax = (b.y1 - 1) / (int)N;
        max_ns = std::max(max_ns, b.s1 - b.s0);
        ntgM = std::max(ntgM, (int)cdiv(b.t1 - b.t0, kLibT));
        span = std::max(span, std::max(umax - umin, vmax - vmin));
        nrv = std::max(nrv, (int)std::max(cdiv(b.x1 - b.x0, N), cdiv(b.y1 - b.y0, N)));
        bwm = std::max(bwm, b.x1 - b.x0);
    }
    // tiled kernel: output windows of W x Wt lenslets, W <= 32 (one lane per row)
    LibTileArgs ta;
    ta.N = (int)N; ta.D = (int)D; ta.dlo = (int)p->g.dlo; ta.span = span;
    ta.W = (int)D + span; ta.Wt = (int)D + span;
    const int tb = tile_tb(ta.Wt);
    ta.rows = ta.W + span;
    ta.cb = span + nrv - 1;
    ta.pitch = (tb + ta.cb) | 1;  // odd: the 32 lanes' rows fall in distinct banks
    ta.tsz = ta.rows * ta.pitch;
    ta.bwm = bwm;
    const size_t tiled_bytes = (size_t)(2 * N * ta.tsz + 2 * kLibG * std::max(nrv, 1) * bwm) * sizeof(float) +
                               (size_t)kLibG * (8 + 4 * N) * sizeof(int);
    const bool tiled = ta.W <= 32 && ta.Wt <= 32 && nrv >= 1 && nrv <= 3 && D * D <= 768 &&
                       tiled_bytes <= 200 * 1024;
    const int Dp = (int)D + 2 * span;
    const size_t tile_bytes =
        (size_t)N * Dp * (Dp + kLibT) * sizeof(float) + (size_t)(D * D + 4 * N * kLibG) * sizeof(int);
    if (!tiled) {
        SID_REQUIRE(tile_bytes <= 200 * 1024, "%s: tap tiles (%zu bytes) exceed shared memory", who, tile_bytes);
        SID_REQUIRE(max_ns * ntgM <= 256, "%s: neuron radius too large for one CTA (%d output groups)", who,
                    max_ns * ntgM);
    }
    // groups of up to kLibG neurons with the same depth window, in window order
    std::vector<int64_t> order(n_neur);
    for (int64_t n = 0; n < n_neur; ++n) order[n] = n;
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
        return boxes[x].z0 != boxes[y].z0 ? boxes[x].z0 < boxes[y].z0 : boxes[x].z1 < boxes[y].z1;
    });
    std::vector<int> groups;
    for (size_t i = 0; i < order.size();) {
        size_t e = i + 1;
        while (e < order.size() && (int)(e - i) < kLibG && boxes[order[e]].z0 == boxes[order[i]].z0 &&
               boxes[order[e]].z1 == boxes[order[i]].z1)
            ++e;
        groups.push_back((int)(e - i));
        for (size_t k = i; k < i + kLibG; ++k) groups.push_back(k < e ? (int)order[k] : 0);
        i = e;
    }
    const int64_t ngroups = (int64_t)groups.size() / (kLibG + 1);
    DBuf& dgrp = p->ws[0];
    SID_TRY(dgrp.alloc(groups.size() * sizeof(int)));
    SID_CUDA_TRY(cudaMemcpyAsync(dgrp.p, groups.data(), groups.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const LibBox* dbox = p->ws[3].as<LibBox>();
    const float* dpack = p->ws[2].as<float>();
    const int64_t P = p->X * p->Y;
    SID_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)(P * n_neur) * sizeof(float), st));
    const int64_t tbs = cdiv(N * D * D, 32) * 32;
    const int64_t ldn = out_layout == 0 ? 1 : P, ldp = out_layout == 0 ? n_neur : 1;
    dim3 grid((unsigned)ngroups, (unsigned)(N * N));
    if (tiled) {
        ta.tbs = tbs; ta.Lx = (int)p->Lx; ta.Ly = (int)p->Ly; ta.X = p->X; ta.Y = p->Y; ta.ldn = ldn; ta.ldp = ldp;
        SID_TRY(launch_lib_tile(tb, nrv, grid, tiled_bytes, p->taps_f.as<float>(), dpack,
                                dbox, dgrp.as<int>(), ta, out, st));
    } else {
        SID_CUDA_TRY(cudaFuncSetAttribute(k_lib_project<kLibG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)tile_bytes));
        k_lib_project<kLibG><<<grid, 256, tile_bytes, st>>>(p->taps_f.as<float>(), dpack,
                                                            dbox, dgrp.as<int>(), (int)N, (int)D,
                                                            (int)p->g.dlo, span, ntgM, tbs, (int)p->Lx, (int)p->Ly,
                                                            p->X, p->Y, out, ldn, ldp);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

// ---------------------------------------------------------------------------
// generate_LFM_library_CPU.m:18-70 with project_forward_patched.m:8-73: every
// neuron is a kernel W (given, or the ball x^2 + y^2 + (z r/rr)^2 <= r^2 over
// meshgrid(-r:r, -r:r, -rr:rr), rr = r / dim(3)) painted at its centre,
// forward-projected, and L2-normalised.  The patch projection of
// project_forward_patched.m (an odd number of lenslets, conv2 'full', pasted
// centred and clipped to the sensor) equals the frame's conv2 'same'
// projection of the painted volume for odd Nnum, so the rows come from the
// library kernels above.

// Voxel (0-based) and value of the kernel entries neuron n keeps:
// bbb = round(BWW - [r+1, r+1, rr+1] + centre) inside [1, X] x [1, Y] x [1, Z]
// for every nonzero W(BWW) in find(W) order (generate_LFM_library_CPU.m:39-49).
struct KernVox {
    int x, y, z;
    float v;
};

static double mround_d(double v) { return v < 0 ? -std::floor(-v + 0.5) : std::floor(v + 0.5); }

// W in MATLAB order (wx x wy x wz) with its r, rr; or the ball when W is null
struct KernelShape {
    std::vector<float> w;
    int64_t wx = 0, wy = 0, wz = 0;
    double r = 0, rr = 0;
};

static int kernel_shape(const char* who, double r, double dim_z, const float* W, int64_t wx, int64_t wy, int64_t wz,
                        KernelShape& ks)
{
    if (W) {
        SID_REQUIRE(wx >= 1 && wy >= 1 && wz >= 1, "%s: kernel dimensions must be positive", who);
        ks.wx = wx; ks.wy = wy; ks.wz = wz;
        ks.w.assign(W, W + wx * wy * wz);
        ks.r = (double)(wx - 1) / 2.0;   // generate_LFM_library_CPU.m:31-32
        ks.rr = (double)(wz - 1) / 2.0;
        return SID_OK;
    }
    SID_REQUIRE(r >= 0 && r == std::floor(r) && r <= 1024, "%s: the ball radius must be a whole number in [0, 1024]",
                who);
    SID_REQUIRE(dim_z > 0, "%s: dim(3) must be positive", who);
    ks.r = r;
    ks.rr = r / dim_z;  // generate_LFM_library_CPU.m:18
    // meshgrid(-r:r, -r:r, -rr:rr): X along columns, Y along rows, Z along pages;
    // -rr:rr holds floor(2 rr) + 1 values -rr + k
    const int64_t n = 2 * (int64_t)r + 1, nz = (int64_t)std::floor(2.0 * ks.rr + 1e-10) + 1;
    SID_REQUIRE(nz >= 1 && nz <= 4096, "%s: axial extent %lld outside [1, 4096]", who, (long long)nz);
    ks.wx = n; ks.wy = n; ks.wz = nz;
    ks.w.assign((size_t)(n * n * nz), 0.f);
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < n; ++i) {
                const double xv = -r + (double)j, yv = -r + (double)i, zv = -ks.rr + (double)k;
                const double t = zv * r / ks.rr;
                const bool in = ks.rr > 0 ? (xv * xv + yv * yv + t * t <= r * r) : (xv * xv + yv * yv <= r * r);
                ks.w[(size_t)(i + n * (j + n * k))] = in ? 1.f : 0.f;
            }
    return SID_OK;
}

static void kernel_voxels(const KernelShape& ks, const double* centers, int64_t n_neur, int64_t n, int64_t X,
                          int64_t Y, int64_t Z, std::vector<KernVox>& out)
{
    out.clear();
    const double cx = centers[n], cy = centers[n + n_neur], cz = centers[n + 2 * n_neur];
    for (int64_t k = 0; k < ks.wz; ++k)
        for (int64_t j = 0; j < ks.wy; ++j)
            for (int64_t i = 0; i < ks.wx; ++i) {
                const float v = ks.w[(size_t)(i + ks.wx * (j + ks.wy * k))];
                if (v == 0.f) continue;  // find(W): nonzero entries (NaN included)
                const double bx = mround_d(((double)(i + 1) - (ks.r + 1)) + cx);
                const double by = mround_d(((double)(j + 1) - (ks.r + 1)) + cy);
                const double bz = mround_d(((double)(k + 1) - (ks.rr + 1)) + cz);
                if (bx <= (double)X && bx > 0 && by <= (double)Y && by > 0 && bz <= (double)Z && bz > 0)
                    out.push_back({(int)bx - 1, (int)by - 1, (int)bz - 1, v});
            }
}

// Boxes around each neuron's painted voxels, their values packed into p->ws[2].
static int lib_stage_kernel(sid_plan* p, const char* who, const KernelShape& ks, const double* centers,
                            int64_t n_neur, std::vector<LibBox>& boxes, cudaStream_t st)
{
    boxes.resize((size_t)n_neur);
    std::vector<float> packed;
    std::vector<KernVox> vox;
    for (int64_t n = 0; n < n_neur; ++n) {
        kernel_voxels(ks, centers, n_neur, n, p->X, p->Y, p->Z, vox);
        SID_REQUIRE(!vox.empty(), "%s: neuron %lld has no kernel voxel inside the volume", who, (long long)(n + 1));
        LibBox b;
        b.x0 = b.y0 = b.z0 = INT32_MAX;
        b.x1 = b.y1 = b.z1 = 0;
        for (const KernVox& q : vox) {
            b.x0 = std::min(b.x0, q.x); b.x1 = std::max(b.x1, q.x + 1);
            b.y0 = std::min(b.y0, q.y); b.y1 = std::max(b.y1, q.y + 1);
            b.z0 = std::min(b.z0, q.z); b.z1 = std::max(b.z1, q.z + 1);
        }
        b.ncomp = 1;
        b.off = (int)packed.size();
        const int bw = b.x1 - b.x0, bh = b.y1 - b.y0;
        packed.resize(packed.size() + (size_t)bw * bh * (b.z1 - b.z0), 0.f);
        for (const KernVox& q : vox)
            packed[(size_t)b.off + (size_t)((q.x - b.x0) + bw * ((q.y - b.y0) + (int64_t)bh * (q.z - b.z0)))] = q.v;
        SID_REQUIRE(packed.size() < (size_t)INT32_MAX, "%s: kernels too large", who);
        lib_box_window(p, b);
        boxes[(size_t)n] = b;
    }
    SID_TRY(p->ws[3].alloc(boxes.size() * sizeof(LibBox)));
    SID_TRY(p->ws[2].alloc(packed.size() * sizeof(float)));
    SID_CUDA_TRY(cudaMemcpyAsync(p->ws[3].p, boxes.data(), boxes.size() * sizeof(LibBox), cudaMemcpyHostToDevice, st));
    SID_CUDA_TRY(cudaMemcpyAsync(p->ws[2].p, packed.data(), packed.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    // the host tables must outlive the copies
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    return SID_OK;
}

constexpr int kNormChunks = 256;

// part[c][n] = sum of squares of row n over pixel chunk c (FP64 sums)
__global__ void k_row_sumsq(const float* __restrict__ out, int64_t n_neur, int64_t P, int64_t ldn, int64_t ldp,
                            double* __restrict__ part)
{
    const int64_t chunk = (P + kNormChunks - 1) / kNormChunks;
    const int c = blockIdx.x;
    const int64_t p0 = c * chunk, p1 = min(P, p0 + chunk);
    for (int64_t n = blockIdx.y * (int64_t)blockDim.x + threadIdx.x; n < n_neur; n += (int64_t)gridDim.y * blockDim.x) {
        double s = 0.0;
        for (int64_t q = p0; q < p1; ++q) {
            const double v = out[n * ldn + q * ldp];
            s += v * v;
        }
        part[c * n_neur + n] = s;
    }
}

// row n /= sqrt(sum over chunks of part[c][n]) (generate_LFM_library_CPU.m:52: Q = Q / norm(Q))
__global__ void k_row_scale(float* __restrict__ out, int64_t n_neur, int64_t P, int64_t ldn, int64_t ldp,
                            const double* __restrict__ part)
{
    __shared__ double inv;
    for (int64_t n = blockIdx.y; n < n_neur; n += gridDim.y) {
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int c = 0; c < kNormChunks; ++c) s += part[c * n_neur + n];
            inv = 1.0 / sqrt(s);
        }
        __syncthreads();
        for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < P; q += (int64_t)gridDim.x * blockDim.x) {
            float* o = out + n * ldn + q * ldp;
            *o = (float)((double)*o * inv);
        }
    }
}

}  // namespace sid

using namespace sid;

extern "C" int sid_library(sid_plan* p, const float* const* recon, int64_t n_comp, const double* centers,
                           const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial, float* out,
                           int out_layout, void* stream)
{
    SID_REQUIRE(p && recon && centers && neur_id && out, "sid_library: NULL argument");
    SID_REQUIRE(n_comp >= 1 && n_neur >= 1 && neur_rad >= 0 && axial > 0,
                "sid_library: need n_comp >= 1, n_neur >= 1, neur_rad >= 0, axial > 0");
    SID_REQUIRE(out_layout == 0 || out_layout == 1, "sid_library: out_layout must be 0 (n x P) or 1 (P x n)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<LibBox> boxes;
    SID_TRY(lib_stage(p, "sid_library", recon, n_comp, centers, neur_id, n_neur, neur_rad, axial, boxes, st));
    SID_TRY(lib_run_direct(p, "sid_library", boxes, out, out_layout, st));
    // the staging buffers are read by the kernels above: wait before the
    // workspaces can be reused
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    return SID_OK;
}

extern "C" int sid_library_kernel(sid_plan* p, int method, const double* centers, int64_t n_neur, double r,
                                  double dim_z, const float* kernel, int64_t kx, int64_t ky, int64_t kz, float* out,
                                  int out_layout, void* stream)
{
    const char* who = "sid_library_kernel";
    SID_REQUIRE(p && centers && out, "%s: NULL argument", who);
    SID_REQUIRE(n_neur >= 1, "%s: need n_neur >= 1", who);
    SID_REQUIRE(out_layout == 0 || out_layout == 1, "%s: out_layout must be 0 (n x P) or 1 (P x n)", who);
    SID_REQUIRE(method == SID_METHOD_DIRECT || method == SID_METHOD_SPECTRAL_MIXED,
                "%s: method must be SID_METHOD_DIRECT or SID_METHOD_SPECTRAL_MIXED", who);
    // the centred paste of project_forward_patched.m:63-72 matches the frame's 'same' projection for odd Nnum
    // and odd PSF width; with an even width its index range runs past the projection (MATLAB stops there)
    SID_REQUIRE(p->N % 2 == 1, "%s: the patch projection's centring needs an odd Nnum", who);
    SID_REQUIRE(p->M % 2 == 1, "%s: the patch projection's paste needs an odd PSF width (M = %lld)", who,
                (long long)p->M);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    KernelShape ks;
    SID_TRY(kernel_shape(who, r, dim_z, kernel, kx, ky, kz, ks));
    std::vector<LibBox> boxes;
    SID_TRY(lib_stage_kernel(p, who, ks, centers, n_neur, boxes, st));
    SID_TRY(method == SID_METHOD_DIRECT ? lib_run_direct(p, who, boxes, out, out_layout, st)
                                        : lib_run_spectral(p, who, boxes, out, out_layout, st));
    const int64_t P = p->X * p->Y;
    const int64_t ldn = out_layout == 0 ? 1 : P, ldp = out_layout == 0 ? n_neur : 1;
    SID_TRY(p->red.alloc((size_t)(kNormChunks * n_neur) * sizeof(double)));
    k_row_sumsq<<<dim3(kNormChunks, (unsigned)std::min<int64_t>(cdiv(n_neur, 128), 64)), 128, 0, st>>>(
        out, n_neur, P, ldn, ldp, p->red.as<double>());
    SID_CHECK_LAUNCH();
    k_row_scale<<<dim3(64, (unsigned)std::min<int64_t>(n_neur, 65535)), 256, 0, st>>>(out, n_neur, P, ldn, ldp,
                                                                                    p->red.as<double>());
    SID_CHECK_LAUNCH();
    return plan_sync(p, st);
}

extern "C" int sid_library_kernel_voxels(const double* centers, int64_t n_neur, double r, double dim_z,
                                         const float* kernel, int64_t kx, int64_t ky, int64_t kz, int64_t X, int64_t Y,
                                         int64_t Z, int64_t* counts, int32_t* xyz, float* values, int64_t cap)
{
    const char* who = "sid_library_kernel_voxels";
    SID_REQUIRE(centers && counts && n_neur >= 0, "%s: bad argument", who);
    KernelShape ks;
    SID_TRY(kernel_shape(who, r, dim_z, kernel, kx, ky, kz, ks));
    std::vector<KernVox> vox;
    int64_t at = 0;
    for (int64_t n = 0; n < n_neur; ++n) {
        kernel_voxels(ks, centers, n_neur, n, X, Y, Z, vox);
        counts[n] = (int64_t)vox.size();
        for (const KernVox& q : vox) {
            if (xyz && at < cap) {
                xyz[3 * at] = q.x;
                xyz[3 * at + 1] = q.y;
                xyz[3 * at + 2] = q.z;
                if (values) values[at] = q.v;
            }
            ++at;
        }
    }
    SID_REQUIRE(!xyz || at <= cap, "%s: %lld voxels exceed the capacity %lld", who, (long long)at, (long long)cap);
    return SID_OK;
}
