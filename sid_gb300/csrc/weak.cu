// weak.cu -- exact back projection at the weakly observed voxels of the
// spectral projector.
//
// A voxel whose PSF falls mostly outside the sensor (border voxels at depths
// where the PSF is narrow and offset outwards by its lenslet phase) has a small
// column mass s_i = (A'1)_i.  Every back projection (A'u)_i of such a voxel is
// then small against the absolute rounding level of an FFT-based back
// projection, which is set by the largest values of the transform rather than
// by the entry, so the spectral forms give it few or no correct digits (and
// negative values are possible).  The multiplicative solvers divide by exactly
// these quantities (ISRA: X .* Htf ./ A'AX, deconvRL.m:52; Poisson RL:
// X .* A'r ./ A'1) and amplify the error every iteration.  The plan therefore
// lists, once, the voxels with s_i < frac * max(s) (frac 1e-2 unless the caller
// sets it; sid_plan_set_weak_fraction) and, after each spectral back
// projection, recomputes them exactly from the lenslet taps:
//   B(c,b,a,v,u) = sum_{b',a',m1,m2} K[c][b][a][b'][a'](m1,m2) Ip[b'][a'](v+m2+dlo, u+m1+dlo)
// (the transpose of the direct forward projection, FP32 sums).
//
// The weak voxels of a polyphase plane (c, b, a) lie on its border lines (the
// column u = 0 or Lx-1, the row v = 0 or Ly-1), so they are grouped into runs
// of <= 24 consecutive voxels along v (column runs) or u (row runs).  For a
// column run, lane m1 of a warp holds the D taps K(m1, :) and the lattice
// column s = u + m1 + dlo over the run's rows plus D - 1 in registers and
// accumulates all run outputs (run x D FMAs per D + run loads); the warps of
// the CTA split the N^2 tap arrays.  Row runs do the same on a transposed copy
// of the lattice.  Both read zero-padded copies of the sensor lattice, so no
// tap needs a bounds test.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

namespace {

constexpr int kWeakThreads = 256;
constexpr int kRunMax = 24;   // voxels per run
constexpr int kRunDMax = 32;  // largest tap extent the run kernel handles (else per voxel)

struct WeakRun {
    int plane;  // (c N + b) N + a
    int fixed;  // u of a column run, v of a row run
    int start;  // first v (column run) or u (row run)
    int len;
};

__global__ void k_fill_ones(float* __restrict__ x, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = 1.f;
}

// Zero-padded copies of the sensor lattice Ip[q][t][s] (q < N^2): pad[q][t + lo][s + lo]
// (Hp x Wp) and its transpose padT[q][s + lo][t + lo] (Wp x Hp).
__global__ void k_pad_lattice(const float* __restrict__ ip, float* __restrict__ pad, float* __restrict__ padT,
                              int nq, int Lx, int Ly, int lo, int Wp, int Hp)
{
    const int64_t plane = (int64_t)Wp * Hp, n = plane * nq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i / plane);
        const int64_t r = i - q * plane;
        const int tp = (int)(r / Wp), sp = (int)(r - (int64_t)tp * Wp);
        const int t = tp - lo, s = sp - lo;
        const float v = (t >= 0 && t < Ly && s >= 0 && s < Lx) ? ip[((int64_t)q * Ly + t) * Lx + s] : 0.f;
        pad[i] = v;
        if (padT) padT[q * plane + (int64_t)sp * Hp + tp] = v;
    }
}

// ROW = false: column runs (fixed u, v = start + j) on pad[q][t][s];
// ROW = true:  row runs (fixed v, u = start + j) on padT[q][s][t].
// Lanes take the cross-axis taps c (m1 of a column run, m2 of a row run) whose
// lattice line lies on the sensor; when at most 16 do, each half-warp takes its
// own tap array.  DM >= D bounds the tap loop (taps m >= D are zero), JR >=
// run length the outputs; the lattice line is streamed through the taps, so a
// thread holds DM taps and JR sums.
// blockIdx.z splits the N^2 tap arrays into qs ranges when there are too few
// runs to fill the GPU: each CTA then writes its partial sums to
// qpart[((z nb + volume) nrun_all + run0 + run) JR + j] and k_runs_finish adds
// them (in a fixed order) into the back projection.
template <bool ROW, int DM, int JR>
__global__ void __launch_bounds__(kWeakThreads, 2)
k_adj_runs(const float* __restrict__ taps, const float* __restrict__ lat, float* __restrict__ bp,
           const WeakRun* __restrict__ runs, int nrun, int N, int Lx, int Ly, int D, int dlo, int lo, int Wp, int Hp,
           int64_t tbs, int64_t lat_vol, int64_t bp_vol, int qs, float* __restrict__ qpart, int run0, int nrun_all)
{
    constexpr int NW = kWeakThreads / 32;
    // blockIdx.y: the volume of a batch (lattice copies and back projections back to back)
    const int vol = blockIdx.y;
    lat += vol * lat_vol;
    bp += vol * bp_vol;
    const int qper = (N * N + qs - 1) / qs, qbeg = blockIdx.z * qper, qend = min(N * N, qbeg + qper);
    constexpr int CM = JR + DM - 1;
    __shared__ float part[NW][JR];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = ROW ? Hp : Wp;   // pitch of the lattice copy along the run axis
    const int Lc = ROW ? Ly : Lx;  // lattice extent along the cross axis
    const int64_t plane = (int64_t)Wp * Hp;
    for (int rk = blockIdx.x; rk < nrun; rk += gridDim.x) {
        const WeakRun R = runs[rk];
        const int64_t blk0 = (int64_t)R.plane * N;
        const int clo = max(0, -R.fixed - dlo), chi = min(D, Lc - R.fixed - dlo);
        const int G = (chi - clo) <= 16 ? 2 : 1;  // tap arrays per warp step
        const int gw = 32 / G, g = lane / gw, c = clo + (lane - g * gw);
        float acc[JR];
#pragma unroll
        for (int j = 0; j < JR; ++j) acc[j] = 0.f;
        if (c < chi) {
            for (int q = qbeg + warp * G + g; q < qend; q += NW * G) {
                const int bq = q / N, aq = q - bq * N;
                const float* kb = taps + (blk0 + bq) * tbs + (int64_t)aq * D * D;
                // lattice line along the run axis at cross position fixed + c + dlo
                const float* line = lat + q * plane + (int64_t)(R.fixed + c + dlo + lo) +
                                    (int64_t)(R.start + dlo + lo) * W;
                const int nr = R.len + D - 1;
                float col[CM];
#pragma unroll
                for (int r = 0; r < CM; ++r) col[r] = r < nr ? __ldg(line + (int64_t)r * W) : 0.f;
                // taps along the run axis, streamed: K(m1 = c, m2) (column) or K(m1, m2 = c) (row)
#pragma unroll
                for (int m = 0; m < DM; ++m) {
                    const float km = m < D ? __ldg(ROW ? kb + (int64_t)m * D + c : kb + (int64_t)c * D + m) : 0.f;
#pragma unroll
                    for (int j = 0; j < JR; ++j) acc[j] = fmaf(km, col[j + m], acc[j]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < JR; ++j) {
            float a = acc[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (lane == 0) part[warp][j] = a;
        }
        __syncthreads();
        if (threadIdx.x < R.len) {
            float s = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) s += part[w][threadIdx.x];
            if (qs > 1) {
                qpart[(((int64_t)blockIdx.z * gridDim.y + vol) * nrun_all + run0 + rk) * JR + threadIdx.x] = s;
            } else {
                const int u = ROW ? R.start + (int)threadIdx.x : R.fixed;
                const int v = ROW ? R.fixed : R.start + (int)threadIdx.x;
                bp[((int64_t)R.plane * Ly + v) * Lx + u] = s;
            }
        }
        __syncthreads();
    }
}

// bp[volume][voxel of run, j] = sum over z < qs of the split partial sums, for
// the runs [lo1, hi1) and [lo2, hi2) (runs [0, ncol) are column runs, the rest
// row runs)
template <int JR>
__global__ void k_runs_finish(const float* __restrict__ qpart, const WeakRun* __restrict__ runs, int nrun_all,
                              int ncol, int qs, int nb, int Lx, int Ly, float* __restrict__ bp, int64_t bp_vol,
                              int lo1, int hi1, int lo2, int hi2)
{
    const int n1 = hi1 - lo1, cnt = n1 + (hi2 - lo2);
    const int64_t total = (int64_t)nb * cnt * JR;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i % JR);
        const int64_t vr = i / JR;
        const int t = (int)(vr % cnt), vol = (int)(vr / cnt);
        const int rk = t < n1 ? lo1 + t : lo2 + (t - n1);
        const WeakRun R = runs[rk];
        if (j >= R.len) continue;
        float s = 0.f;
        for (int z = 0; z < qs; ++z) s += qpart[(((int64_t)z * nb + vol) * nrun_all + rk) * JR + j];
        const bool row = rk >= ncol;
        const int u = row ? R.start + j : R.fixed;
        const int v = row ? R.fixed : R.start + j;
        bp[vol * bp_vol + ((int64_t)R.plane * Ly + v) * Lx + u] = s;
    }
}

// Generic path (tap extent above kRunDMax): one CTA per voxel.
__global__ void __launch_bounds__(kWeakThreads)
k_adj_voxel(const float* __restrict__ taps, const float* __restrict__ ip, float* __restrict__ bp,
            const int* __restrict__ list, int nweak, int N, int Lx, int Ly, int D, int dlo, int64_t tbs)
{
    __shared__ float red[kWeakThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int w = blockIdx.x; w < nweak; w += gridDim.x) {
        const int64_t i = list[w];
        const int u = (int)(i % Lx);
        const int64_t r0 = i / Lx;
        const int v = (int)(r0 % Ly);
        const int64_t blk0 = (r0 / Ly) * N;
        const int m1lo = max(0, -u - dlo), m1hi = min(D, Lx - u - dlo);
        const int m2lo = max(0, -v - dlo), m2hi = min(D, Ly - v - dlo);
        const int n1 = m1hi - m1lo, n2 = m2hi - m2lo;
        float acc = 0.f;
        if (n1 > 0 && n2 > 0) {
            const int items = N * N * n1;
            for (int it = threadIdx.x; it < items; it += kWeakThreads) {
                const int q = it / n1, m1 = m1lo + (it - q * n1);
                const int bq = q / N, aq = q - bq * N;
                const float* tp = taps + (blk0 + bq) * tbs + ((int64_t)aq * D + m1) * D + m2lo;
                const float* xp = ip + ((int64_t)q * Ly + (v + m2lo + dlo)) * Lx + (u + m1 + dlo);
                for (int j2 = 0; j2 < n2; ++j2) acc = fmaf(__ldg(tp + j2), __ldg(xp + (int64_t)j2 * Lx), acc);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (warp == 0) {
            acc = lane < kWeakThreads / 32 ? red[lane] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) bp[i] = acc;
        }
        __syncthreads();
    }
}

// A maximal run of `len` voxels as ceil(len / kRunMax) runs of near-equal length.
void split_run(int plane, int fixed, int start, int len, std::vector<WeakRun>& out)
{
    const int pieces = (len + kRunMax - 1) / kRunMax;
    for (int k = 0, s = start; k < pieces; ++k) {
        const int l = len / pieces + (k < len % pieces ? 1 : 0);
        out.push_back({plane, fixed, s, l});
        s += l;
    }
}

// Cover one plane's weak voxels (v, u), sorted by (v, u), with runs: each voxel
// goes to the direction of its longer maximal run (ties: column).
void plane_runs(int plane, const std::vector<std::pair<int, int>>& vu, int Lx, int Ly, std::vector<WeakRun>& cols,
                std::vector<WeakRun>& rows)
{
    std::vector<unsigned char> in((size_t)Lx * Ly, 0), as_row((size_t)Lx * Ly, 0);
    for (auto& e : vu) in[(size_t)e.first * Lx + e.second] = 1;
    auto at = [&](int v, int u) { return v >= 0 && v < Ly && u >= 0 && u < Lx && in[(size_t)v * Lx + u]; };
    for (auto& e : vu) {
        const int v = e.first, u = e.second;
        int h = 1, c = 1;
        for (int x = u - 1; at(v, x); --x) ++h;
        for (int x = u + 1; at(v, x); ++x) ++h;
        for (int y = v - 1; at(y, u); --y) ++c;
        for (int y = v + 1; at(y, u); ++y) ++c;
        as_row[(size_t)v * Lx + u] = h > c;
    }
    // row runs: consecutive u at fixed v among the voxels assigned to rows
    for (int v = 0; v < Ly; ++v)
        for (int u = 0; u < Lx;) {
            if (!(in[(size_t)v * Lx + u] && as_row[(size_t)v * Lx + u])) { ++u; continue; }
            int e = u;
            while (e < Lx && in[(size_t)v * Lx + e] && as_row[(size_t)v * Lx + e]) ++e;
            split_run(plane, v, u, e - u, rows);
            u = e;
        }
    for (int u = 0; u < Lx; ++u)
        for (int v = 0; v < Ly;) {
            if (!(in[(size_t)v * Lx + u] && !as_row[(size_t)v * Lx + u])) { ++v; continue; }
            int e = v;
            while (e < Ly && in[(size_t)e * Lx + u] && !as_row[(size_t)e * Lx + u]) ++e;
            split_run(plane, u, v, e - v, cols);
            v = e;
        }
}

// the run kernel for the smallest tap bound DM >= D
template <bool ROW>
int launch_runs(int D, dim3 grid, const float* taps, const float* lat, float* bp, const WeakRun* runs, int nrun, int N,
                int Lx, int Ly, int dlo, int lo, int Wp, int Hp, int64_t tbs, int64_t pv, int64_t nv, float* qpart,
                int run0, int nrun_all, cudaStream_t st)
{
#define SID_RUNS_CASE(DMV)                                                                                         \
    if (D <= DMV) {                                                                                                \
        k_adj_runs<ROW, DMV, kRunMax><<<grid, kWeakThreads, 0, st>>>(taps, lat, bp, runs, nrun, N, Lx, Ly, D, dlo, \
                                                                      lo, Wp, Hp, tbs, pv, nv, (int)grid.z, qpart, \
                                                                      run0, nrun_all);                             \
        SID_CHECK_LAUNCH();                                                                                        \
        return SID_OK;                                                                                             \
    }
    SID_RUNS_CASE(16) SID_RUNS_CASE(20) SID_RUNS_CASE(25) SID_RUNS_CASE(28) SID_RUNS_CASE(32)
#undef SID_RUNS_CASE
    set_error("spectral plan: tap extent %d above the run kernel's %d", D, kRunDMax);
    return SID_EINVAL;
}

}  // namespace

// List the weakly observed voxels: s = A'1 through the plan's most accurate
// spectral back projection (its error is far below the threshold), then the
// in-frame voxels with s < p->weak_frac * max(s), grouped into runs.
int weak_build(sid_plan* p)
{
    p->nweak = p->nweak_cols = p->nweak_rows = 0;
    p->weak.release();
    p->weak_pad.release();
    if (p->weak_frac <= 0.0) return SID_OK;
    const int64_t N = p->N, Lx = p->Lx, Ly = p->Ly, Z = p->Z;
    const int64_t ni = N * N * Lx * Ly, n = ni * Z;
    SID_REQUIRE(n < INT32_MAX, "spectral plan: volume too large for the weak-voxel list");
    const int fmt = p->spec_f32 ? FMT_F32 : (p->spec_f24 ? FMT_F24 : FMT_I16);
    DBuf ones, s;
    SID_TRY(ones.alloc((size_t)ni * sizeof(float)));
    SID_TRY(s.alloc((size_t)n * sizeof(float)));
    k_fill_ones<<<1024, 256>>>(ones.as<float>(), ni);
    SID_CHECK_LAUNCH();
    SID_TRY(mask_vp(p, ones.as<float>(), 1, 0));
    SID_TRY(spectral_adjoint(p, fmt, ones.as<float>(), s.as<float>(), 0));
    std::vector<float> h((size_t)n);
    SID_CUDA_TRY(cudaMemcpy(h.data(), s.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost));
    ones.release();
    s.release();
    const int64_t plane = Lx * Ly;
    // in-frame test of polyphase index i: x = a + N u < X and y = b + N v < Y
    auto in_frame = [&](int64_t i) {
        const int64_t u = i % Lx, v = (i / Lx) % Ly, a = (i / plane) % N, b = (i / (plane * N)) % N;
        return a + N * u < p->X && b + N * v < p->Y;
    };
    double smax = 0.0;
    for (int64_t i = 0; i < n; ++i)
        if (h[(size_t)i] > smax && in_frame(i)) smax = h[(size_t)i];
    const double thr = p->weak_frac * smax;
    std::vector<int> list;
    for (int64_t i = 0; i < n; ++i)
        if ((double)h[(size_t)i] < thr && in_frame(i)) list.push_back((int)i);
    if (list.empty()) return SID_OK;
    p->nweak = (int64_t)list.size();
    if (p->g.D > kRunDMax) {  // per-voxel path
        SID_TRY(p->weak.alloc(list.size() * sizeof(int)));
        SID_CUDA_TRY(cudaMemcpy(p->weak.p, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
        return SID_OK;
    }
    std::vector<WeakRun> cols, rows;
    for (size_t k = 0; k < list.size();) {
        const int pl = (int)(list[k] / plane);
        std::vector<std::pair<int, int>> vu;
        for (; k < list.size() && list[k] / plane == pl; ++k)
            vu.push_back({(int)((list[k] % plane) / Lx), (int)(list[k] % Lx)});
        plane_runs(pl, vu, (int)Lx, (int)Ly, cols, rows);
    }
    // runs of depths [0, z): the runs come plane by plane, depth-major
    p->weak_cz.assign((size_t)Z + 1, 0);
    p->weak_rz.assign((size_t)Z + 1, 0);
    for (const WeakRun& r : cols) ++p->weak_cz[(size_t)(r.plane / (N * N)) + 1];
    for (const WeakRun& r : rows) ++p->weak_rz[(size_t)(r.plane / (N * N)) + 1];
    for (int64_t z = 0; z < Z; ++z) {
        p->weak_cz[(size_t)z + 1] += p->weak_cz[(size_t)z];
        p->weak_rz[(size_t)z + 1] += p->weak_rz[(size_t)z];
    }
    std::vector<WeakRun> all(cols);
    all.insert(all.end(), rows.begin(), rows.end());
    SID_TRY(p->weak.alloc(all.size() * sizeof(WeakRun)));
    SID_CUDA_TRY(cudaMemcpy(p->weak.p, all.data(), all.size() * sizeof(WeakRun), cudaMemcpyHostToDevice));
    p->nweak_cols = (int64_t)cols.size();
    p->nweak_rows = (int64_t)rows.size();
    // padded lattice copies (plain and transposed)
    const int64_t lo = std::max<int64_t>(0, -p->g.dlo), hi = std::max<int64_t>(0, p->g.D - 1 + p->g.dlo);
    const int64_t Wp = Lx + lo + hi, Hp = Ly + lo + hi;
    SID_TRY(p->weak_pad.alloc((size_t)(2 * N * N * Wp * Hp) * sizeof(float)));
    return SID_OK;
}

// Tap-array split of the run kernel for nb volumes: qs CTAs per run until
// ~16 CTAs per SM are in the grid (one volume's few hundred runs, each walking
// all N^2 tap arrays in one CTA, left most SMs idle).
int weak_qsplit(const sid_plan* p, int64_t nb)
{
    const int64_t nall = p->nweak_cols + p->nweak_rows;
    if (nall == 0) return 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>(16, cdiv(16 * sm_count(), nall * nb)));
}

// Overwrite the listed voxels of nb spectral back projections bp[b] = A' ip[b]
// (polyphase volumes and images back to back) with their exact values.
struct WeakGeom {
    int N, Lx, Ly, D, dlo, lo, Wp, Hp;
    int64_t tbs, ni, nv, pv;
};

static WeakGeom weak_geom(const sid_plan* p)
{
    WeakGeom g;
    g.N = (int)p->N; g.Lx = (int)p->Lx; g.Ly = (int)p->Ly; g.D = (int)p->g.D; g.dlo = (int)p->g.dlo;
    g.lo = (int)std::max<int64_t>(0, -p->g.dlo);
    const int hi = (int)std::max<int64_t>(0, p->g.D - 1 + p->g.dlo);
    g.Wp = g.Lx + g.lo + hi;
    g.Hp = g.Ly + g.lo + hi;
    g.tbs = cdiv(p->N * p->g.D * p->g.D, 32) * 32;
    g.ni = (int64_t)g.N * g.N * g.Lx * g.Ly;
    g.nv = g.ni * p->Z;
    g.pv = (int64_t)g.N * g.N * g.Wp * g.Hp;  // one volume's padded lattice copy
    return g;
}

bool weak_runs_path(const sid_plan* p) { return p->nweak == 0 || p->g.D <= kRunDMax; }

// Zero-padded (and transposed) copies of nb sensor lattices for the run kernel.
int weak_pad(sid_plan* p, const float* ip, int nb, cudaStream_t st)
{
    if (p->nweak == 0) return SID_OK;
    SID_REQUIRE(weak_runs_path(p), "weak voxels: the run kernel needs a tap extent of at most %d", kRunDMax);
    const WeakGeom g = weak_geom(p);
    SID_TRY(p->weak_pad.alloc((size_t)(2 * nb * g.pv) * sizeof(float)));
    float* pad = p->weak_pad.as<float>();
    k_pad_lattice<<<1024, 256, 0, st>>>(ip, pad, p->nweak_rows ? pad + nb * g.pv : nullptr, nb * g.N * g.N, g.Lx,
                                        g.Ly, g.lo, g.Wp, g.Hp);
    SID_CHECK_LAUNCH();
    return SID_OK;
}

// The weak voxels of depths [z0, z1) of nb back projections, from the copies
// of weak_pad.
int weak_runs(sid_plan* p, float* bp, int nb, int64_t z0, int64_t z1, cudaStream_t st)
{
    if (p->nweak == 0) return SID_OK;
    SID_REQUIRE(p->taps_f.p, "spectral plan: lenslet taps missing for the weak-voxel back projection");
    const WeakGeom g = weak_geom(p);
    const float* pad = p->weak_pad.as<float>();
    const float* padT = pad + nb * g.pv;
    const WeakRun* runs = p->weak.as<WeakRun>();
    const float* taps = p->taps_f.as<float>();
    const int nc = (int)p->nweak_cols, nall = nc + (int)p->nweak_rows;
    const int c0 = p->weak_cz[(size_t)z0], c1 = p->weak_cz[(size_t)z1];
    const int r0 = p->weak_rz[(size_t)z0], r1 = p->weak_rz[(size_t)z1];
    if (c1 == c0 && r1 == r0) return SID_OK;
    const int qs = weak_qsplit(p, nb);
    float* qpart = nullptr;
    if (qs > 1) {
        SID_TRY(p->weak_part.alloc((size_t)qs * nb * nall * kRunMax * sizeof(float)));
        qpart = p->weak_part.as<float>();
    }
    if (c1 > c0)
        SID_TRY(launch_runs<false>(g.D, dim3((unsigned)(c1 - c0), (unsigned)nb, (unsigned)qs), taps, pad, bp,
                                   runs + c0, c1 - c0, g.N, g.Lx, g.Ly, g.dlo, g.lo, g.Wp, g.Hp, g.tbs, g.pv, g.nv,
                                   qpart, c0, nall, st));
    if (r1 > r0)
        SID_TRY(launch_runs<true>(g.D, dim3((unsigned)(r1 - r0), (unsigned)nb, (unsigned)qs), taps, padT, bp,
                                  runs + nc + r0, r1 - r0, g.N, g.Lx, g.Ly, g.dlo, g.lo, g.Wp, g.Hp, g.tbs, g.pv,
                                  g.nv, qpart, nc + r0, nall, st));
    if (qs > 1) {
        const int64_t tot = (int64_t)nb * ((c1 - c0) + (r1 - r0)) * kRunMax;
        k_runs_finish<kRunMax><<<(unsigned)std::min<int64_t>(cdiv(tot, 256), 4096), 256, 0, st>>>(
            qpart, runs, nall, nc, qs, nb, g.Lx, g.Ly, bp, g.nv, c0, c1, nc + r0, nc + r1);
        SID_CHECK_LAUNCH();
    }
    return SID_OK;
}

int weak_fix_n(sid_plan* p, const float* ip, float* bp, int nb, cudaStream_t st)
{
    if (p->nweak == 0) return SID_OK;
    SID_REQUIRE(p->taps_f.p, "spectral plan: lenslet taps missing for the weak-voxel back projection");
    if (!weak_runs_path(p)) {
        const WeakGeom g = weak_geom(p);
        const unsigned grid = (unsigned)std::min<int64_t>(p->nweak, 152 * 8);
        for (int b = 0; b < nb; ++b) {
            k_adj_voxel<<<grid, kWeakThreads, 0, st>>>(p->taps_f.as<float>(), ip + b * g.ni, bp + b * g.nv,
                                                       p->weak.as<int>(), (int)p->nweak, g.N, g.Lx, g.Ly, g.D, g.dlo,
                                                       g.tbs);
            SID_CHECK_LAUNCH();
        }
        return SID_OK;
    }
    SID_TRY(weak_pad(p, ip, nb, st));
    return weak_runs(p, bp, nb, 0, p->Z, st);
}

int weak_fix(sid_plan* p, const float* ip, float* bp, cudaStream_t st) { return weak_fix_n(p, ip, bp, 1, st); }

}  // namespace sid

using namespace sid;

extern "C" int sid_plan_set_weak_fraction(sid_plan* p, double frac)
{
    SID_REQUIRE(p, "sid_plan_set_weak_fraction: NULL plan");
    SID_REQUIRE(frac >= 0.0 && frac <= 1.0, "sid_plan_set_weak_fraction: fraction %g outside [0, 1]", frac);
    SID_REQUIRE(p->spec_f32 || p->spec_f24 || p->spec_i16, "sid_plan_set_weak_fraction: plan has no spectral form");
    p->weak_frac = frac;
    return weak_build(p);
}

extern "C" int sid_weak_runs_plan(const int32_t* list, int64_t n, int64_t N, int64_t Lx, int64_t Ly, int32_t* runs,
                                  int64_t cap, int64_t* ncols, int64_t* nrows)
{
    SID_REQUIRE((list || n == 0) && ncols && nrows && N >= 1 && Lx >= 1 && Ly >= 1, "sid_weak_runs_plan: bad argument");
    const int64_t plane = Lx * Ly;
    for (int64_t k = 1; k < n; ++k)
        SID_REQUIRE(list[k] > list[k - 1], "sid_weak_runs_plan: voxel list not strictly ascending at %lld",
                    (long long)k);
    // the grouping of weak_build: plane by plane, each plane's voxels into column and row runs
    std::vector<WeakRun> cols, rows;
    for (int64_t k = 0; k < n;) {
        const int pl = (int)(list[k] / plane);
        std::vector<std::pair<int, int>> vu;
        for (; k < n && list[k] / plane == pl; ++k)
            vu.push_back({(int)((list[k] % plane) / Lx), (int)(list[k] % Lx)});
        plane_runs(pl, vu, (int)Lx, (int)Ly, cols, rows);
    }
    *ncols = (int64_t)cols.size();
    *nrows = (int64_t)rows.size();
    const int64_t total = *ncols + *nrows;
    if (runs) {
        SID_REQUIRE(total <= cap, "sid_weak_runs_plan: %lld runs exceed the capacity %lld", (long long)total,
                    (long long)cap);
        int64_t at = 0;
        for (const std::vector<WeakRun>* v : {&cols, &rows})
            for (const WeakRun& r : *v) {
                runs[4 * at] = r.plane;
                runs[4 * at + 1] = r.fixed;
                runs[4 * at + 2] = r.start;
                runs[4 * at + 3] = r.len;
                ++at;
            }
    }
    return SID_OK;
}
