// rect.cu -- lenslet rectification of sensor frames (ImageRect.m), batched
// over the frames of a movie as read_sensor_movie.m applies it.
//
// The host computes the resampling grid once per geometry (ImageRect.m:7-24,
// MATLAB colon semantics): coordinates stepping dx/M pixels around the lenslet
// centre, cut so the grid starts on a lenslet boundary, trimmed to whole
// lenslets, then cropped by the border lenslets (:29-45).  The kernel evaluates
// interp2's bilinear rule (NaN outside the image) at every output pixel of
// every frame, frames optionally multiplied by a mask first
// (read_sensor_movie.m:94-99); the output is the P x F movie layout (frame
// columns of out_rows x out_cols pixels).
#include <cmath>
#include <cstring>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

namespace {

// MATLAB a:step:b
std::vector<double> colon(double a, double step, double b)
{
    std::vector<double> v;
    if (step == 0.0 || (step > 0 && a > b) || (step < 0 && a < b)) return v;
    const int64_t n = (int64_t)std::floor((b - a) / step + 1e-10) + 1;
    v.reserve((size_t)n);
    for (int64_t k = 0; k < n; ++k) v.push_back(a + (double)k * step);
    return v;
}

struct RectGeom {
    std::vector<double> xq, yq;  // query coordinates (1-based pixels) of the output columns / rows
};

int rect_geometry(int64_t rows, int64_t cols, double xc, double yc, double dx, int64_t M, int crop,
                  const int32_t* cuts, RectGeom* g)
{
    SID_REQUIRE(rows > 1 && cols > 1 && M > 0 && dx > 0, "sid_image_rect: bad geometry");
    const double s = dx / (double)M;
    auto axis = [&](double c, int64_t size, std::vector<double>& out, int64_t& init) -> int {
        std::vector<double> lo = colon(c + 1, -s, 1.0);
        SID_REQUIRE(!lo.empty(), "sid_image_rect: centre %g outside the image", c);
        std::vector<double> hi = colon(c + 1 + s, s, (double)size);
        std::vector<double> all(lo.rbegin(), lo.rend());
        all.insert(all.end(), hi.begin(), hi.end());
        const int64_t centre = (int64_t)lo.size() - M / 2;  // find(== c + 1) - floor(M/2), 1-based
        init = centre - M * (int64_t)std::floor((double)centre / (double)M) + M;
        SID_REQUIRE(init >= 1 && init <= (int64_t)all.size(), "sid_image_rect: grid start outside the image");
        out.assign(all.begin() + (init - 1), all.end());
        return SID_OK;
    };
    int64_t xi = 0, yi = 0;
    SID_TRY(axis(xc, cols, g->xq, xi));
    SID_TRY(axis(yc, rows, g->yq, yi));
    // whole lenslets (ImageRect.m:27): M * floor((numel - init) / M)
    const int64_t nr = M * (int64_t)std::floor((double)((int64_t)g->yq.size() - yi) / (double)M);
    const int64_t nc = M * (int64_t)std::floor((double)((int64_t)g->xq.size() - xi) / (double)M);
    SID_REQUIRE(nr > 0 && nc > 0, "sid_image_rect: no whole lenslet in the image");
    int64_t r0 = 0, c0 = 0, r1 = nr, c1 = nc;
    if (crop) {
        const int64_t xs = nc / M, ys = nr / M;
        SID_REQUIRE(cuts[0] + cuts[1] < xs, "X-cut range is larger than the x-size of image");
        SID_REQUIRE(cuts[2] + cuts[3] < ys, "Y-cut range is larger than the y-size of image");
        c0 = (int64_t)cuts[0] * M;
        c1 = (xs - cuts[1]) * M;
        r0 = (int64_t)cuts[2] * M;
        r1 = (ys - cuts[3]) * M;
    }
    g->xq = std::vector<double>(g->xq.begin() + c0, g->xq.begin() + c1);
    g->yq = std::vector<double>(g->yq.begin() + r0, g->yq.begin() + r1);
    return SID_OK;
}

template <typename T> __device__ __forceinline__ float px(const T* f, int64_t i);
template <> __device__ __forceinline__ float px<float>(const float* f, int64_t i) { return f[i]; }
template <> __device__ __forceinline__ float px<uint16_t>(const uint16_t* f, int64_t i) { return (float)f[i]; }

// interp2's bilinear rule along one axis, evaluated on the host in FP64 for
// each output column (or row): the 1-based base index (the last interval
// serves the far edge) and the FP32 fraction, or index -1 outside [1, size].
// The kernel then needs no FP64 arithmetic per output pixel (GB300's FP64 rate
// is about 1/64 of its FP32 rate).
struct AxisTap {
    int32_t i;
    float f;
};

std::vector<AxisTap> axis_taps(const std::vector<double>& q, int64_t size)
{
    std::vector<AxisTap> t(q.size());
    for (size_t k = 0; k < q.size(); ++k) {
        const double v = q[k];
        if (!(v >= 1.0 && v <= (double)size)) {
            t[k] = {-1, 0.f};
            continue;
        }
        int64_t iv = (int64_t)std::floor(v);
        if (iv == size) --iv;
        t[k] = {(int32_t)iv, (float)(v - (double)iv)};
    }
    return t;
}

// out[(r + R c) + R C n] = interp2 at (xq[c], yq[r]) of frame n (times the mask).
template <typename T>
__global__ void k_rect(const T* __restrict__ in, const float* __restrict__ mask, int64_t rows, int64_t cols,
                       int64_t nframes, const AxisTap* __restrict__ tx, const AxisTap* __restrict__ ty, int64_t R,
                       int64_t C, float* __restrict__ out)
{
    const int64_t plane = R * C, total = plane * nframes;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / plane, rc = i - n * plane;
        const int64_t c = rc / R, r = rc - c * R;
        const AxisTap ax = tx[c], ay = ty[r];
        float v = __int_as_float(0x7fc00000);  // NaN outside the grid
        if (ax.i >= 0 && ay.i >= 0) {
            const int64_t ix = ax.i, iy = ay.i;
            const float fx = ax.f, fy = ay.f;
            const T* f = in + n * rows * cols;
            const int64_t i00 = (iy - 1) + rows * (ix - 1);
            auto at = [&](int64_t k) { return mask ? px<T>(f, k) * mask[k] : px<T>(f, k); };
            const float v00 = at(i00), v10 = ix < cols ? at(i00 + rows) : 0.f;
            const float v01 = iy < rows ? at(i00 + 1) : 0.f, v11 = (ix < cols && iy < rows) ? at(i00 + rows + 1) : 0.f;
            v = (1.f - fy) * ((1.f - fx) * v00 + fx * v10) + fy * ((1.f - fx) * v01 + fx * v11);
        }
        out[i] = v;
    }
}

}  // namespace

}  // namespace sid

using namespace sid;

extern "C" int sid_image_rect_size(int64_t rows, int64_t cols, double xCenter, double yCenter, double dx, int64_t M,
                                   int crop, const int32_t* cuts, int64_t* out_rows, int64_t* out_cols)
{
    SID_REQUIRE(out_rows && out_cols && (!crop || cuts), "sid_image_rect_size: NULL argument");
    RectGeom g;
    SID_TRY(rect_geometry(rows, cols, xCenter, yCenter, dx, M, crop, cuts, &g));
    *out_rows = (int64_t)g.yq.size();
    *out_cols = (int64_t)g.xq.size();
    return SID_OK;
}

extern "C" int sid_image_rect(sid_ctx* c, const void* frames, int dtype, int64_t rows, int64_t cols, int64_t nframes,
                              const float* mask, double xCenter, double yCenter, double dx, int64_t M, int crop,
                              const int32_t* cuts, float* out, void* stream)
{
    SID_REQUIRE(c && frames && out && (!crop || cuts), "sid_image_rect: NULL argument");
    SID_REQUIRE(dtype == SID_DTYPE_F32 || dtype == SID_DTYPE_U16, "sid_image_rect: frames must be single or uint16");
    SID_REQUIRE(nframes > 0, "sid_image_rect: no frames");
    RectGeom g;
    SID_TRY(rect_geometry(rows, cols, xCenter, yCenter, dx, M, crop, cuts, &g));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t R = (int64_t)g.yq.size(), C = (int64_t)g.xq.size();
    const std::vector<AxisTap> tx = axis_taps(g.xq, cols), ty = axis_taps(g.yq, rows);
    SID_TRY(c->mf[6].alloc((size_t)(R + C) * sizeof(AxisTap)));
    AxisTap* dq = c->mf[6].as<AxisTap>();
    SID_CUDA_TRY(cudaMemcpyAsync(dq, tx.data(), (size_t)C * sizeof(AxisTap), cudaMemcpyHostToDevice, st));
    SID_CUDA_TRY(cudaMemcpyAsync(dq + C, ty.data(), (size_t)R * sizeof(AxisTap), cudaMemcpyHostToDevice, st));
    const unsigned grid = (unsigned)std::min<int64_t>(cdiv(R * C * nframes, 256), 152 * 32);
    if (dtype == SID_DTYPE_U16)
        k_rect<uint16_t><<<grid, 256, 0, st>>>(static_cast<const uint16_t*>(frames), mask, rows, cols, nframes, dq,
                                               dq + C, R, C, out);
    else
        k_rect<float><<<grid, 256, 0, st>>>(static_cast<const float*>(frames), mask, rows, cols, nframes, dq, dq + C, R,
                                            C, out);
    SID_CHECK_LAUNCH();
    // the coordinate upload reads host vectors that go out of scope here
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    return SID_OK;
}
