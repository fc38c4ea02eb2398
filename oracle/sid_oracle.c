/*
 * sid_oracle.c -- CPU restatement (FP64) of the SID light-field projector and
 * of the Lawson-Hanson non-negative quadratic solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA path is compared
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm may load it.  The product library (libsid.so) never links it.
 *
 * Parity status: parity unpinned against the real reference.  The reference is
 * MATLAB (R2017b built-ins conv2, imrotate, linsolve); neither MATLAB nor GNU
 * Octave is available, and the reference ships no test vectors.  The
 * restatement is cross-checked against an independent NumPy/SciPy
 * transcription of the reference's loop structure (tests/golden/make_golden.py,
 * scipy.signal.convolve2d standing in for MATLAB conv2 'same').
 *
 * Layout: MATLAB column-major throughout.
 *   H  (M, M, N, N, Z)   H(i,j,a,b,c) at i + M*(j + M*(a + N*(b + N*c)))
 *   V  (X, Y, Z)         V(x,y,c)     at x + X*(y + Y*c)
 *   I  (X, Y)            I(x,y)       at x + X*y
 *   ca (Z, 2) int, 1-based CAindex; ca == NULL means [1, M] for every depth
 *      (the forwardProjectGPU / backwardProjectGPU_new semantics).
 *
 * Semantics restated (0-based indices):
 *   forwardProjectACC.m:14-29 / forwardProjectGPU.m:16-28 with conv2FFT_.m:3-15:
 *     For depth c the PSF window is rows/cols lo..hi of H (lo = ca(c,1)-1,
 *     hi = ca(c,2)-1, Mc = hi-lo+1).  conv2(.,.,'same') aligns kernel element
 *     floor(Mc/2) with the output pixel, so
 *       I(x,y) = sum_c sum_{px,py} V(px,py,c) *
 *                H(x-px+cf+lo, y-py+cf+lo, px mod N, py mod N, c),  cf = floor(Mc/2)
 *     restricted to 0 <= x-px+cf < Mc (and likewise for y).  The FFT form of
 *     forwardProjectGPU.m (exindex.m:249 circular roll by floor(M/2), exsize >=
 *     X + floor(M/2)) has no wrap-around inside the crop, so it equals the same sum.
 *   backwardProjectACC_new.m:14-26 / backwardProjectGPU_new.m:16-24:
 *     filter = imrotate(Hc,180) = Hc flipped in both axes, conv2 'same', then
 *     keep only the voxels of phase (a,b):
 *       B(px,py,c) = sum_{x,y} I(x,y) * H(x-px+cb+lo, y-py+cb+lo, px mod N, py mod N, c)
 *     with cb = Mc-1-floor(Mc/2).  For odd Mc, cb == cf and B is the exact adjoint.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

typedef int64_t i64;

static void depth_window(i64 M, i64 Z, const int* ca, i64 c, i64* lo, i64* mc)
{
    if (ca) {
        *lo = (i64)ca[c] - 1;
        *mc = (i64)ca[Z + c] - (i64)ca[c] + 1;
    } else {
        *lo = 0;
        *mc = M;
    }
}

static inline i64 imax(i64 a, i64 b) { return a > b ? a : b; }
static inline i64 imin(i64 a, i64 b) { return a < b ? a : b; }

/* One forward-projected sensor pixel (x, y). */
static double fwd_pixel(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                        const double* V, i64 X, i64 Y, i64 x, i64 y)
{
    double acc = 0.0;
    for (i64 c = 0; c < Z; ++c) {
        i64 lo, mc;
        depth_window(M, Z, ca, c, &lo, &mc);
        i64 cf = mc / 2;
        /* px in [x+cf-mc+1, x+cf] */
        i64 px0 = imax(0, x + cf - mc + 1), px1 = imin(X - 1, x + cf);
        i64 py0 = imax(0, y + cf - mc + 1), py1 = imin(Y - 1, y + cf);
        for (i64 py = py0; py <= py1; ++py) {
            i64 j = y - py + cf + lo;
            i64 b = py % N;
            const double* vcol = V + X * (py + Y * c);
            for (i64 px = px0; px <= px1; ++px) {
                double v = vcol[px];
                if (v == 0.0) continue;
                i64 i = x - px + cf + lo;
                i64 a = px % N;
                acc += v * (double)H[i + M * (j + M * (a + N * (b + N * c)))];
            }
        }
    }
    return acc;
}

/* One back-projected voxel (px, py, c). */
static double adj_voxel(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                        const double* I, i64 X, i64 Y, i64 px, i64 py, i64 c)
{
    i64 lo, mc;
    depth_window(M, Z, ca, c, &lo, &mc);
    i64 cb = mc - 1 - mc / 2;
    i64 a = px % N, b = py % N;
    /* x in [px-cb, px-cb+mc-1] */
    i64 x0 = imax(0, px - cb), x1 = imin(X - 1, px - cb + mc - 1);
    i64 y0 = imax(0, py - cb), y1 = imin(Y - 1, py - cb + mc - 1);
    const float* Hs = H + M * M * (a + N * (b + N * c));
    double acc = 0.0;
    for (i64 y = y0; y <= y1; ++y) {
        i64 j = y - py + cb + lo;
        const double* icol = I + X * y;
        const float* hcol = Hs + M * j;
        for (i64 x = x0; x <= x1; ++x) {
            i64 i = x - px + cb + lo;
            acc += icol[x] * (double)hcol[i];
        }
    }
    return acc;
}

/* Full forward projection: I = A V (forwardProjectACC.m:14-29). */
void oracle_forward(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                    const double* V, i64 X, i64 Y, double* I)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (i64 y = 0; y < Y; ++y)
        for (i64 x = 0; x < X; ++x)
            I[x + X * y] = fwd_pixel(H, M, N, Z, ca, V, X, Y, x, y);
}

/* Full back projection: V = A^T I (backwardProjectACC_new.m:14-26). */
void oracle_adjoint(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                    const double* I, i64 X, i64 Y, double* V)
{
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (i64 c = 0; c < Z; ++c)
        for (i64 py = 0; py < Y; ++py)
            for (i64 px = 0; px < X; ++px)
                V[px + X * (py + Y * c)] = adj_voxel(H, M, N, Z, ca, I, X, Y, px, py, c);
}

/* Sampled forward: out[k] = (A V)(pix[2k], pix[2k+1]). */
void oracle_forward_pixels(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                           const double* V, i64 X, i64 Y,
                           const i64* pix, i64 n, double* out)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (i64 k = 0; k < n; ++k)
        out[k] = fwd_pixel(H, M, N, Z, ca, V, X, Y, pix[2 * k], pix[2 * k + 1]);
}

/* Sampled adjoint: out[k] = (A^T I)(vox[3k], vox[3k+1], vox[3k+2]). */
void oracle_adjoint_voxels(const float* H, i64 M, i64 N, i64 Z, const int* ca,
                           const double* I, i64 X, i64 Y,
                           const i64* vox, i64 n, double* out)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (i64 k = 0; k < n; ++k)
        out[k] = adj_voxel(H, M, N, Z, ca, I, X, Y, vox[3 * k], vox[3 * k + 1], vox[3 * k + 2]);
}

/* FP32 lenslet-sparse forward projection, timed as the CPU baseline.  Same sum
 * as oracle_forward (uncropped PSF), single-precision accumulation, OpenMP over
 * the output pixels of sensor columns [y_begin, y_end).  `nthreads` <= 0 means
 * the OpenMP default. */
void baseline_forward_f32(const float* H, i64 M, i64 N, i64 Z,
                          const float* V, i64 X, i64 Y, float* I,
                          i64 y_begin, i64 y_end, int nthreads)
{
    if (nthreads > 0) {
        extern void omp_set_num_threads(int);
        omp_set_num_threads(nthreads);
    }
    i64 cf = M / 2;
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (i64 y = y_begin; y < y_end; ++y) {
        for (i64 x = 0; x < X; ++x) {
            float acc = 0.f;
            for (i64 c = 0; c < Z; ++c) {
                i64 px0 = imax(0, x + cf - M + 1), px1 = imin(X - 1, x + cf);
                i64 py0 = imax(0, y + cf - M + 1), py1 = imin(Y - 1, y + cf);
                for (i64 py = py0; py <= py1; ++py) {
                    i64 j = y - py + cf;
                    i64 b = py % N;
                    const float* vcol = V + X * (py + Y * c);
                    for (i64 px = px0; px <= px1; ++px) {
                        i64 i = x - px + cf;
                        acc += vcol[px] * H[i + M * (j + M * (px % N + N * (b + N * c)))];
                    }
                }
            }
            I[x + X * y] = acc;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Lawson-Hanson non-negative quadratic program (NQP.m:42-178):
 *     argmin_{x >= 0} 0.5 x'Qx + q'x
 * with the default options (no Order, tol = 3*eps, maxiter = 4n).  The active
 * ("positive") set P grows by the variable with the largest scaled multiplier
 * w - wsc; the sub-problem on P is solved through a lower-triangular factor L
 * that is extended one row at a time (NQP.m:122-134) and truncated when a
 * variable leaves P (NQP.m:163-171).  A pivot below AA*tol is replaced by 1e300
 * (NQP.m:127-131).  Returns 0, or -1 when the iteration cap is exceeded (the
 * reference raises error() at NQP.m:116-119).
 * Q is n x n column-major.  x, w have n entries.  Work is O(n^2) doubles. */
int oracle_nqp(const double* Q, const double* q, i64 n, double* x, double* w_out, i64* iters_out)
{
    const double tol = 3.0 * DBL_EPSILON;
    const i64 maxiter = 4 * n;
    unsigned char* P = (unsigned char*)calloc((size_t)n, 1);
    double* z = (double*)calloc((size_t)n, sizeof(double));
    double* w = (double*)calloc((size_t)n, sizeof(double));
    double* b = (double*)calloc((size_t)n, sizeof(double));
    double* wsc = (double*)calloc((size_t)n, sizeof(double));
    double* L = (double*)calloc((size_t)(n * n), sizeof(double)); /* L[r + n*c], lower */
    double* t = (double*)calloc((size_t)n, sizeof(double));
    i64* pn = (i64*)calloc((size_t)n + 1, sizeof(i64));
    int status = 0;
    double wsc0 = 0.0;
    for (i64 k = 0; k < n; ++k) {
        x[k] = 0.0;
        w[k] = -q[k];
        b[k] = -q[k];
        wsc0 += w[k] * w[k];
    }
    wsc0 = sqrt(wsc0);
    i64 pn1 = 0, pn2 = 0, iter = 0;

    for (;;) {
        /* stop when every variable is positive or no multiplier exceeds its scale */
        int all_p = 1, any_up = 0;
        for (i64 k = 0; k < n; ++k) {
            if (!P[k]) {
                all_p = 0;
                if (w[k] > wsc[k]) any_up = 1;
            }
        }
        if (all_p || !any_up) break;
        /* add the variable with the largest w - wsc (first on ties) */
        i64 best = -1;
        double bv = 0.0;
        for (i64 k = 0; k < n; ++k) {
            if (P[k]) continue;
            double v = w[k] - wsc[k];
            if (best < 0 || v > bv) { best = k; bv = v; }
        }
        P[best] = 1;
        pn2 = pn1 + 1;
        pn[pn2 - 1] = best;

        for (;;) {
            ++iter;
            if (iter >= 2 * n) {
                if (iter > maxiter) { status = -1; goto done; }
                if (iter % n == 0)
                    for (i64 k = 0; k < n; ++k) wsc[k] = (wsc[k] + wsc0 * tol) * 2.0;
            }
            for (i64 k = 0; k < n; ++k) z[k] = 0.0;
            /* extend the factor with rows pn1 .. pn2-1 (0-based) */
            for (i64 r = pn1; r < pn2; ++r) {
                i64 vr = pn[r];
                for (i64 s = 0; s < r; ++s) {
                    double acc = Q[pn[s] + n * vr];
                    for (i64 u = 0; u < s; ++u) acc -= L[s + n * u] * t[u];
                    t[s] = acc / L[s + n * s];
                }
                double AA = Q[vr + n * vr];
                double tt = AA;
                for (i64 s = 0; s < r; ++s) tt -= t[s] * t[s];
                tt = (tt <= AA * tol) ? 1e300 : sqrt(tt);
                for (i64 s = 0; s < r; ++s) L[r + n * s] = t[s];
                L[r + n * r] = tt;
            }
            /* solve L L' z_P = b_P */
            for (i64 s = 0; s < pn2; ++s) {
                double acc = b[pn[s]];
                for (i64 u = 0; u < s; ++u) acc -= L[s + n * u] * t[u];
                t[s] = acc / L[s + n * s];
            }
            for (i64 s = pn2 - 1; s >= 0; --s) {
                double acc = t[s];
                for (i64 u = s + 1; u < pn2; ++u) acc -= L[u + n * s] * z[pn[u]];
                z[pn[s]] = acc / L[s + n * s];
            }
            pn1 = pn2;

            int all_pos = 1;
            for (i64 k = 0; k < n; ++k)
                if (P[k] && z[k] < 0.0) { all_pos = 0; break; }
            if (all_pos) {
                for (i64 k = 0; k < n; ++k) x[k] = z[k];
                for (i64 k = 0; k < n; ++k) {
                    double acc = b[k];
                    for (i64 u = 0; u < n; ++u) acc -= Q[k + n * u] * x[u];
                    w[k] = acc;
                }
                for (i64 k = 0; k < n; ++k)
                    if (P[k] && 2.0 * fabs(w[k]) > wsc[k]) wsc[k] = 2.0 * fabs(w[k]);
                break;
            }
            /* remove the variable that hits zero first along x -> z */
            i64 worst = -1;
            double alpha = 0.0;
            for (i64 k = 0; k < n; ++k) {
                if (!(z[k] < 0.0)) continue;
                double v = x[k] / (x[k] - z[k] + DBL_MIN);
                if (worst < 0 || v < alpha) { worst = k; alpha = v; }
            }
            if (x[worst] == 0.0) {
                double acc = b[worst];
                for (i64 u = 0; u < n; ++u) acc -= Q[worst + n * u] * x[u];
                wsc[worst] = (fabs(acc) + wsc[worst]) * 2.0;
                /* the reference refreshes the whole w here (NQP.m:153); only
                 * entry `worst` is read before the next full refresh */
                w[worst] = acc;
            }
            P[worst] = 0;
            for (i64 k = 0; k < n; ++k) x[k] = x[k] - alpha * (x[k] - z[k]);
            i64 pos = 0;
            while (pn[pos] != worst) ++pos;
            for (i64 s = pos; s + 1 < pn2; ++s) pn[s] = pn[s + 1];
            pn[pn2 - 1] = 0;
            pn1 = pos;
            pn2 = pn2 - 1;
        }
    }
done:
    if (w_out) for (i64 k = 0; k < n; ++k) w_out[k] = w[k];
    if (iters_out) *iters_out = iter;
    free(P); free(z); free(w); free(b); free(wsc); free(L); free(t); free(pn);
    return status;
}
