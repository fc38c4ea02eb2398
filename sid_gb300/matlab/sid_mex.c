/*
 * sid_mex.c -- MATLAB MEX gateway onto libsid (include/sid.h).
 *
 * Build (needs MATLAB R2018a+ with the Parallel Computing Toolbox headers and
 * the CUDA toolkit; not compiled in this repository's CI, which has no MATLAB):
 *   mex -R2018a -I<repo>/include sid_mex.c -L<repo>/sid_gb300/_build -lsid -lcudart
 *
 * Usage: sid_mex(command, ...) with command one of
 *   plan     = sid_mex('plan', H, CAindex, X, Y, flags)        CAindex may be []
 *   I        = sid_mex('forward', plan, V, method)
 *   B        = sid_mex('adjoint', plan, I, method)
 *   X        = sid_mex('isra', plan, Htf, Xguess, maxIter, lambda, method)
 *   X        = sid_mex('ls_deconv', plan, df, max_iter, lamb_L1, lamb_L2, method)
 *   X        = sid_mex('rl_poisson', plan, y, Xguess, maxIter, method)
 *   sid_mex('weak_fraction', plan, frac)
 *   [X, G]   = sid_mex('ls_nnls', A, Y, opts)
 *   [X, Q]   = sid_mex('fast_nnls', A, Y, opts)
 *   [S, T]   = sid_mex('t_update', Y, T, S, opts)        opts.active, opts.Y optional
 *   [S, T]   = sid_mex('s_update', Y, S, T, opts)        opts.Y, opts.hilf optional
 *   q        = sid_mex('quantile', x, p)
 *   [x, w, it] = sid_mex('nqp', Q, b)     Q n x n x B, b n x B double gpuArrays (n <= 32)
 *   [s, t, sd] = sid_mex('rank1_background', Y, maxIter)    rank_1_factorization + compute_std_image
 *   sid_mex('set_kernel', plan, kernel)                      neuron-kernel composition ([] removes)
 *   [keep, template] = sid_mex('merge_filters', timeseries, template, limit, bg_sub)
 *   n        = sid_mex('snr_order', traces, bg_sub)
 *   h        = sid_mex('pinv_create', F)                  F: K x P forward model
 *   T        = sid_mex('pinv_apply', h, Y, baseline)      baseline may be []
 *   sid_mex('pinv_destroy', h)
 *   [X, lam] = sid_mex('reconstruct', plan, img, microlenses, opts, method)
 *   [X, lam] = sid_mex('reconstruct_batch', plan, imgs, microlenses, opts, method)
 *              imgs X x Y x n, X X x Y x Z x n (groups of components per pass)
 *   [X, hist] = sid_mex('isra_ex', plan, Htf, Xguess, maxIter, mode, p, lambda, method)   mode 0 basic, 1 TV
 *   X        = sid_mex('ls_deconv_ex', plan, df, max_iter, lamb_L1, lamb_L2, lamb_TV_L2, lamb_TV_L1, method)
 *   F        = sid_mex('library_kernel', plan, centers, r, dim, kernel, method)   kernel [] for the ball;
 *              method 'direct' or 'spectral'; F n x P single gpuArray of L2-normalised rows
 *   F        = sid_mex('library', plan, recon, centers, neur_id, neur_rad, axial[, method])   recon: cell of
 *              volumes; method 'direct' (default, FP32 lenslet taps) or 'spectral' (tensor-core windows)
 *   Fm       = sid_mex('spatial_update', T, Y, template, opts)     template: logical (R - bg_sub) x P
 *   [xx, Q, df, h] = sid_mex('fast_nnls_ex', A, Y, opts, Q, df, h)  every fast_nnls input and output
 *   x        = sid_mex('reg_nnls', A, d, opts)                      A m x n, d m double gpuArrays
 *   sid_mex('destroy', plan)
 * Matrix arguments of the NNLS / NMF / extraction commands are single
 * gpuArrays (the movie Y may be half); results are gpuArrays.
 * gpuArray inputs use the device entry points directly (mxGPUArray); other
 * inputs go through the _host entry points.  A non-zero libsid status becomes a
 * MATLAB error with identifier 'sid:<command>' and sid_last_error() as text.
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "gpu/mxGPUArray.h"
#include "mex.h"
#include "sid.h"

#define MAX_PLANS 64
#define MAX_PINV 16
static sid_plan* g_plans[MAX_PLANS];
static sid_pinv* g_pinv[MAX_PINV];
static int64_t g_pinv_K[MAX_PINV];
static sid_ctx* g_ctx = NULL;

static double field_or(const mxArray* s, const char* name, double dflt);
static void check(int rc, const char* cmd);

static void cleanup(void)
{
    for (int i = 0; i < MAX_PLANS; ++i)
        if (g_plans[i]) {
            sid_plan_destroy(g_plans[i]);
            g_plans[i] = NULL;
        }
    for (int i = 0; i < MAX_PINV; ++i)
        if (g_pinv[i]) {
            sid_pinv_destroy(g_pinv[i]);
            g_pinv[i] = NULL;
        }
    if (g_ctx) {
        sid_ctx_destroy(g_ctx);
        g_ctx = NULL;
    }
}

static sid_ctx* ctx(const char* cmd)
{
    if (!g_ctx) check(sid_ctx_create(&g_ctx), cmd);
    return g_ctx;
}

/* single (or, where allowed, half) gpuArray argument */
static const mxGPUArray* gpu_arg(const mxArray* a, int allow_half, const char* cmd)
{
    if (!mxIsGPUArray(a)) mexErrMsgIdAndTxt("sid:type", "%s: gpuArray arguments expected", cmd);
    const mxGPUArray* g = mxGPUCreateFromMxArray(a);
    const mxClassID c = mxGPUGetClassID(g);
    if (c != mxSINGLE_CLASS && !(allow_half && c == mxUINT16_CLASS))
        mexErrMsgIdAndTxt("sid:type", "%s: single gpuArray expected", cmd);
    return g;
}

static int ydtype(const mxGPUArray* g) { return mxGPUGetClassID(g) == mxSINGLE_CLASS ? SID_DTYPE_F32 : SID_DTYPE_F16; }

static mxGPUArray* gpu_copy(const mxGPUArray* g)
{
    return mxGPUCopyGPUArray(g);
}

static void nmf_opts(const mxArray* o, sid_nmf_opts* out)
{
    sid_nmf_defaults(out);
    out->lamb_temp = field_or(o, "lamb_temp", 0.0);
    out->lamb_corr = field_or(o, "lamb_corr", 0.0);
    out->lamb_temp_TV = field_or(o, "lamb_temp_TV", 0.0);
    out->lamb_spat = field_or(o, "lamb_spat", 0.0);
    out->lamb_spat_TV = field_or(o, "lamb_spat_TV", 0.0);
    out->lamb_orth_L1 = field_or(o, "lamb_orth_L1", 0.0);
    out->lamb_orth_L2 = field_or(o, "lamb_orth_L2", 0.0);
    out->use_std = (int)field_or(o, "use_std", 0.0);
    out->pointwise = (int)field_or(o, "pointwise", 0.0);
}

static void check(int rc, const char* cmd)
{
    if (rc != SID_OK) {
        char id[64];
        snprintf(id, sizeof(id), "sid:%s", cmd);
        mexErrMsgIdAndTxt(id, "%s", sid_last_error());
    }
}

static sid_plan* plan_arg(const mxArray* a)
{
    const double h = mxGetScalar(a);
    const int i = (int)h;
    if (i < 0 || i >= MAX_PLANS || !g_plans[i]) mexErrMsgIdAndTxt("sid:plan", "invalid plan handle");
    return g_plans[i];
}

static int method_arg(int nrhs, const mxArray* prhs[], int pos)
{
    return (nrhs > pos) ? (int)mxGetScalar(prhs[pos]) : SID_METHOD_SPECTRAL_MIXED;
}

static double field_or(const mxArray* s, const char* name, double dflt)
{
    if (!s || !mxIsStruct(s)) return dflt;
    const mxArray* f = mxGetField(s, 0, name);
    return (f && !mxIsEmpty(f)) ? mxGetScalar(f) : dflt;
}

/* A microlens mask (double or logical, X*Y elements) as a uint8 host array
 * the caller destroys. */
static mxArray* mask_u8(const mxArray* a, mwSize n, const char* cmd)
{
    if (mxGetNumberOfElements(a) != n)
        mexErrMsgIdAndTxt("sid:type", "%s: microlenses must have the image's X*Y elements", cmd);
    if (!mxIsLogical(a) && !(mxIsDouble(a) && !mxIsComplex(a)))
        mexErrMsgIdAndTxt("sid:type", "%s: microlenses must be a real double or logical array", cmd);
    mxArray* t = mxCreateNumericMatrix(n, 1, mxUINT8_CLASS, mxREAL);
    uint8_t* dst = (uint8_t*)mxGetData(t);
    if (mxIsLogical(a)) {
        const mxLogical* src = mxGetLogicals(a);
        for (mwSize i = 0; i < n; ++i) dst[i] = src[i] ? 1 : 0;
    } else {
        const double* src = mxGetPr(a);
        for (mwSize i = 0; i < n; ++i) dst[i] = src[i] != 0.0;
    }
    return t;
}

/* out = f(plan, in) for a single-precision array, on the device or the host */
/* Elements of the plan's volume (what = 'v': X*Y*Z) or sensor image ('i': X*Y). */
static mwSize plan_numel(const sid_plan* p, char what)
{
    int64_t info[14];
    sid_plan_info(p, info);
    return (mwSize)(info[3] * info[4] * (what == 'v' ? info[2] : 1));
}

/* A device argument must hold exactly n elements: the kernels read that many. */
static void need_numel(const mxGPUArray* g, mwSize n, const char* cmd, const char* what)
{
    if (mxGPUGetNumberOfElements(g) != n)
        mexErrMsgIdAndTxt("sid:type", "%s: %s has %llu elements, the plan needs %llu", cmd, what,
                          (unsigned long long)mxGPUGetNumberOfElements(g), (unsigned long long)n);
}

typedef int (*dev_fn)(sid_plan*, int, const float*, float*, void*);
typedef int (*host_fn)(sid_plan*, int, const float*, float*);

static mxArray* project(sid_plan* p, int method, const mxArray* in, mwSize in_n, mwSize nd, const mwSize* dims,
                        dev_fn fd, host_fn fh, const char* cmd)
{
    if (mxIsGPUArray(in)) {
        const mxGPUArray* gin = mxGPUCreateFromMxArray(in);
        if (mxGPUGetClassID(gin) != mxSINGLE_CLASS || mxGPUGetNumberOfElements(gin) != in_n) {
            mxGPUDestroyGPUArray(gin);
            mexErrMsgIdAndTxt("sid:type", "%s: input must be a single array of the plan's size", cmd);
        }
        mxGPUArray* gout = mxGPUCreateGPUArray(nd, dims, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = fd(p, method, (const float*)mxGPUGetDataReadOnly(gin), (float*)mxGPUGetData(gout), NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(gin);
        check(rc, cmd);
        mxArray* out = mxGPUCreateMxArrayOnGPU(gout);
        mxGPUDestroyGPUArray(gout);
        return out;
    }
    if (!mxIsSingle(in)) mexErrMsgIdAndTxt("sid:type", "%s: input must be single", cmd);
    if (mxGetNumberOfElements(in) != in_n) mexErrMsgIdAndTxt("sid:type", "%s: input has the wrong size for the plan", cmd);
    mxArray* out = mxCreateNumericArray(nd, dims, mxSINGLE_CLASS, mxREAL);
    check(fh(p, method, (const float*)mxGetData(in), (float*)mxGetData(out)), cmd);
    return out;
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[])
{
    char cmd[32];
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof(cmd)) != 0)
        mexErrMsgIdAndTxt("sid:usage", "sid_mex(command, ...)");
    mxInitGPU();
    mexAtExit(cleanup);

    if (!strcmp(cmd, "plan")) {
        const mxArray* H = prhs[1];
        if (!mxIsSingle(H) || mxGetNumberOfDimensions(H) < 4) mexErrMsgIdAndTxt("sid:plan", "H must be single M x M x N x N x Z");
        const mwSize* d = mxGetDimensions(H);
        if (d[0] != d[1] || d[2] != d[3]) mexErrMsgIdAndTxt("sid:plan", "H must be single M x M x N x N x Z");
        const int64_t Z = mxGetNumberOfDimensions(H) > 4 ? (int64_t)d[4] : 1;
        int32_t* ca = NULL;
        int32_t cabuf[2 * 4096];
        if (!mxIsEmpty(prhs[2])) {
            if (!mxIsDouble(prhs[2]) || mxIsComplex(prhs[2]) || Z > 4096 ||
                mxGetNumberOfElements(prhs[2]) != (mwSize)(2 * Z))
                mexErrMsgIdAndTxt("sid:plan", "CAindex must be a real Z x 2 double array (Z <= 4096)");
            const double* c = mxGetPr(prhs[2]);
            for (int64_t i = 0; i < 2 * Z && i < 2 * 4096; ++i) cabuf[i] = (int32_t)c[i];
            ca = cabuf;
        }
        int slot = -1;
        for (int i = 0; i < MAX_PLANS; ++i)
            if (!g_plans[i]) { slot = i; break; }
        if (slot < 0) mexErrMsgIdAndTxt("sid:plan", "too many plans");
        const int flags = nrhs > 5 ? (int)mxGetScalar(prhs[5]) : (SID_PLAN_SPECTRAL_I16 | SID_PLAN_SPECTRAL_F24);
        check(sid_plan_create((const float*)mxGetData(H), (int64_t)d[0], (int64_t)d[2], Z, ca,
                              (int64_t)mxGetScalar(prhs[3]), (int64_t)mxGetScalar(prhs[4]), flags, &g_plans[slot]),
              cmd);
        plhs[0] = mxCreateDoubleScalar((double)slot);
        return;
    }
    if (!strcmp(cmd, "destroy")) {
        const int i = (int)mxGetScalar(prhs[1]);
        if (i >= 0 && i < MAX_PLANS && g_plans[i]) {
            sid_plan_destroy(g_plans[i]);
            g_plans[i] = NULL;
        }
        return;
    }
    if (!strcmp(cmd, "forward") || !strcmp(cmd, "adjoint")) {
        sid_plan* p = plan_arg(prhs[1]);
        int64_t info[14];
        sid_plan_info(p, info);
        const int fwd = !strcmp(cmd, "forward");
        mwSize dims[3] = {(mwSize)info[3], (mwSize)info[4], (mwSize)info[2]};
        const mwSize in_n = (mwSize)(info[3] * info[4] * (fwd ? info[2] : 1));
        plhs[0] = project(p, method_arg(nrhs, prhs, 3), prhs[2], in_n, fwd ? 2 : 3, dims,
                          fwd ? sid_forward : sid_adjoint, fwd ? sid_forward_host : sid_adjoint_host, cmd);
        return;
    }
    if (!strcmp(cmd, "isra")) {
        sid_plan* p = plan_arg(prhs[1]);
        if (!mxIsSingle(prhs[2]) || !mxIsSingle(prhs[3])) mexErrMsgIdAndTxt("sid:type", "isra: single inputs");
        int64_t info[14];
        sid_plan_info(p, info);
        if (mxGetNumberOfElements(prhs[2]) != (mwSize)(info[3] * info[4] * info[2]) ||
            mxGetNumberOfElements(prhs[3]) != (mwSize)(info[3] * info[4] * info[2]))
            mexErrMsgIdAndTxt("sid:type", "isra: Htf and Xguess must be X x Y x Z volumes of the plan");
        plhs[0] = mxDuplicateArray(prhs[3]);
        check(sid_deconv_isra_host(p, method_arg(nrhs, prhs, 6), (const float*)mxGetData(prhs[2]),
                                   (float*)mxGetData(plhs[0]), (int)mxGetScalar(prhs[4]), (float)mxGetScalar(prhs[5])),
              cmd);
        return;
    }
    if (!strcmp(cmd, "ls_nnls") || !strcmp(cmd, "fast_nnls")) {
        /* A: P x K single gpuArray, Y: P x F single or half gpuArray */
        if (!g_ctx) check(sid_ctx_create(&g_ctx), cmd);
        const mxGPUArray* A = mxGPUCreateFromMxArray(prhs[1]);
        const mxGPUArray* Y = mxGPUCreateFromMxArray(prhs[2]);
        const mwSize* da = mxGPUGetDimensions(A);
        const mwSize* dy = mxGPUGetDimensions(Y);
        const int64_t P = (int64_t)da[0], K = (int64_t)da[1], F = (int64_t)dy[1];
        const int ydt = mxGPUGetClassID(Y) == mxSINGLE_CLASS ? SID_DTYPE_F32 : SID_DTYPE_F16;
        const mxArray* o = nrhs > 3 ? prhs[3] : NULL;
        sid_nnls_opts opts;
        int ls = !strcmp(cmd, "ls_nnls");
        if (ls) sid_ls_nnls_defaults(&opts); else sid_fast_nnls_defaults(&opts);
        opts.lambda = field_or(o, "lambda", opts.lambda);
        opts.sample = (int64_t)field_or(o, "sample", (double)opts.sample);
        opts.tol = field_or(o, "tol", opts.tol);
        opts.tol_ = field_or(o, "tol_", opts.tol_);
        opts.max_iter = (int64_t)field_or(o, "max_iter", (double)opts.max_iter);
        opts.use_std = (int)field_or(o, "use_std", 0);
        opts.tol_p = (int)field_or(o, "tol_p", 1);
        mwSize dx[2] = {(mwSize)K, (mwSize)F}, dg[2] = {(mwSize)K, (mwSize)K};
        mxGPUArray* X = mxGPUCreateGPUArray(2, dx, mxSINGLE_CLASS, mxREAL, MX_GPU_INITIALIZE_VALUES);
        mxGPUArray* G = mxGPUCreateGPUArray(2, dg, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc;
        if (ls)
            rc = sid_ls_nnls(g_ctx, (const float*)mxGPUGetDataReadOnly(A), mxGPUGetDataReadOnly(Y), ydt, P, K, F,
                             &opts, (float*)mxGPUGetData(G), 0, (float*)mxGPUGetData(X), 0, SID_PREC_SPLIT, NULL,
                             NULL);
        else
            rc = sid_fast_nnls(g_ctx, (const float*)mxGPUGetDataReadOnly(A), mxGPUGetDataReadOnly(Y), ydt, P, K, F,
                               &opts, NULL, (float*)mxGPUGetData(X), (float*)mxGPUGetData(G), SID_PREC_SPLIT, NULL,
                               NULL);
        mxGPUDestroyGPUArray(A);
        mxGPUDestroyGPUArray(Y);
        if (rc != SID_OK) {
            mxGPUDestroyGPUArray(X);
            mxGPUDestroyGPUArray(G);
            check(rc, cmd);
        }
        plhs[0] = mxGPUCreateMxArrayOnGPU(X);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(G);
        mxGPUDestroyGPUArray(X);
        mxGPUDestroyGPUArray(G);
        return;
    }
    if (!strcmp(cmd, "ls_deconv")) {
        /* X = sid_mex('ls_deconv', plan, df, max_iter, lamb_L1, lamb_L2, method): df single, host or gpuArray;
         * the result lives where df did */
        sid_plan* p = plan_arg(prhs[1]);
        const int method = method_arg(nrhs, prhs, 6);
        const int on_gpu = mxIsGPUArray(prhs[2]);
        if (!on_gpu && !mxIsSingle(prhs[2])) mexErrMsgIdAndTxt("sid:type", "ls_deconv: df must be single");
        const mxGPUArray* df = mxGPUCreateFromMxArray(prhs[2]); /* host arrays are copied to the device */
        if (mxGPUGetClassID(df) != mxSINGLE_CLASS) mexErrMsgIdAndTxt("sid:type", "ls_deconv: df must be single");
        mxGPUArray* X = gpu_copy(df);
        mxGPUDestroyGPUArray(df);
        int rc = sid_deconv_ls(p, method, (float*)mxGPUGetData(X), (int)mxGetScalar(prhs[3]),
                               (float)mxGetScalar(prhs[4]), (float)mxGetScalar(prhs[5]), NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        if (rc != SID_OK) mxGPUDestroyGPUArray(X);
        check(rc, cmd);
        plhs[0] = on_gpu ? mxGPUCreateMxArrayOnGPU(X) : mxGPUCreateMxArrayOnCPU(X);
        mxGPUDestroyGPUArray(X);
        return;
    }
    if (!strcmp(cmd, "rl_poisson")) {
        /* X = sid_mex('rl_poisson', plan, y, Xguess, maxIter, method): y (X x Y) and Xguess (X x Y x Z)
         * single, host or gpuArray; the result lives where Xguess did */
        sid_plan* p = plan_arg(prhs[1]);
        const int method = method_arg(nrhs, prhs, 5);
        const int on_gpu = mxIsGPUArray(prhs[3]);
        const mxGPUArray* y = mxGPUCreateFromMxArray(prhs[2]);
        const mxGPUArray* x0 = mxGPUCreateFromMxArray(prhs[3]);
        if (mxGPUGetClassID(y) != mxSINGLE_CLASS || mxGPUGetClassID(x0) != mxSINGLE_CLASS)
            mexErrMsgIdAndTxt("sid:type", "rl_poisson: y and Xguess must be single");
        mxGPUArray* X = gpu_copy(x0);
        mxGPUDestroyGPUArray(x0);
        int rc = sid_deconv_rl_poisson(p, method, (const float*)mxGPUGetDataReadOnly(y), (float*)mxGPUGetData(X),
                                       (int)mxGetScalar(prhs[4]), NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(y);
        if (rc != SID_OK) mxGPUDestroyGPUArray(X);
        check(rc, cmd);
        plhs[0] = on_gpu ? mxGPUCreateMxArrayOnGPU(X) : mxGPUCreateMxArrayOnCPU(X);
        mxGPUDestroyGPUArray(X);
        return;
    }
    if (!strcmp(cmd, "weak_fraction")) {
        /* sid_mex('weak_fraction', plan, frac) */
        check(sid_plan_set_weak_fraction(plan_arg(prhs[1]), mxGetScalar(prhs[2])), cmd);
        return;
    }
    if (!strcmp(cmd, "t_update") || !strcmp(cmd, "s_update")) {
        /* [S, T] = sid_mex('t_update', Y, T, S, opts)  /  [S, T] = sid_mex('s_update', Y, S, T, opts) */
        const int tu = !strcmp(cmd, "t_update");
        const mxArray* o = nrhs > 4 ? prhs[4] : NULL;
        const mxGPUArray* Y = gpu_arg(prhs[1], 1, cmd);
        const mxGPUArray* A1 = gpu_arg(prhs[2], 0, cmd); /* T (t_update) or S (s_update) */
        const mxGPUArray* A2 = gpu_arg(prhs[3], 0, cmd);
        mxGPUArray* T = gpu_copy(tu ? A1 : A2);
        mxGPUArray* S = gpu_copy(tu ? A2 : A1);
        const mwSize* ds = mxGPUGetDimensions(S);
        const mwSize* dt = mxGPUGetDimensions(T);
        const int64_t P = (int64_t)ds[0], R = (int64_t)ds[1], F = (int64_t)dt[1];
        sid_nmf_opts no;
        nmf_opts(o, &no);
        const mxGPUArray *act = NULL, *ym = NULL, *hl = NULL;
        mxArray* tmp_act = NULL;
        if (o && mxIsStruct(o)) {
            const mxArray* f;
            if (tu && (f = mxGetField(o, 0, "active")) && !mxIsEmpty(f)) {
                /* logical P-vector -> uint8 gpuArray */
                if (!mxIsLogical(f) || mxGetNumberOfElements(f) != (mwSize)P)
                    mexErrMsgIdAndTxt("sid:type", "%s: opts.active must be a logical vector of P elements", cmd);
                tmp_act = mxCreateNumericMatrix((mwSize)P, 1, mxUINT8_CLASS, mxREAL);
                const mxLogical* src = mxGetLogicals(f);
                uint8_t* dst = (uint8_t*)mxGetData(tmp_act);
                for (int64_t i = 0; i < P; ++i) dst[i] = src[i] ? 1 : 0;
                act = mxGPUCreateFromMxArray(tmp_act);
            }
            if ((f = mxGetField(o, 0, "Y")) && !mxIsEmpty(f) && no.use_std) ym = mxGPUCreateFromMxArray(f);
            if (!tu && (f = mxGetField(o, 0, "hilf")) && !mxIsEmpty(f)) hl = mxGPUCreateFromMxArray(f);
        }
        int rc;
        if (tu)
            rc = sid_t_update(ctx(cmd), mxGPUGetDataReadOnly(Y), ydtype(Y), (float*)mxGPUGetData(T),
                              (float*)mxGPUGetData(S), P, R, F, act ? (const uint8_t*)mxGPUGetDataReadOnly(act) : NULL,
                              ym ? (const float*)mxGPUGetDataReadOnly(ym) : NULL, &no, SID_PREC_SPLIT, NULL);
        else
            rc = sid_s_update(ctx(cmd), mxGPUGetDataReadOnly(Y), ydtype(Y), (float*)mxGPUGetData(S),
                              (float*)mxGPUGetData(T), P, R, F, ym ? (const float*)mxGPUGetDataReadOnly(ym) : NULL,
                              hl ? (const float*)mxGPUGetDataReadOnly(hl) : NULL, &no, SID_PREC_SPLIT, NULL);
        if (rc == SID_OK) rc = sid_ctx_sync(g_ctx, NULL);
        mxGPUDestroyGPUArray(Y);
        mxGPUDestroyGPUArray(A1);
        mxGPUDestroyGPUArray(A2);
        if (act) mxGPUDestroyGPUArray(act);
        if (tmp_act) mxDestroyArray(tmp_act);
        if (ym) mxGPUDestroyGPUArray(ym);
        if (hl) mxGPUDestroyGPUArray(hl);
        if (rc != SID_OK) {
            mxGPUDestroyGPUArray(S);
            mxGPUDestroyGPUArray(T);
            check(rc, cmd);
        }
        plhs[0] = mxGPUCreateMxArrayOnGPU(S);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(T);
        mxGPUDestroyGPUArray(S);
        mxGPUDestroyGPUArray(T);
        return;
    }
    if (!strcmp(cmd, "rank1_background")) {
        /* [bg_spatial, bg_temporal, std_image] = sid_mex('rank1_background', Y, maxIter):
         * Y P x F single or half gpuArray; std_image computed in the last pass */
        const mxGPUArray* Y = gpu_arg(prhs[1], 1, cmd);
        const mwSize* dy = mxGPUGetDimensions(Y);
        const int64_t P = (int64_t)dy[0], F = (int64_t)dy[1];
        mwSize ds[2] = {(mwSize)P, 1}, dt[2] = {1, (mwSize)F};
        mxGPUArray* s_ = mxGPUCreateGPUArray(2, ds, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* t_ = mxGPUCreateGPUArray(2, dt, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* sd = nlhs > 2 ? mxGPUCreateGPUArray(2, ds, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE) : NULL;
        int rc = sid_rank1_background(ctx(cmd), mxGPUGetDataReadOnly(Y), ydtype(Y), P, F, (int)mxGetScalar(prhs[2]),
                                      (float*)mxGPUGetData(s_), (float*)mxGPUGetData(t_),
                                      sd ? (float*)mxGPUGetData(sd) : NULL, NULL);
        if (rc == SID_OK) rc = sid_ctx_sync(g_ctx, NULL);
        mxGPUDestroyGPUArray(Y);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(s_);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(t_);
        if (sd) plhs[2] = mxGPUCreateMxArrayOnGPU(sd);
        mxGPUDestroyGPUArray(s_);
        mxGPUDestroyGPUArray(t_);
        if (sd) mxGPUDestroyGPUArray(sd);
        return;
    }
    if (!strcmp(cmd, "set_kernel")) {
        /* sid_mex('set_kernel', plan, kernel): kernel single (host) 3-D, [] removes it */
        sid_plan* p = plan_arg(prhs[1]);
        const mxArray* k = prhs[2];
        if (mxIsEmpty(k)) {
            check(sid_plan_set_kernel(p, NULL, 0, 0, 0), cmd);
            return;
        }
        if (!mxIsSingle(k)) mexErrMsgIdAndTxt("sid:type", "set_kernel: single kernel expected");
        const mwSize nd = mxGetNumberOfDimensions(k);
        const mwSize* d = mxGetDimensions(k);
        check(sid_plan_set_kernel(p, (const float*)mxGetData(k), (int64_t)d[0], nd > 1 ? (int64_t)d[1] : 1,
                                  nd > 2 ? (int64_t)d[2] : 1), cmd);
        return;
    }
    if (!strcmp(cmd, "merge_filters")) {
        /* keep = sid_mex('merge_filters', timeseries, template, limit, bg_sub): K x F and
         * (K - bg_sub) x P single gpuArrays; template merged in place (returned as the
         * second output); keep: logical K x 1 of the surviving rows */
        const mxGPUArray* ts = gpu_arg(prhs[1], 0, cmd);
        const mxGPUArray* t0 = gpu_arg(prhs[2], 0, cmd);
        mxGPUArray* tp = gpu_copy(t0);
        mxGPUDestroyGPUArray(t0);
        const mwSize* dt = mxGPUGetDimensions(ts);
        const mwSize* dp = mxGPUGetDimensions(tp);
        const int64_t K = (int64_t)dt[0], F = (int64_t)dt[1], P = (int64_t)dp[1];
        plhs[0] = mxCreateNumericMatrix((mwSize)K, 1, mxINT32_CLASS, mxREAL);
        const int rc = sid_merge_filters(ctx(cmd), (const float*)mxGPUGetDataReadOnly(ts), K, F, (float*)mxGPUGetData(tp),
                                         P, mxGetScalar(prhs[3]), (int)mxGetScalar(prhs[4]), (int32_t*)mxGetData(plhs[0]),
                                         NULL);
        mxGPUDestroyGPUArray(ts);
        if (rc != SID_OK) mxGPUDestroyGPUArray(tp);
        check(rc, cmd);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(tp);
        mxGPUDestroyGPUArray(tp);
        return;
    }
    if (!strcmp(cmd, "snr_order")) {
        /* n = sid_mex('snr_order', traces, bg_sub): traces K x F single gpuArray; n 1-based */
        const mxGPUArray* tr = gpu_arg(prhs[1], 0, cmd);
        const mwSize* d = mxGPUGetDimensions(tr);
        plhs[0] = mxCreateNumericMatrix(1, d[0], mxINT32_CLASS, mxREAL);
        int32_t* o = (int32_t*)mxGetData(plhs[0]);
        const int rc = sid_snr_order(ctx(cmd), (const float*)mxGPUGetDataReadOnly(tr), (int64_t)d[0], (int64_t)d[1],
                                     (int)mxGetScalar(prhs[2]), o, NULL);
        mxGPUDestroyGPUArray(tr);
        check(rc, cmd);
        for (mwSize i = 0; i < d[0]; ++i) o[i] += 1;
        return;
    }
    if (!strcmp(cmd, "nqp")) {
        /* [x, w, it] = sid_mex('nqp', Q, b): B independent NQPs (NQP.m:42-178) */
        if (!mxIsGPUArray(prhs[1]) || !mxIsGPUArray(prhs[2]))
            mexErrMsgIdAndTxt("sid:type", "%s: gpuArray arguments expected", cmd);
        const mxGPUArray* Q = mxGPUCreateFromMxArray(prhs[1]);
        const mxGPUArray* b = mxGPUCreateFromMxArray(prhs[2]);
        if (mxGPUGetClassID(Q) != mxDOUBLE_CLASS || mxGPUGetClassID(b) != mxDOUBLE_CLASS)
            mexErrMsgIdAndTxt("sid:type", "%s: double gpuArrays expected", cmd);
        const mwSize* dq = mxGPUGetDimensions(Q);
        const mwSize n = dq[0];
        const mwSize B = (mwSize)(mxGPUGetNumberOfElements(b) / (n ? n : 1));
        const mwSize dx[2] = {n, B}, di[2] = {1, B};
        mxGPUArray* x = mxGPUCreateGPUArray(2, dx, mxDOUBLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* w = mxGPUCreateGPUArray(2, dx, mxDOUBLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* it = mxGPUCreateGPUArray(2, di, mxINT32_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        const int rc = sid_nqp_batched(ctx(cmd), (const double*)mxGPUGetDataReadOnly(Q),
                                       (const double*)mxGPUGetDataReadOnly(b), (int)n, (int64_t)B,
                                       (double*)mxGPUGetData(x), (double*)mxGPUGetData(w), (int32_t*)mxGPUGetData(it),
                                       NULL, NULL);
        plhs[0] = mxGPUCreateMxArrayOnGPU(x);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(w);
        if (nlhs > 2) plhs[2] = mxGPUCreateMxArrayOnGPU(it);
        mxGPUDestroyGPUArray(Q);
        mxGPUDestroyGPUArray(b);
        mxGPUDestroyGPUArray(x);
        mxGPUDestroyGPUArray(w);
        mxGPUDestroyGPUArray(it);
        check(rc, cmd);
        return;
    }
    if (!strcmp(cmd, "quantile")) {
        /* q = sid_mex('quantile', x, p): x single gpuArray, p double vector */
        const mxGPUArray* x = gpu_arg(prhs[1], 0, cmd);
        if (!mxIsDouble(prhs[2]) || mxIsComplex(prhs[2]))
            mexErrMsgIdAndTxt("sid:type", "quantile: p must be a real double vector");
        const int np = (int)mxGetNumberOfElements(prhs[2]);
        plhs[0] = mxCreateDoubleMatrix(1, (mwSize)np, mxREAL);
        const int rc = sid_quantile(ctx(cmd), (const float*)mxGPUGetDataReadOnly(x),
                                    (int64_t)mxGPUGetNumberOfElements(x), NULL, mxGetPr(prhs[2]), np,
                                    mxGetPr(plhs[0]), NULL);
        mxGPUDestroyGPUArray(x);
        check(rc, cmd);
        return;
    }
    if (!strcmp(cmd, "pinv_create")) {
        /* h = sid_mex('pinv_create', F): F K x P single gpuArray (the forward model) */
        const mxGPUArray* F = gpu_arg(prhs[1], 0, cmd);
        const mwSize* d = mxGPUGetDimensions(F);
        int slot = -1;
        for (int i = 0; i < MAX_PINV; ++i)
            if (!g_pinv[i]) { slot = i; break; }
        if (slot < 0) {
            mxGPUDestroyGPUArray(F);
            mexErrMsgIdAndTxt("sid:pinv", "too many extraction handles");
        }
        const int rc = sid_pinv_create(ctx(cmd), (const float*)mxGPUGetDataReadOnly(F), (int64_t)d[0],
                                       (int64_t)d[1], 0, SID_PREC_SPLIT, &g_pinv[slot], NULL);
        g_pinv_K[slot] = (int64_t)d[0];
        mxGPUDestroyGPUArray(F);
        check(rc, cmd);
        plhs[0] = mxCreateDoubleScalar((double)slot);
        return;
    }
    if (!strcmp(cmd, "pinv_apply")) {
        /* T = sid_mex('pinv_apply', h, Y, baseline): Y P x n single/half gpuArray, baseline n single gpuArray or [] */
        const int h = (int)mxGetScalar(prhs[1]);
        if (h < 0 || h >= MAX_PINV || !g_pinv[h]) mexErrMsgIdAndTxt("sid:pinv", "invalid extraction handle");
        const mxGPUArray* Y = gpu_arg(prhs[2], 1, cmd);
        const mwSize* dy = mxGPUGetDimensions(Y);
        const int64_t n = (int64_t)dy[1];
        const mxGPUArray* b = (nrhs > 3 && !mxIsEmpty(prhs[3])) ? gpu_arg(prhs[3], 0, cmd) : NULL;
        mwSize dt[2] = {(mwSize)g_pinv_K[h], (mwSize)n};
        mxGPUArray* T = mxGPUCreateGPUArray(2, dt, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = sid_pinv_apply(g_pinv[h], mxGPUGetDataReadOnly(Y), ydtype(Y), n,
                                b ? (const float*)mxGPUGetDataReadOnly(b) : NULL, (float*)mxGPUGetData(T),
                                g_pinv_K[h], NULL);
        if (rc == SID_OK) rc = sid_ctx_sync(g_ctx, NULL);
        mxGPUDestroyGPUArray(Y);
        if (b) mxGPUDestroyGPUArray(b);
        if (rc != SID_OK) mxGPUDestroyGPUArray(T);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(T);
        mxGPUDestroyGPUArray(T);
        return;
    }
    if (!strcmp(cmd, "pinv_destroy")) {
        const int h = (int)mxGetScalar(prhs[1]);
        if (h >= 0 && h < MAX_PINV && g_pinv[h]) {
            sid_pinv_destroy(g_pinv[h]);
            g_pinv[h] = NULL;
        }
        return;
    }
    if (!strcmp(cmd, "reconstruct_batch")) {
        /* [X, lam] = sid_mex('reconstruct_batch', plan, imgs, microlenses, opts, method): imgs X x Y x n single
         * gpuArray (one component image per slice); X: X x Y x Z x n, lam: n x 1 */
        sid_plan* p = plan_arg(prhs[1]);
        const mxGPUArray* imgs = gpu_arg(prhs[2], 0, cmd);
        const mxGPUArray* ml = NULL;
        mxArray* tmp_ml = NULL;
        if (nrhs > 3 && !mxIsEmpty(prhs[3])) {
            int64_t pinfo[14];
            sid_plan_info(p, pinfo);
            tmp_ml = mask_u8(prhs[3], (mwSize)(pinfo[3] * pinfo[4]), cmd);
            ml = mxGPUCreateFromMxArray(tmp_ml);
        }
        const mxArray* o = nrhs > 4 ? prhs[4] : NULL;
        sid_recon_opts ro;
        sid_recon_defaults(&ro);
        ro.q = field_or(o, "q", ro.q);
        ro.lamb_L1 = field_or(o, "lamb_L1", ro.lamb_L1);
        ro.lamb_L2 = field_or(o, "lamb_L2", ro.lamb_L2);
        ro.max_iter = (int)field_or(o, "max_iter", ro.max_iter);
        if (o && mxIsStruct(o)) {
            const mxArray* w = mxGetField(o, 0, "whichSolver");
            char sv[16] = "fast_nnls";
            if (w && mxIsChar(w)) mxGetString(w, sv, sizeof(sv));
            ro.solver = !strcmp(sv, "ISRA") ? 1 : 0;
        }
        int64_t info[14];
        sid_plan_info(p, info);
        const int64_t nI = info[3] * info[4], nV = nI * info[2];
        const mwSize ne = mxGPUGetNumberOfElements(imgs);
        if (ne % (mwSize)nI != 0) mexErrMsgIdAndTxt("sid:reconstruct_batch", "imgs must be X x Y x n");
        const int64_t nc = (int64_t)(ne / (mwSize)nI);
        mwSize dv[4] = {(mwSize)info[3], (mwSize)info[4], (mwSize)info[2], (mwSize)nc};
        mxGPUArray* X = mxGPUCreateGPUArray(4, dv, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        const float** ip = (const float**)mxMalloc((size_t)nc * sizeof(float*));
        float** xp = (float**)mxMalloc((size_t)nc * sizeof(float*));
        double* lam = (double*)mxMalloc((size_t)nc * sizeof(double));
        const float* ib = (const float*)mxGPUGetDataReadOnly(imgs);
        float* xb = (float*)mxGPUGetData(X);
        for (int64_t c = 0; c < nc; ++c) {
            ip[c] = ib + c * nI;
            xp[c] = xb + c * nV;
        }
        int rc = sid_reconstruct_components(p, method_arg(nrhs, prhs, 5), nc, ip,
                                            ml ? (const uint8_t*)mxGPUGetDataReadOnly(ml) : NULL, &ro, xp, lam, NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(imgs);
        if (ml) mxGPUDestroyGPUArray(ml);
        if (tmp_ml) mxDestroyArray(tmp_ml);
        mxFree(ip);
        mxFree(xp);
        if (rc != SID_OK) {
            mxFree(lam);
            mxGPUDestroyGPUArray(X);
        }
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(X);
        if (nlhs > 1) {
            plhs[1] = mxCreateDoubleMatrix((mwSize)nc, 1, mxREAL);
            for (int64_t c = 0; c < nc; ++c) mxGetPr(plhs[1])[c] = lam[c];
        }
        mxFree(lam);
        mxGPUDestroyGPUArray(X);
        return;
    }
    if (!strcmp(cmd, "reconstruct")) {
        /* [X, lam] = sid_mex('reconstruct', plan, img, microlenses, opts, method): img X x Y single gpuArray */
        sid_plan* p = plan_arg(prhs[1]);
        const mxGPUArray* img = gpu_arg(prhs[2], 0, cmd);
        need_numel(img, plan_numel(p, 'i'), cmd, "img");
        const mxGPUArray* ml = NULL;
        mxArray* tmp_ml = NULL;
        if (nrhs > 3 && !mxIsEmpty(prhs[3])) {
            int64_t pinfo[14];
            sid_plan_info(p, pinfo);
            tmp_ml = mask_u8(prhs[3], (mwSize)(pinfo[3] * pinfo[4]), cmd);
            ml = mxGPUCreateFromMxArray(tmp_ml);
        }
        const mxArray* o = nrhs > 4 ? prhs[4] : NULL;
        sid_recon_opts ro;
        sid_recon_defaults(&ro);
        ro.q = field_or(o, "q", ro.q);
        ro.lamb_L1 = field_or(o, "lamb_L1", ro.lamb_L1);
        ro.lamb_L2 = field_or(o, "lamb_L2", ro.lamb_L2);
        ro.max_iter = (int)field_or(o, "max_iter", ro.max_iter);
        if (o && mxIsStruct(o)) {
            const mxArray* w = mxGetField(o, 0, "whichSolver");
            char sv[16] = "fast_nnls";
            if (w && mxIsChar(w)) mxGetString(w, sv, sizeof(sv));
            ro.solver = !strcmp(sv, "ISRA") ? 1 : 0;
        }
        int64_t info[14];
        sid_plan_info(p, info);
        mwSize dv[3] = {(mwSize)info[3], (mwSize)info[4], (mwSize)info[2]};
        mxGPUArray* X = mxGPUCreateGPUArray(3, dv, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        double lam = 0.0;
        int rc = sid_reconstruct_component(p, method_arg(nrhs, prhs, 5), (const float*)mxGPUGetDataReadOnly(img),
                                           ml ? (const uint8_t*)mxGPUGetDataReadOnly(ml) : NULL, &ro,
                                           (float*)mxGPUGetData(X), &lam, NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(img);
        if (ml) mxGPUDestroyGPUArray(ml);
        if (tmp_ml) mxDestroyArray(tmp_ml);
        if (rc != SID_OK) mxGPUDestroyGPUArray(X);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(X);
        if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(lam);
        mxGPUDestroyGPUArray(X);
        return;
    }
    if (!strcmp(cmd, "isra_ex")) {
        /* [X, hist] = sid_mex('isra_ex', plan, Htf, Xguess, maxIter, mode, p, lambda, method): Htf, Xguess single
         * gpuArrays; lambda a scalar ('basic') or 1 x 3 ('TV') */
        sid_plan* p = plan_arg(prhs[1]);
        const mxGPUArray* htf = gpu_arg(prhs[2], 0, cmd);
        const mxGPUArray* x0 = gpu_arg(prhs[3], 0, cmd);
        need_numel(htf, plan_numel(p, 'v'), cmd, "Htf");
        need_numel(x0, plan_numel(p, 'v'), cmd, "Xguess");
        const int maxIter = (int)mxGetScalar(prhs[4]);
        const int mode = (int)mxGetScalar(prhs[5]);
        const int pn = (int)mxGetScalar(prhs[6]);
        float lam3[3] = {0.f, 0.f, 0.f};
        const mwSize nl = mxGetNumberOfElements(prhs[7]);
        if (nl && (!mxIsDouble(prhs[7]) || mxIsComplex(prhs[7])))
            mexErrMsgIdAndTxt("sid:type", "isra_ex: the TV weights must be a real double vector");
        for (mwSize i = 0; i < nl && i < 3; ++i) lam3[i] = (float)mxGetPr(prhs[7])[i];
        mxGPUArray* X = gpu_copy(x0);
        mxGPUArray* hist = NULL;
        if (nlhs > 1) {
            int64_t info[14];
            sid_plan_info(p, info);
            mwSize dh[4] = {(mwSize)maxIter, (mwSize)info[3], (mwSize)info[4], (mwSize)info[2]};
            hist = mxGPUCreateGPUArray(4, dh, mxSINGLE_CLASS, mxREAL, MX_GPU_INITIALIZE_VALUES);
        }
        int rc = sid_deconv_isra_ex(p, method_arg(nrhs, prhs, 8), (const float*)mxGPUGetDataReadOnly(htf),
                                    (float*)mxGPUGetData(X), maxIter, mode, pn, lam3,
                                    hist ? (float*)mxGPUGetData(hist) : NULL, NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(htf);
        mxGPUDestroyGPUArray(x0);
        if (rc != SID_OK) {
            mxGPUDestroyGPUArray(X);
            if (hist) mxGPUDestroyGPUArray(hist);
            check(rc, cmd);
        }
        plhs[0] = mxGPUCreateMxArrayOnGPU(X);
        mxGPUDestroyGPUArray(X);
        if (hist) {
            plhs[1] = mxGPUCreateMxArrayOnGPU(hist);
            mxGPUDestroyGPUArray(hist);
        }
        return;
    }
    if (!strcmp(cmd, "ls_deconv_ex")) {
        /* X = sid_mex('ls_deconv_ex', plan, df, max_iter, lamb_L1, lamb_L2, lamb_TV_L2, lamb_TV_L1, method) */
        sid_plan* p = plan_arg(prhs[1]);
        const mxGPUArray* df = gpu_arg(prhs[2], 0, cmd);
        need_numel(df, plan_numel(p, 'v'), cmd, "df");
        float tv[3] = {0.f, 0.f, 0.f};
        const mwSize nt = mxGetNumberOfElements(prhs[6]);
        if (nt && (!mxIsDouble(prhs[6]) || mxIsComplex(prhs[6])))
            mexErrMsgIdAndTxt("sid:type", "ls_deconv_ex: lamb_TV_L2 must be a real double vector");
        for (mwSize i = 0; i < nt && i < 3; ++i) tv[i] = (float)mxGetPr(prhs[6])[i];
        mxGPUArray* X = gpu_copy(df);
        int rc = sid_deconv_ls_ex(p, method_arg(nrhs, prhs, 8), (float*)mxGPUGetData(X), (int)mxGetScalar(prhs[3]),
                                  (float)mxGetScalar(prhs[4]), (float)mxGetScalar(prhs[5]), tv,
                                  (float)mxGetScalar(prhs[7]), NULL);
        if (rc == SID_OK) rc = sid_plan_sync(p, NULL);
        mxGPUDestroyGPUArray(df);
        if (rc != SID_OK) mxGPUDestroyGPUArray(X);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(X);
        mxGPUDestroyGPUArray(X);
        return;
    }
    if (!strcmp(cmd, "library")) {
        /* F = sid_mex('library', plan, recon, centers, neur_id, neur_rad, axial[, method]): recon a cell of
         * X x Y x Z single gpuArrays, centers n x 3 double, neur_id n x numel(recon) logical; method 'direct'
         * or 'spectral'; F n x P single gpuArray */
        sid_plan* p = plan_arg(prhs[1]);
        int spectral = 0;
        if (nrhs > 7) {
            char m[16];
            if (mxGetString(prhs[7], m, sizeof(m)) != 0 || (strcmp(m, "direct") && strcmp(m, "spectral")))
                mexErrMsgIdAndTxt("sid:library", "method must be 'direct' or 'spectral'");
            spectral = !strcmp(m, "spectral");
        }
        const mxArray* rc_cell = prhs[2];
        const mwSize nc = mxGetNumberOfElements(rc_cell);
        if (nc < 1 || nc > 4096) mexErrMsgIdAndTxt("sid:library", "recon must be a cell of 1..4096 volumes");
        const mxGPUArray* vols[4096];
        const float* ptrs[4096];
        for (mwSize k = 0; k < nc; ++k) {
            vols[k] = gpu_arg(mxGetCell(rc_cell, k), 0, cmd);
            need_numel(vols[k], plan_numel(p, 'v'), cmd, "recon{k}");
            ptrs[k] = (const float*)mxGPUGetDataReadOnly(vols[k]);
        }
        const mwSize n = mxGetDimensions(prhs[3])[0];
        if (!mxIsLogical(prhs[4]) || mxGetNumberOfElements(prhs[4]) != n * nc) {
            for (mwSize k = 0; k < nc; ++k) mxGPUDestroyGPUArray(vols[k]);
            mexErrMsgIdAndTxt("sid:library", "neur_id must be an n x numel(recon) logical array");
        }
        mxArray* ids = mxCreateNumericMatrix(n, nc, mxUINT8_CLASS, mxREAL);
        const mxLogical* nid = mxGetLogicals(prhs[4]);
        uint8_t* idp = (uint8_t*)mxGetData(ids);
        for (mwSize i = 0; i < n * nc; ++i) idp[i] = nid[i] ? 1 : 0;
        int64_t info[14];
        sid_plan_info(p, info);
        mwSize df[2] = {n, (mwSize)(info[3] * info[4])};
        mxGPUArray* F = mxGPUCreateGPUArray(2, df, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = (spectral ? sid_library_spectral : sid_library)(p, ptrs, (int64_t)nc, mxGetPr(prhs[3]), idp,
                                                                 (int64_t)n, (int64_t)mxGetScalar(prhs[5]),
                                                                 mxGetScalar(prhs[6]), (float*)mxGPUGetData(F), 0,
                                                                 NULL);
        for (mwSize k = 0; k < nc; ++k) mxGPUDestroyGPUArray(vols[k]);
        mxDestroyArray(ids);
        if (rc != SID_OK) mxGPUDestroyGPUArray(F);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(F);
        mxGPUDestroyGPUArray(F);
        return;
    }
    if (!strcmp(cmd, "library_kernel")) {
        /* F = sid_mex('library_kernel', plan, centers, r, dim, kernel, method): centers n x 3 double, kernel a
         * single array (or [] for the ball of radius r, axial radius r / dim(3)); F n x P single gpuArray */
        if (nrhs < 7) mexErrMsgIdAndTxt("sid:library_kernel", "usage: sid_mex('library_kernel', plan, centers, r, dim, kernel, method)");
        sid_plan* p = plan_arg(prhs[1]);
        char m[16];
        if (mxGetString(prhs[6], m, sizeof(m)) != 0 || (strcmp(m, "direct") && strcmp(m, "spectral")))
            mexErrMsgIdAndTxt("sid:library_kernel", "method must be 'direct' or 'spectral'");
        if (!mxIsDouble(prhs[2]) || mxGetNumberOfDimensions(prhs[2]) != 2 || mxGetN(prhs[2]) != 3)
            mexErrMsgIdAndTxt("sid:library_kernel", "centers must be an n x 3 double matrix");
        if (!mxIsDouble(prhs[4]) || mxGetNumberOfElements(prhs[4]) < 3)
            mexErrMsgIdAndTxt("sid:library_kernel", "dim must be a 3-element double vector");
        const mwSize n = mxGetM(prhs[2]);
        const float* W = NULL;
        int64_t kd[3] = {0, 0, 0};
        if (!mxIsEmpty(prhs[5])) {
            if (!mxIsSingle(prhs[5])) mexErrMsgIdAndTxt("sid:library_kernel", "kernel must be single");
            const mwSize nd = mxGetNumberOfDimensions(prhs[5]);
            const mwSize* dd = mxGetDimensions(prhs[5]);
            kd[0] = (int64_t)dd[0];
            kd[1] = (int64_t)dd[1];
            kd[2] = nd > 2 ? (int64_t)dd[2] : 1;
            W = (const float*)mxGetData(prhs[5]);
        }
        int64_t info[14];
        sid_plan_info(p, info);
        mwSize df[2] = {n, (mwSize)(info[3] * info[4])};
        mxGPUArray* F = mxGPUCreateGPUArray(2, df, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = sid_library_kernel(p, strcmp(m, "direct") ? SID_METHOD_SPECTRAL_MIXED : SID_METHOD_DIRECT,
                                    mxGetPr(prhs[2]), (int64_t)n, mxGetScalar(prhs[3]), mxGetPr(prhs[4])[2], W, kd[0],
                                    kd[1], kd[2], (float*)mxGPUGetData(F), 0, NULL);
        if (rc != SID_OK) mxGPUDestroyGPUArray(F);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(F);
        mxGPUDestroyGPUArray(F);
        return;
    }
    if (!strcmp(cmd, "spatial_update")) {
        /* Fm = sid_mex('spatial_update', T, Y, template, opts): T R x F single gpuArray, Y P x F single or half
         * gpuArray, template (R - bg_sub) x P logical (host); Fm R x P single gpuArray */
        const mxGPUArray* T = gpu_arg(prhs[1], 0, cmd);
        const mxGPUArray* Y = gpu_arg(prhs[2], 1, cmd);
        const mwSize* dt = mxGPUGetDimensions(T);
        const mwSize* dy = mxGPUGetDimensions(Y);
        const mxArray* o = nrhs > 4 ? prhs[4] : NULL;
        const int bg = (int)field_or(o, "bg_sub", 1.0);
        const mwSize R = dt[0], F = dt[1], P = dy[0];
        if (!mxIsLogical(prhs[3]) || mxGetNumberOfElements(prhs[3]) != (R - (mwSize)bg) * P)
            mexErrMsgIdAndTxt("sid:spatial_update", "template must be a (R - bg_sub) x P logical array");
        mxArray* tm = mxCreateNumericMatrix(R - (mwSize)bg, P, mxUINT8_CLASS, mxREAL);
        const mxLogical* tl = mxGetLogicals(prhs[3]);
        uint8_t* tp = (uint8_t*)mxGetData(tm);
        for (mwSize i = 0; i < (R - (mwSize)bg) * P; ++i) tp[i] = tl[i] ? 1 : 0;
        const mxGPUArray* tg = mxGPUCreateFromMxArray(tm);
        mwSize dfm[2] = {R, P};
        mxGPUArray* Fm = mxGPUCreateGPUArray(2, dfm, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = sid_spatial_update(ctx(cmd), (const float*)mxGPUGetDataReadOnly(T), mxGPUGetDataReadOnly(Y), ydtype(Y),
                                    (const uint8_t*)mxGPUGetDataReadOnly(tg), (int64_t)R, (int64_t)F, (int64_t)P,
                                    field_or(o, "lamb_L1", 0.0), field_or(o, "lamb_L2", 0.0),
                                    field_or(o, "lamb_orth_L1", 0.0), (int)field_or(o, "use_std", 0.0), bg,
                                    (float*)mxGPUGetData(Fm), NULL, NULL);
        mxGPUDestroyGPUArray(T);
        mxGPUDestroyGPUArray(Y);
        mxGPUDestroyGPUArray(tg);
        mxDestroyArray(tm);
        if (rc != SID_OK) mxGPUDestroyGPUArray(Fm);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(Fm);
        mxGPUDestroyGPUArray(Fm);
        return;
    }
    if (!strcmp(cmd, "fast_nnls_ex")) {
        /* [xx, Q, df, h] = sid_mex('fast_nnls_ex', A, Y, opts, Q, df, h): A P x K and Y P x F single (Y may be
         * half) gpuArrays, or [] when Q, h and df are all given; opts.warm_start a K x F single gpuArray or 1;
         * opts.total; Q K x K, df K x F, h K single gpuArrays or [] */
        const int hasA = !mxIsEmpty(prhs[1]);
        const mxGPUArray* A = hasA ? gpu_arg(prhs[1], 0, cmd) : NULL;
        const mxGPUArray* Y = hasA ? gpu_arg(prhs[2], 1, cmd) : NULL;
        const mxArray* o = nrhs > 3 ? prhs[3] : NULL;
        const mxGPUArray* Qi = (nrhs > 4 && !mxIsEmpty(prhs[4])) ? gpu_arg(prhs[4], 0, cmd) : NULL;
        const mxGPUArray* dfi = (nrhs > 5 && !mxIsEmpty(prhs[5])) ? gpu_arg(prhs[5], 0, cmd) : NULL;
        const mxGPUArray* hi = (nrhs > 6 && !mxIsEmpty(prhs[6])) ? gpu_arg(prhs[6], 0, cmd) : NULL;
        int64_t P = 0, K = 0, F = 0;
        if (A) {
            P = (int64_t)mxGPUGetDimensions(A)[0];
            K = (int64_t)mxGPUGetDimensions(A)[1];
            F = (int64_t)mxGPUGetDimensions(Y)[1];
        } else if (Qi && dfi) {
            K = (int64_t)mxGPUGetDimensions(Qi)[0];
            F = (int64_t)mxGPUGetDimensions(dfi)[1];
        } else {
            mexErrMsgIdAndTxt("sid:fast_nnls_ex", "A and Y, or Q, df and h, are needed");
        }
        sid_nnls_opts opts;
        sid_fast_nnls_defaults(&opts);
        if (nrhs < 4) opts.tol = 1e-12; /* two-argument call, fast_nnls.m:12-15 */
        opts.lambda = field_or(o, "lambda", opts.lambda);
        opts.sample = (int64_t)field_or(o, "sample", (double)opts.sample);
        opts.tol = field_or(o, "tol", opts.tol);
        opts.tol_ = field_or(o, "tol_", opts.tol_);
        opts.max_iter = (int64_t)field_or(o, "max_iter", (double)opts.max_iter);
        opts.tol_p = (int)field_or(o, "tol_p", 1);
        const int total = (int)field_or(o, "total", 0.0) != 0;
        int warm_mode = 0;
        const mxGPUArray* W = NULL;
        const mxArray* wf = (o && mxIsStruct(o)) ? mxGetField(o, 0, "warm_start") : NULL;
        if (wf && !mxIsEmpty(wf)) {
            if (mxGetNumberOfElements(wf) == 1 && !mxIsGPUArray(wf)) warm_mode = 1;
            else { W = gpu_arg(wf, 0, cmd); warm_mode = 2; }
        }
        mwSize dx[2] = {(mwSize)K, (mwSize)F}, dq[2] = {(mwSize)K, (mwSize)K}, dh[2] = {(mwSize)K, 1};
        mwSize ddf[2] = {(mwSize)K, total ? (mwSize)F : 0};
        mxGPUArray* X = mxGPUCreateGPUArray(2, dx, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* Qo = mxGPUCreateGPUArray(2, dq, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* dfo = mxGPUCreateGPUArray(2, ddf, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        mxGPUArray* ho = mxGPUCreateGPUArray(2, dh, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = sid_fast_nnls_ex(ctx(cmd), A ? (const float*)mxGPUGetDataReadOnly(A) : NULL,
                                  Y ? mxGPUGetDataReadOnly(Y) : NULL, Y ? ydtype(Y) : SID_DTYPE_F32, P, K, F, &opts,
                                  total, warm_mode, W ? (const float*)mxGPUGetDataReadOnly(W) : NULL,
                                  Qi ? (const float*)mxGPUGetDataReadOnly(Qi) : NULL,
                                  dfi ? (const float*)mxGPUGetDataReadOnly(dfi) : NULL,
                                  hi ? (const float*)mxGPUGetDataReadOnly(hi) : NULL, (float*)mxGPUGetData(X),
                                  (float*)mxGPUGetData(Qo), total ? (float*)mxGPUGetData(dfo) : NULL,
                                  (float*)mxGPUGetData(ho), SID_PREC_SPLIT, NULL, NULL);
        const mxGPUArray* ins[6] = {A, Y, Qi, dfi, hi, W};
        for (int i = 0; i < 6; ++i)
            if (ins[i]) mxGPUDestroyGPUArray(ins[i]);
        mxGPUArray* outs[4] = {X, Qo, dfo, ho};
        if (rc != SID_OK)
            for (int i = 0; i < 4; ++i) mxGPUDestroyGPUArray(outs[i]);
        check(rc, cmd);
        for (int i = 0; i < 4; ++i) {
            if (i < (nlhs > 0 ? nlhs : 1)) plhs[i] = mxGPUCreateMxArrayOnGPU(outs[i]);
            mxGPUDestroyGPUArray(outs[i]);
        }
        return;
    }
    if (!strcmp(cmd, "reg_nnls")) {
        /* x = sid_mex('reg_nnls', A, d, opts): A m x n, d m double gpuArrays; x n double gpuArray */
        if (!mxIsGPUArray(prhs[1]) || !mxIsGPUArray(prhs[2]))
            mexErrMsgIdAndTxt("sid:type", "%s: gpuArray arguments expected", cmd);
        const mxGPUArray* A = mxGPUCreateFromMxArray(prhs[1]);
        const mxGPUArray* d = mxGPUCreateFromMxArray(prhs[2]);
        if (mxGPUGetClassID(A) != mxDOUBLE_CLASS || mxGPUGetClassID(d) != mxDOUBLE_CLASS)
            mexErrMsgIdAndTxt("sid:type", "%s: double gpuArrays expected", cmd);
        const mwSize* da = mxGPUGetDimensions(A);
        const mxArray* o = nrhs > 3 ? prhs[3] : NULL;
        const mxArray* hf = (o && mxIsStruct(o)) ? mxGetField(o, 0, "hilf") : NULL;
        const mxGPUArray* hg = (hf && !mxIsEmpty(hf)) ? mxGPUCreateFromMxArray(hf) : NULL;
        mwSize dxx[2] = {da[1], 1};
        mxGPUArray* x = mxGPUCreateGPUArray(2, dxx, mxDOUBLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
        int rc = sid_reg_nnls(ctx(cmd), (const double*)mxGPUGetDataReadOnly(A), (int64_t)da[0], (int)da[1],
                              (const double*)mxGPUGetDataReadOnly(d), field_or(o, "lamb_L1", 0.0),
                              field_or(o, "lamb_L2", 0.0), field_or(o, "lamb_orth_L1", 0.0),
                              (int)field_or(o, "use_std", 0.0), (int)field_or(o, "bg_sub", 0.0),
                              hg ? (const double*)mxGPUGetDataReadOnly(hg) : NULL, (double*)mxGPUGetData(x), NULL);
        mxGPUDestroyGPUArray(A);
        mxGPUDestroyGPUArray(d);
        if (hg) mxGPUDestroyGPUArray(hg);
        if (rc != SID_OK) mxGPUDestroyGPUArray(x);
        check(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(x);
        mxGPUDestroyGPUArray(x);
        return;
    }
    mexErrMsgIdAndTxt("sid:usage", "unknown command '%s'", cmd);
}
