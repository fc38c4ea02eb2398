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
 *   [X, G]   = sid_mex('ls_nnls', A, Y, opts)
 *   [X, Q]   = sid_mex('fast_nnls', A, Y, opts)
 *   sid_mex('destroy', plan)
 * gpuArray inputs use the device entry points directly (mxGPUArray); other
 * inputs go through the _host entry points.  A non-zero libsid status becomes a
 * MATLAB error with identifier 'sid:<command>' and sid_last_error() as text.
 */
#include <stdint.h>
#include <string.h>

#include "gpu/mxGPUArray.h"
#include "mex.h"
#include "sid.h"

#define MAX_PLANS 64
static sid_plan* g_plans[MAX_PLANS];
static sid_ctx* g_ctx = NULL;

static void cleanup(void)
{
    for (int i = 0; i < MAX_PLANS; ++i)
        if (g_plans[i]) {
            sid_plan_destroy(g_plans[i]);
            g_plans[i] = NULL;
        }
    if (g_ctx) {
        sid_ctx_destroy(g_ctx);
        g_ctx = NULL;
    }
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

/* out = f(plan, in) for a single-precision array, on the device or the host */
typedef int (*dev_fn)(sid_plan*, int, const float*, float*, void*);
typedef int (*host_fn)(sid_plan*, int, const float*, float*);

static mxArray* project(sid_plan* p, int method, const mxArray* in, mwSize nd, const mwSize* dims, dev_fn fd,
                        host_fn fh, const char* cmd)
{
    if (mxIsGPUArray(in)) {
        const mxGPUArray* gin = mxGPUCreateFromMxArray(in);
        if (mxGPUGetClassID(gin) != mxSINGLE_CLASS) mexErrMsgIdAndTxt("sid:type", "%s: input must be single", cmd);
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
        const int64_t Z = mxGetNumberOfDimensions(H) > 4 ? (int64_t)d[4] : 1;
        int32_t* ca = NULL;
        int32_t cabuf[2 * 4096];
        if (!mxIsEmpty(prhs[2])) {
            const double* c = mxGetPr(prhs[2]);
            for (int64_t i = 0; i < 2 * Z && i < 2 * 4096; ++i) cabuf[i] = (int32_t)c[i];
            ca = cabuf;
        }
        int slot = -1;
        for (int i = 0; i < MAX_PLANS; ++i)
            if (!g_plans[i]) { slot = i; break; }
        if (slot < 0) mexErrMsgIdAndTxt("sid:plan", "too many plans");
        const int flags = nrhs > 5 ? (int)mxGetScalar(prhs[5]) : (SID_PLAN_SPECTRAL_F32 | SID_PLAN_SPECTRAL_I16);
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
        int64_t info[12];
        sid_plan_info(p, info);
        const int fwd = !strcmp(cmd, "forward");
        mwSize dims[3] = {(mwSize)info[3], (mwSize)info[4], (mwSize)info[2]};
        plhs[0] = project(p, method_arg(nrhs, prhs, 3), prhs[2], fwd ? 2 : 3, dims, fwd ? sid_forward : sid_adjoint,
                          fwd ? sid_forward_host : sid_adjoint_host, cmd);
        return;
    }
    if (!strcmp(cmd, "isra")) {
        sid_plan* p = plan_arg(prhs[1]);
        if (!mxIsSingle(prhs[2]) || !mxIsSingle(prhs[3])) mexErrMsgIdAndTxt("sid:type", "isra: single inputs");
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
    mexErrMsgIdAndTxt("sid:usage", "unknown command '%s'", cmd);
}
