// contract.cu -- solver context and the Gram / cross-product entry points.
//
// G = A'A and h = A'Y are the only dense contractions of the NNLS path
// (LS_nnls.m:76,82; fast_nnls.m:54-57; T_update.m:24-25;
// incremental_temporal_update_gpu.m:83,89).  Three precisions:
//   SID_PREC_FP32  FP32 SIMT (gemm_simt.cu) -- the plain path;
//   SID_PREC_SPLIT tensor cores (gemm_tc.cu) on 16-bit hi/lo splits of the
//                  FP32 operands (hi*hi + hi*lo + lo*hi, FP32 accumulation in
//                  TMEM); FP16 movies enter unsplit (A_hi*Y + A_lo*Y);
//   SID_PREC_BF16  one BF16 tensor-core pass.
#include <cmath>
#include <cstring>

#include "sid_internal.cuh"

namespace sid {
int gemm_tn(const void* const* A, const void* const* B, int npass, int64_t m, int64_t n, int64_t k, bool bf16,
            float* C, int64_t ldc, float alpha, float beta, int bn, int splitk, float* ws, int64_t ws_elems, int* err,
            cudaStream_t st);
void gemm_autotune(int m, int n, int nkb, int* bn, int* splitk);
void gemm_autotune_sym(int m, int nkb, int* bn, int* splitk);
int gemm_tn_sym(const void* const* A, const void* const* B, int npass, int64_t m, int64_t k, bool bf16, float* C,
                int64_t ldc, float alpha, int bn, int splitk, float* ws, int64_t ws_elems, int* err, cudaStream_t st);
int sgemm_tn(const float* A, const float* B, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, float* C,
             int64_t ldc, float alpha, float beta, float* ws, int64_t ws_elems, cudaStream_t st);
int64_t sgemm_ws_elems(int64_t m, int64_t n, int64_t k);
int split16(const float* src, int64_t k, int64_t rows, int64_t lds, uint16_t* hi, uint16_t* lo, bool bf16,
            float scale, cudaStream_t st);
int copy16_blk(const uint16_t* src, int64_t k, int64_t rows, int64_t lds, uint16_t* dst, cudaStream_t st);
int64_t blk16_elems(int64_t k, int64_t rows);
}  // namespace sid

namespace sid {

int ctx_sync(sid_ctx* c, cudaStream_t st)
{
    SID_CUDA_TRY(cudaStreamSynchronize(st));
    int flag = 0;
    SID_CUDA_TRY(cudaMemcpy(&flag, c->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        cudaMemset(c->errflag.p, 0, sizeof(int));
        set_error("a device-side wait exceeded its budget (code %d)", flag);
        return SID_ETIMEOUT;
    }
    return SID_OK;
}

// C (m x n) = alpha * A'B + beta*C with A: k x m (lda), B: k x n (ldb), FP32
// operands, at precision `prec`.  B may instead be FP16 (b_f16 != 0).
int contract(sid_ctx* c, const float* A, const void* B, bool b_f16, int64_t m, int64_t n, int64_t k, int64_t lda,
             int64_t ldb, float* C, int64_t ldc, float alpha, float beta, int prec, cudaStream_t st)
{
    int* err = c->errflag.as<int>();
    if (prec == SID_PREC_FP32) {
        SID_REQUIRE(!b_f16, "FP32 contraction needs an FP32 right operand");
        SID_TRY(c->ws.alloc((size_t)sgemm_ws_elems(m, n, k) * sizeof(float)));
        return sgemm_tn(A, static_cast<const float*>(B), m, n, k, lda, ldb, C, ldc, alpha, beta, c->ws.as<float>(),
                        (int64_t)(c->ws.bytes / sizeof(float)), st);
    }
    SID_REQUIRE(prec == SID_PREC_SPLIT || prec == SID_PREC_BF16, "unknown precision %d", prec);
    int bn = 0, splitk = 0;
    const bool same = (static_cast<const void*>(A) == B && lda == ldb && m == n && !b_f16);
    if (same && beta == 0.f) gemm_autotune_sym((int)m, (int)cdiv(k, 64), &bn, &splitk);
    else gemm_autotune((int)m, (int)n, (int)cdiv(k, 64), &bn, &splitk);
    SID_TRY(c->ws.alloc((size_t)(splitk * m * n) * sizeof(float)));
    const bool split = prec == SID_PREC_SPLIT;
    const size_t abytes = (size_t)blk16_elems(k, m) * 2, bbytes = (size_t)blk16_elems(k, n) * 2;
    if (b_f16) {
        // FP16 right operand used unsplit; A split into FP16 hi/lo with a
        // power-of-two scale sa found and applied on the device (alpha / sa
        // goes to the GEMM epilogue), so nothing waits on the host
        float* sw = c->scales.as<float>();
        unsigned int* amax = reinterpret_cast<unsigned int*>(sw + 12);
        SID_TRY(pow2_scale_dev(A, m * lda, amax, sw + 13, st));  // over the whole stored matrix
        SID_TRY(scale_ratio_dev(sw + 13, nullptr, 1.f, sw + 14, st));
        SID_TRY(c->a_hi.alloc(abytes));
        if (split) SID_TRY(c->a_lo.alloc(abytes));
        SID_TRY(split16_ds(A, k, m, lda, c->a_hi.as<uint16_t>(), split ? c->a_lo.as<uint16_t>() : nullptr, false, 1.f,
                           sw + 13, st));
        SID_TRY(c->b_hi.alloc(bbytes));
        SID_TRY(copy16_blk(static_cast<const uint16_t*>(B), k, n, ldb, c->b_hi.as<uint16_t>(), st));
        const void* As[2] = {c->a_hi.p, c->a_lo.p};
        const void* Bs[2] = {c->b_hi.p, c->b_hi.p};
        c->timer.begin(st);
        const int rc = gemm_tn_ds(As, Bs, split ? 2 : 1, m, n, k, false, C, ldc, alpha, sw + 14, beta, bn, splitk,
                                  c->ws.as<float>(), (int64_t)(c->ws.bytes / sizeof(float)), err, st);
        c->timer.finish(st);
        return rc;
    }
    // FP32 x FP32: BF16 hi/lo splits of both (no scaling needed: BF16 keeps the FP32 exponent range)
    SID_TRY(c->a_hi.alloc(abytes));
    if (split) SID_TRY(c->a_lo.alloc(abytes));
    SID_TRY(split16(A, k, m, lda, c->a_hi.as<uint16_t>(), split ? c->a_lo.as<uint16_t>() : nullptr, true, 1.f, st));
    const void *bh = c->a_hi.p, *bl = c->a_lo.p;
    if (!same) {
        SID_TRY(c->b_hi.alloc(bbytes));
        if (split) SID_TRY(c->b_lo.alloc(bbytes));
        SID_TRY(split16(static_cast<const float*>(B), k, n, ldb, c->b_hi.as<uint16_t>(),
                        split ? c->b_lo.as<uint16_t>() : nullptr, true, 1.f, st));
        bh = c->b_hi.p;
        bl = c->b_lo.p;
    }
    const void* As[3] = {c->a_hi.p, c->a_hi.p, c->a_lo.p};
    const void* Bs[3] = {bh, bl, bh};
    int rc;
    c->timer.begin(st);
    if (same && beta == 0.f)  // A'A: hi*hi + hi*lo + lo*hi is symmetric as a whole
        rc = gemm_tn_sym(As, Bs, split ? 3 : 1, m, k, true, C, ldc, alpha, bn, splitk, c->ws.as<float>(),
                         (int64_t)(c->ws.bytes / sizeof(float)), err, st);
    else
        rc = gemm_tn(As, Bs, split ? 3 : 1, m, n, k, true, C, ldc, alpha, beta, bn, splitk, c->ws.as<float>(),
                     (int64_t)(c->ws.bytes / sizeof(float)), err, st);
    c->timer.finish(st);
    return rc;
}

}  // namespace sid

using namespace sid;

extern "C" int sid_ctx_create(sid_ctx** out)
{
    SID_REQUIRE(out, "sid_ctx_create: NULL output");
    sid_ctx* c = new sid_ctx();
    cudaGetDevice(&c->device);
    if (c->errflag.alloc(sizeof(int)) != SID_OK || cudaMemset(c->errflag.p, 0, sizeof(int)) != cudaSuccess ||
        c->scales.alloc(kScaleWords * 4) != SID_OK ||
        cudaMemset(c->scales.p, 0, kScaleWords * 4) != cudaSuccess) {
        c->errflag.release();
        c->scales.release();
        delete c;
        *out = nullptr;
        return SID_ENOMEM;
    }
    *out = c;
    return SID_OK;
}

extern "C" int sid_ctx_destroy(sid_ctx* c)
{
    if (!c) return SID_OK;
    DBuf* b[] = {&c->a_hi, &c->a_lo, &c->b_hi, &c->b_lo, &c->ws, &c->scal, &c->errflag, &c->scales};
    for (DBuf* x : b) x->release();
    c->timer.release();
    for (DBuf& x : c->nn) x.release();
    for (DBuf& x : c->mf) x.release();
    for (DBuf& x : c->bg) x.release();
    for (DBuf& x : c->pix) x.release();
    delete c;
    return SID_OK;
}

extern "C" int sid_ctx_sync(sid_ctx* c, void* stream)
{
    SID_REQUIRE(c, "sid_ctx_sync: NULL context");
    return ctx_sync(c, static_cast<cudaStream_t>(stream));
}

extern "C" int sid_gram(sid_ctx* c, const float* A, int64_t P, int64_t K, float* G, int prec, void* stream)
{
    SID_REQUIRE(c && A && G, "sid_gram: NULL argument");
    SID_REQUIRE(P > 0 && K > 0, "sid_gram: empty matrix");
    return contract(c, A, A, false, K, K, P, P, P, G, K, 1.f, 0.f, prec, static_cast<cudaStream_t>(stream));
}

extern "C" int sid_cross(sid_ctx* c, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                         float* h, int prec, void* stream)
{
    SID_REQUIRE(c && A && Y && h, "sid_cross: NULL argument");
    SID_REQUIRE(P > 0 && K > 0 && F > 0, "sid_cross: empty matrix");
    SID_REQUIRE(ydtype == SID_DTYPE_F32 || ydtype == SID_DTYPE_F16, "sid_cross: unknown Y dtype %d", ydtype);
    const bool f16 = ydtype == SID_DTYPE_F16;
    SID_REQUIRE(!(f16 && prec == SID_PREC_FP32), "sid_cross: an FP16 movie needs SID_PREC_SPLIT or SID_PREC_BF16");
    return contract(c, A, Y, f16, K, F, P, P, P, h, K, 1.f, 0.f, prec, static_cast<cudaStream_t>(stream));
}

extern "C" int sid_ctx_timing_enable(sid_ctx* c, int on)
{
    SID_REQUIRE(c, "sid_ctx_timing_enable: NULL context");
    if (on && !c->timer.on) c->timer.used = 0;
    c->timer.on = on != 0;
    return SID_OK;
}

extern "C" int sid_ctx_timing_read(sid_ctx* c, double* total_ms, int64_t* launches)
{
    SID_REQUIRE(c && total_ms && launches, "sid_ctx_timing_read: NULL argument");
    double t = 0.0;
    for (size_t i = 0; i < c->timer.used; ++i) {
        SID_CUDA_TRY(cudaEventSynchronize(c->timer.end[i]));
        float ms = 0.f;
        SID_CUDA_TRY(cudaEventElapsedTime(&ms, c->timer.beg[i], c->timer.end[i]));
        t += ms;
    }
    *total_ms = t;
    *launches = (int64_t)c->timer.used;
    c->timer.used = 0;
    return SID_OK;
}
