// qr_s.cu — float instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T float
#define RNPGPU_CT float
#define RNPGPU_P s
#define RNPGPU_REAL 1
#include "qr_type.inc"

// C = alpha op(A) op(B) + beta C for FP32 on the tensor cores (three-term
// BF16 split, FP32 accumulation); op "N" or "T", beta 0 or 1.  No reference
// counterpart: the contraction the FP32 trailing updates use, exported so it
// can be checked on its own.
extern "C" int rnpgpu_sgemm_tc(const char *transa, const char *transb, size_t m, size_t n, size_t k, float alpha, const float *a, size_t lda, const float *b, size_t ldb, float beta, float *c, size_t ldc) {
    using namespace rnpgpu;
    if (transa == nullptr || (transa[0] != 'N' && transa[0] != 'T')) return -1;
    if (transb == nullptr || (transb[0] != 'N' && transb[0] != 'T')) return -2;
    if (m == 0 || n == 0) return kOk;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX || k > (size_t)INT32_MAX) return -3;
    const bool ta = transa[0] == 'T', tb = transb[0] == 'T';
    if (lda < std::max<size_t>(1, ta ? k : m)) return -8;
    if (ldb < std::max<size_t>(1, tb ? n : k)) return -10;
    if (ldc < std::max<size_t>(1, m)) return -13;
    if (beta != 0.0f && beta != 1.0f) return -12;
    GemmArgs<float> g = gemm_args<float>(a, lda, ta ? kOpT : kOpN, 0, b, ldb, tb ? kOpT : kOpN, 0, c, ldc, (int)m, (int)n, (int)k, alpha, beta == 1.0f ? kBetaOne : kBetaZero);
    if (k == 0) g.kchunk = 1;
    return launch_gemm_tc(g, 1, current_stream());
}

// The mixed solvers' internal FP32 factorization, exported for checking.
extern "C" int rnpgpu_sgeqrf_mixed(size_t m, size_t n, float *a, size_t lda, float *tau, float *tstore, int flags, int *cqr_failed, size_t *lwork, float *work) {
    using namespace rnpgpu;
    if (lwork == nullptr) return -9;
    const size_t k = std::min(m, n);
    if (k == 0) return kOk;
    if (lda < std::max<size_t>(1, m)) return -4;
    if (m > (size_t)INT32_MAX / 2 || n > (size_t)INT32_MAX / 2) return -1;
    const size_t fbytes = (geqrf_bytes<float>(m, n, smax_for<float>(m)) + 255) / 256 * 256;
    const bool wide_ok = wide::usable(m, n, reinterpret_cast<const float *>(256), 4);  // sized by the shape alone
    const size_t need = elems_for<float>(fbytes + cqr_ws_bytes() + (wide_ok ? wide::ws_bytes(m, n) : 0) + 256);
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -3;
    if (tau == nullptr) return -5;
    if (tstore == nullptr) return -6;
    if (*lwork < need) return -9;
    cudaStream_t st = current_stream();
    Carver cv(work);
    float *wf = cv.take<float>(fbytes / sizeof(float));
    CqrWs cw = carve_cqr(cv);
    if (wide_ok) {
        cw.wide = wide::carve(cv, m, n);
        cw.use_wide = (flags & 2) == 0;
    }
    RNPGPU_CHECK(cudaMemsetAsync(cw.fail, 0, sizeof(int), st));
    size_t lw = fbytes / sizeof(float);
    int rc = geqrf<float>(m, n, a, lda, tau, &lw, wf, tstore, &cw);
    if (rc) return rc;
    if (cqr_failed) {
        RNPGPU_CHECK(cudaMemcpyAsync(cqr_failed, cw.fail, sizeof(int), cudaMemcpyDeviceToHost, st));
        RNPGPU_CHECK(cudaStreamSynchronize(st));
    }
    return kOk;
}
