// qr_s.cu — float instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T float
#define RNPGPU_CT float
#define RNPGPU_P s
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
