// qr_d.cu — double instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T double
#define RNPGPU_CT double
#define RNPGPU_P d
#define RNPGPU_LOW_T float
#define RNPGPU_MIXED_FN rnpgpu_dsgels
#define RNPGPU_REAL 1
#include "qr_type.inc"

extern "C" int rnpgpu_dls_residual(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *x, size_t ldx, const double *b, size_t ldb, double *r, size_t ldr,
                                   double *g, size_t ldg, void *work, size_t *lwork_bytes) {
    return rnpgpu::ls_residual(m, n, nrhs, a, lda, x, ldx, b, ldb, r, ldr, g, ldg, work, lwork_bytes);
}

// the mixed solve from host buffers (RNP's gels call with host arrays)
extern "C" int rnpgpu_dsgels_host(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *b, size_t ldb, double *x, size_t ldx, int max_iter, int flags,
                                  rnpgpu_refine_info *info, size_t *lwork, double *work) {
    return rnpgpu::gels_refine_host<double, float>(m, n, nrhs, a, lda, b, ldb, x, ldx, max_iter, flags, reinterpret_cast<rnpgpu::RefineInfo *>(info), lwork, work);
}
