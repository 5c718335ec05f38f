/* consumers_gb300.h — C ABI of the reference's callers of QR and QL on the
 * GPU: the Q of a Hessenberg reduction (RNP::LA::Hessenberg::MultQ and
 * GenerateQ, LAPACK _unmhr / _unghr), the Q of a Hermitian tridiagonal
 * reduction (RNP::LA::Tridiagonal::MultQHerm and GenerateQHerm, _unmtr /
 * _ungtr), and the QR step of the complex generalized eigensystem driver.
 * Same argument lists and storage as the reference; device pointers,
 * asynchronous on the library's stream, caller-owned workspace with the
 * reference's query (work == NULL or *lwork == 0 stores the length in
 * elements; the GPU's lengths exceed the reference's); status 0, -i for
 * argument i, > 0 for a CUDA error. */
#ifndef RNP_GPU_CONSUMERS_GB300_H
#define RNP_GPU_CONSUMERS_GB300_H

#include <stddef.h>
#include "qr_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNP::LA::Hessenberg::MultQ (RNP/LA/Hessenberg.hpp:477-512): C = op(Q) C
 * or C op(Q) for the Q = H[ilo] ... H[ihi-2] of Hessenberg::Reduce ---- */
int rnpgpu_sunmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::Hessenberg::GenerateQ (RNP/LA/Hessenberg.hpp:539-590): the
 * reduction in a (n x n) is overwritten by Q ---- */
int rnpgpu_sunghr(size_t n, size_t ilo, size_t ihi, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dunghr(size_t n, size_t ilo, size_t ihi, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cunghr(size_t n, size_t ilo, size_t ihi, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunghr(size_t n, size_t ilo, size_t ihi, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::Tridiagonal::GenerateQHerm (RNP/LA/Tridiagonal.hpp:1037-1097):
 * uplo "U" (a QL factor's Q) or "L" (a QR factor's Q) ---- */
int rnpgpu_sungtr(const char *uplo, size_t n, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dungtr(const char *uplo, size_t n, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cungtr(const char *uplo, size_t n, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zungtr(const char *uplo, size_t n, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::Tridiagonal::MultQHerm (RNP/LA/Tridiagonal.hpp:1140-1188) ---- */
int rnpgpu_sunmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);
/* ---- The QR step of ComplexGeneralizedEigensystem
 * (RNP/LA/GeneralizedEigensystems.hpp:451-472, workspace 376-412): with
 * irows = ihi - ilo and icols = n - ilo when vl or vr is given (else irows),
 * B(ilo:ihi, ilo:ilo+icols) is factored (QR::Factor), Q^H is applied to
 * A(ilo:ihi, ilo:ilo+icols) (QR::MultQ "L","C"), vl (may be NULL) is set to
 * the identity with Q generated in its (ilo:ihi, ilo:ihi) block
 * (Triangular::Copy of B's reflectors, QR::GenerateQ), vr (may be NULL) to
 * the identity.  The workspace is laid out as the reference's, [tau (n) |
 * work]: on return its first n elements hold tau.  ilo and ihi come from the
 * caller's balancing, 0 <= ilo < ihi <= n. ---- */
int rnpgpu_cgg_triangularize_b(size_t n, size_t ilo, size_t ihi, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *b, size_t ldb, rnpgpu_complex_float *vl, size_t ldvl, rnpgpu_complex_float *vr, size_t ldvr, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgg_triangularize_b(size_t n, size_t ilo, size_t ihi, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *b, size_t ldb, rnpgpu_complex_double *vl, size_t ldvl, rnpgpu_complex_double *vr, size_t ldvr, size_t *lwork, rnpgpu_complex_double *work);

#ifdef __cplusplus
}
#endif

#endif
