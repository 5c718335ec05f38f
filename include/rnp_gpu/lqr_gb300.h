/* lqr_gb300.h — C ABI of the GB300 LQ, QL and RQ factorizations: the
 * reference's RNP::LA::LQ, RNP::LA::QL and RNP::LA::RQ Factor, MultQ and
 * GenerateQ (same argument lists and storage as their QR counterparts in
 * qr_gb300.h, LAPACK names).  Device pointers, asynchronous on the library's
 * stream, caller-owned workspace with the reference's query (work == NULL or
 * *lwork == 0 stores the length in elements); status 0, -i for argument i,
 * > 0 for a CUDA error.  The workspace holds a transformed copy of the
 * reflector matrix (these run the QR kernels on A^H, J A J or J A^H J), so
 * the queried lengths exceed the reference's.
 *
 * Storage (as the reference): LQ: L in the lower triangle, reflector i in
 * row i to the right of the diagonal; QL: L in the lower trapezoid at the
 * bottom (m >= n), reflector i in column n-k+i above row m-k+i; RQ: R in the
 * upper trapezoid at the right, reflector i in row m-k+i left of column
 * n-k+i.  MultQ takes the reflectors as k rows (LQ, RQ: a is k x nq, lda >= k)
 * or k columns (QL: a is nq x k, lda >= nq). */
#ifndef RNP_GPU_LQR_GB300_H
#define RNP_GPU_LQR_GB300_H

#include <stddef.h>
#include "qr_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNP::LA::LQ::Factor (RNP/LA/LQ.hpp:127-184), LAPACK _gelqf ---- */
int rnpgpu_sgelqf(size_t m, size_t n, float *a, size_t lda, float *tau, size_t *lwork, float *work);
int rnpgpu_dgelqf(size_t m, size_t n, double *a, size_t lda, double *tau, size_t *lwork, double *work);
int rnpgpu_cgelqf(size_t m, size_t n, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgelqf(size_t m, size_t n, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::LQ::MultQ (RNP/LA/LQ.hpp:310-419), _unmlq ---- */
int rnpgpu_sunmlq(const char *side, const char *trans, size_t m, size_t n, size_t k, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmlq(const char *side, const char *trans, size_t m, size_t n, size_t k, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmlq(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmlq(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::LQ::GenerateQ (RNP/LA/LQ.hpp:492-556), _unglq ---- */
int rnpgpu_sunglq(size_t m, size_t n, size_t k, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dunglq(size_t m, size_t n, size_t k, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cunglq(size_t m, size_t n, size_t k, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunglq(size_t m, size_t n, size_t k, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);

/* ---- RNP::LA::QL::Factor (RNP/LA/QL.hpp:129-208), LAPACK _geqlf ---- */
int rnpgpu_sgeqlf(size_t m, size_t n, float *a, size_t lda, float *tau, size_t *lwork, float *work);
int rnpgpu_dgeqlf(size_t m, size_t n, double *a, size_t lda, double *tau, size_t *lwork, double *work);
int rnpgpu_cgeqlf(size_t m, size_t n, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgeqlf(size_t m, size_t n, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::QL::MultQ (RNP/LA/QL.hpp:337-437), _unmql ---- */
int rnpgpu_sunmql(const char *side, const char *trans, size_t m, size_t n, size_t k, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmql(const char *side, const char *trans, size_t m, size_t n, size_t k, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmql(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmql(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::QL::GenerateQ (RNP/LA/QL.hpp:501-566), _ungql ---- */
int rnpgpu_sungql(size_t m, size_t n, size_t k, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dungql(size_t m, size_t n, size_t k, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cungql(size_t m, size_t n, size_t k, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zungql(size_t m, size_t n, size_t k, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);

/* ---- RNP::LA::RQ::Factor (RNP/LA/RQ.hpp:131-210), LAPACK _gerqf ---- */
int rnpgpu_sgerqf(size_t m, size_t n, float *a, size_t lda, float *tau, size_t *lwork, float *work);
int rnpgpu_dgerqf(size_t m, size_t n, double *a, size_t lda, double *tau, size_t *lwork, double *work);
int rnpgpu_cgerqf(size_t m, size_t n, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgerqf(size_t m, size_t n, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::RQ::MultQ (RNP/LA/RQ.hpp:344-449), _unmrq ---- */
int rnpgpu_sunmrq(const char *side, const char *trans, size_t m, size_t n, size_t k, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmrq(const char *side, const char *trans, size_t m, size_t n, size_t k, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmrq(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmrq(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);
/* ---- RNP::LA::RQ::GenerateQ (RNP/LA/RQ.hpp:519-586), _ungrq ---- */
int rnpgpu_sungrq(size_t m, size_t n, size_t k, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dungrq(size_t m, size_t n, size_t k, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cungrq(size_t m, size_t n, size_t k, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zungrq(size_t m, size_t n, size_t k, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_LQR_GB300_H */
