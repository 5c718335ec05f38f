/* ls_gb300.h — C ABI of the least-squares layer on the GB300 QR.
 *
 * Conventions as in qr_gb300.h: column-major DEVICE arrays, caller-owned
 * workspace with the *lwork query (work == NULL or *lwork == 0), asynchronous
 * on the stream set by rnpgpu_set_stream, int status (0 ok, -i bad argument
 * i, > 0 CUDA error).
 */
#ifndef RNP_GPU_LS_GB300_H
#define RNP_GPU_LS_GB300_H

#include <stddef.h>
#include "qr_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Upper triangular solve B <- R^{-1} B (R n x n non-unit, B n x nrhs):
 *      replaces RNP::BLAS::SolveTrM("L","U","N","N", n, nrhs, 1, a, lda, b, ldb)
 *      (RNP/BLAS/BLAS_mix.hpp:2096-2113, forwarded to dtrsm_ at src/BLAS_mix.cpp:682) ---- */
int rnpgpu_strsm_lunn(size_t n, size_t nrhs, const float *a, size_t lda, float *b, size_t ldb);
int rnpgpu_dtrsm_lunn(size_t n, size_t nrhs, const double *a, size_t lda, double *b, size_t ldb);
int rnpgpu_ctrsm_lunn(size_t n, size_t nrhs, const rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *b, size_t ldb);
int rnpgpu_ztrsm_lunn(size_t n, size_t nrhs, const rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *b, size_t ldb);

/* ---- Least squares min ||A x - B|| (m >= n, full column rank) by QR: the
 *      composition a caller of the reference writes — QR::Factor, then
 *      QR::MultQ("L","C") on B, then SolveTrM("L","U","N","N") (no single
 *      reference routine).  On exit A holds the factorization, tau the
 *      reflector scalars and B(0:n, :) the solution. ---- */
int rnpgpu_sgels(size_t m, size_t n, size_t nrhs, float *a, size_t lda, float *tau, float *b, size_t ldb, size_t *lwork, float *work);
int rnpgpu_dgels(size_t m, size_t n, size_t nrhs, double *a, size_t lda, double *tau, double *b, size_t ldb, size_t *lwork, double *work);
int rnpgpu_cgels(size_t m, size_t n, size_t nrhs, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, rnpgpu_complex_float *b, size_t ldb, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgels(size_t m, size_t n, size_t nrhs, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, rnpgpu_complex_double *b, size_t ldb, size_t *lwork, rnpgpu_complex_double *work);

/* ---- Mixed-precision least squares with iterative refinement (no reference
 *      counterpart): A is factored in FP32 (a working copy; A and B are not
 *      modified); the residual r = b - A x, the solution x and the error
 *      metrics are computed in FP64.  Steps  x += R^{-1} (Q^H r)(0:n)  run
 *      until the least-squares backward error bound
 *          max_j ||R^{-H} A^H r_j|| / ||x_j||
 *      (an upper bound of the Karlson-Walden estimate) and the normal-equation
 *      residual  max_j ||A^H r_j|| / (||A||_F (||A||_F ||x_j|| + ||b_j||))
 *      are both at most 10 n eps, the correction stops halving, or max_iter
 *      steps are taken (max_iter <= 0: 10, or 30 in forward mode).
 *      flags bit 0 (RNPGPU_REFINE_FORWARD): continue with corrected
 *      seminormal-equation steps  x += R^{-1} R^{-H} A^H r  until the
 *      correction stops shrinking, for FP64-level forward accuracy.
 *      flags bit 1 (RNPGPU_REFINE_RANK32_UPDATES): the real FP32 factor
 *      updates its trailing matrix after every 32-column panel on the CUDA
 *      cores instead of once per 128 columns on the tensor cores (for
 *      comparisons; the result is the same up to FP32 rounding).
 *      The loop reads a few norms back per step, so these calls synchronize
 *      their stream. ---- */
#define RNPGPU_REFINE_FORWARD 1
#define RNPGPU_REFINE_RANK32_UPDATES 2
typedef struct {
    int iterations;         /* refinement steps taken */
    int converged;          /* 1 if both error measures reached 10 n eps */
    double backward_error;  /* max_j ||R^{-H} A^H r_j|| / ||x_j|| */
    double normal_residual; /* max_j ||A^H r_j|| / (||A||_F (||A||_F ||x_j|| + ||b_j||)) */
    double correction;      /* max_j ||d_j|| / ||x_j|| of the last step */
    double anorm;           /* ||A||_F */
} rnpgpu_refine_info;

int rnpgpu_dsgels(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *b, size_t ldb, double *x, size_t ldx, int max_iter, int flags, rnpgpu_refine_info *info, size_t *lwork, double *work);
/* The same solve from HOST buffers a, b and x (pinned memory keeps the copies
 * asynchronous): A travels to the device in ranges of 128 columns on a copy
 * stream while the ranges already landed are prepared and factored (the
 * FP32 factor runs left-looking by 128-column blocks: each range is brought
 * up to date by the blocks left of it once it has landed); b travels on the
 * library's stream first and x comes back on it last.  work (device) holds
 * A, b and x (m n + m nrhs + n nrhs elements, each rounded up to 256 bytes),
 * the tensor-core slice images of every 128-column block of the factor but
 * the last (about 1.5 KB per row and block, so that each block is sliced
 * once) and the workspace of rnpgpu_dsgels; the query as rnpgpu_dsgels.  The call
 * returns with x enqueued (synchronize the library's stream before reading
 * it).  The stopping tests and the info are those of rnpgpu_dsgels; x agrees
 * with rnpgpu_dsgels's to the refinement's accuracy (the FP32 factor's
 * operations run in another order), and repeated calls give the same bits. */
int rnpgpu_dsgels_host(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *b, size_t ldb, double *x, size_t ldx, int max_iter, int flags, rnpgpu_refine_info *info, size_t *lwork, double *work);
int rnpgpu_zcgels(size_t m, size_t n, size_t nrhs, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *b, size_t ldb, rnpgpu_complex_double *x, size_t ldx, int max_iter, int flags, rnpgpu_refine_info *info, size_t *lwork, rnpgpu_complex_double *work);

/* ---- FP64-accurate residual of a real least-squares problem (no reference
 *      counterpart; the product a refinement loop needs): r = b - A x
 *      (m x nrhs) and, when g != NULL, g = A^T r (n x nrhs).  The products run
 *      on the BF16 tensor cores from exact fixed-point slices of A, x and r
 *      (eight 7-bit digits each, relative to per-column / per-right-hand-side
 *      powers of two), so the error is that of an FP64 dot product, about
 *      2^-50 of sum_k |a_ik| |x_kj| scaled to the column maxima; Inf or NaN in
 *      A or x makes the affected results NaN.  r may be b (in place).
 *      work: device workspace of *lwork_bytes bytes (query with work == NULL
 *      or *lwork_bytes == 0). ---- */
int rnpgpu_dls_residual(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *x, size_t ldx, const double *b, size_t ldb, double *r, size_t ldr, double *g, size_t ldg, void *work, size_t *lwork_bytes);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_LS_GB300_H */
