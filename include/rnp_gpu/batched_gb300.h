/* batched_gb300.h — batched Householder QR on the GB300 (no single reference
 * routine: the reference factors one matrix per QR::Factor call,
 * RNP/LA/QR.hpp:129-197; this runs many such calls in one persistent launch
 * with identical results per matrix).
 *
 * The matrices live in one packed DEVICE buffer: matrix i starts at element
 * a_offset[i], is m[i] x n[i] column-major with leading dimension lda[i]
 * (m[i] <= 512); its tau (min(m[i], n[i]) entries) starts at tau_offset[i]
 * of the tau buffer.  On exit each matrix holds R and its reflectors exactly
 * as after RNP::LA::QR::Factor.  The plan splits the batch into four size
 * classes: m, n <= 32 (one warp per matrix, or a small block, as the
 * autotuner finds faster) and m <= 64, <= 256, <= 512 (one block per matrix).
 *
 *   1. rnpgpu_geqrf_batched_plan(type, batch, m, n, lda, a_offset,
 *      tau_offset, work, &lwork_bytes, &plan): HOST arrays; query the device
 *      workspace size with work == NULL, then build the plan (sorts by cost,
 *      splits small/large size classes, uploads descriptors into work).
 *      type: 0 float, 1 double, 2 complex float, 3 complex double.
 *   2. optional rnpgpu_{s,d,c,z}geqrf_batched_tune with (plan, a_scratch, tau_scratch,
 *      &ms): times the candidate block shapes per class on a scratch copy of
 *      the batch (overwritten) and keeps the fastest in the plan.
 *   3. rnpgpu_{s,d,c,z}geqrf_batched with (plan, a, tau): factors the batch on the current
 *      stream (memset + one persistent kernel per size class, the classes on
 *      two streams joined back); capturable into a CUDA graph.
 *   4. rnpgpu_batch_plan_destroy(plan).
 * The plan's workspace must outlive every run; runs of one plan must not
 * overlap on the GPU (they share its work-queue counters).
 *
 * Batched least squares (no single reference routine either: per problem,
 * the composition Factor, MultQ("L","C"), upper triangular solve of
 * RNP/LA/QR.hpp and RNP/BLAS/BLAS_mix.hpp:2096-2113), one right-hand side per
 * problem, m[i] >= n[i]: the plan comes from rnpgpu_gels_batched_plan, which
 * also takes b_offset[i] (m[i] entries of b) and x_offset[i] (n[i] entries of
 * x) into the packed b and x buffers.
 *   plain, in the plan's precision: rnpgpu_{s,d,c,z}gels_batched with
 *     (plan, a, tau, b, x): factors a in place, then one warp per problem
 *     writes x = R^{-1} (Q^H b)(0:n).
 *   mixed: rnpgpu_dsgels_batched / rnpgpu_zcgels_batched with (plan, a, b,
 *     x, max_iter, iters, berr, eta, work, &lwork_bytes): a FP32 copy of every
 *     problem is factored in work (query its size with work == NULL), then
 *     one warp per problem refines x in FP64 (Q steps, then corrected
 *     seminormal steps) until the backward error estimate
 *     berr[i] = ||R^{-H} A^H r|| / ||x|| and the normal residual
 *     eta[i] = ||A^H r|| / (||A||_F (||A||_F ||x|| + ||b||)) are both below
 *     10 n[i] eps, or the correction stops shrinking (max_iter <= 0: 10).
 *     iters, berr, eta: device arrays indexed like the batch, or NULL.
 *     The _tune variants (plan, a, work, &lwork_bytes, &ms) time the block
 *     shapes of the FP32 factorization on the workspace copy.
 */
#ifndef RNP_GPU_BATCHED_GB300_H
#define RNP_GPU_BATCHED_GB300_H

#include <stddef.h>
#include "qr_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rnpgpu_batch_plan rnpgpu_batch_plan;

int rnpgpu_geqrf_batched_plan(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_offset, const long long *tau_offset, void *work, size_t *lwork_bytes, rnpgpu_batch_plan **plan);
int rnpgpu_gels_batched_plan(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_offset, const long long *tau_offset, const long long *b_offset, const long long *x_offset, void *work, size_t *lwork_bytes, rnpgpu_batch_plan **plan);
int rnpgpu_batch_plan_destroy(rnpgpu_batch_plan *plan);
/* block shape (threads, panel width; threads == 32: one warp per matrix) and
   matrix count of size class cls (0 .. 3) */
int rnpgpu_batch_plan_config(const rnpgpu_batch_plan *plan, int cls, int *threads, int *nb, int *count);
/* set the block shape of class cls to one of the autotuner's candidates
   (class 0: (32, 0) one warp per matrix, or (64, 8); class 1: (64|128, 8),
   (128, 16); class 2: (128, 8|16), (256, 16|32); class 3: (256, 8|16),
   (512, 16)); -3 for any other shape */
int rnpgpu_batch_plan_set_config(rnpgpu_batch_plan *plan, int cls, int threads, int nb);

int rnpgpu_sgeqrf_batched(const rnpgpu_batch_plan *plan, float *a, float *tau);
int rnpgpu_dgeqrf_batched(const rnpgpu_batch_plan *plan, double *a, double *tau);
int rnpgpu_cgeqrf_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_float *a, rnpgpu_complex_float *tau);
int rnpgpu_zgeqrf_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_double *a, rnpgpu_complex_double *tau);

int rnpgpu_sgeqrf_batched_tune(rnpgpu_batch_plan *plan, float *a, float *tau, double *ms);
int rnpgpu_dgeqrf_batched_tune(rnpgpu_batch_plan *plan, double *a, double *tau, double *ms);
int rnpgpu_cgeqrf_batched_tune(rnpgpu_batch_plan *plan, rnpgpu_complex_float *a, rnpgpu_complex_float *tau, double *ms);
int rnpgpu_zgeqrf_batched_tune(rnpgpu_batch_plan *plan, rnpgpu_complex_double *a, rnpgpu_complex_double *tau, double *ms);

int rnpgpu_sgels_batched(const rnpgpu_batch_plan *plan, float *a, float *tau, const float *b, float *x);
int rnpgpu_dgels_batched(const rnpgpu_batch_plan *plan, double *a, double *tau, const double *b, double *x);
int rnpgpu_cgels_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_float *a, rnpgpu_complex_float *tau, const rnpgpu_complex_float *b, rnpgpu_complex_float *x);
int rnpgpu_zgels_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_double *a, rnpgpu_complex_double *tau, const rnpgpu_complex_double *b, rnpgpu_complex_double *x);

int rnpgpu_dsgels_batched(const rnpgpu_batch_plan *plan, const double *a, const double *b, double *x, int max_iter, int *iters, double *berr, double *eta, void *work, size_t *lwork_bytes);
int rnpgpu_zcgels_batched(const rnpgpu_batch_plan *plan, const rnpgpu_complex_double *a, const rnpgpu_complex_double *b, rnpgpu_complex_double *x, int max_iter, int *iters, double *berr, double *eta, void *work, size_t *lwork_bytes);
int rnpgpu_dsgels_batched_tune(rnpgpu_batch_plan *plan, const double *a, void *work, size_t *lwork_bytes, double *ms);
int rnpgpu_zcgels_batched_tune(rnpgpu_batch_plan *plan, const rnpgpu_complex_double *a, void *work, size_t *lwork_bytes, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_BATCHED_GB300_H */
