/* batched_gb300.h — batched Householder QR on the GB300 (no single reference
 * routine: the reference factors one matrix per QR::Factor call,
 * RNP/LA/QR.hpp:129-197; this runs many such calls in one persistent launch
 * with identical results per matrix).
 *
 * The matrices live in one packed DEVICE buffer: matrix i starts at element
 * a_offset[i], is m[i] x n[i] column-major with leading dimension lda[i]
 * (m[i] <= 256); its tau (min(m[i], n[i]) entries) starts at tau_offset[i]
 * of the tau buffer.  On exit each matrix holds R and its reflectors exactly
 * as after RNP::LA::QR::Factor.
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
int rnpgpu_batch_plan_destroy(rnpgpu_batch_plan *plan);
/* block shape (threads, panel width) and matrix count of size class cls (0 small, 1 large) */
int rnpgpu_batch_plan_config(const rnpgpu_batch_plan *plan, int cls, int *threads, int *nb, int *count);

int rnpgpu_sgeqrf_batched(const rnpgpu_batch_plan *plan, float *a, float *tau);
int rnpgpu_dgeqrf_batched(const rnpgpu_batch_plan *plan, double *a, double *tau);
int rnpgpu_cgeqrf_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_float *a, rnpgpu_complex_float *tau);
int rnpgpu_zgeqrf_batched(const rnpgpu_batch_plan *plan, rnpgpu_complex_double *a, rnpgpu_complex_double *tau);

int rnpgpu_sgeqrf_batched_tune(rnpgpu_batch_plan *plan, float *a, float *tau, double *ms);
int rnpgpu_dgeqrf_batched_tune(rnpgpu_batch_plan *plan, double *a, double *tau, double *ms);
int rnpgpu_cgeqrf_batched_tune(rnpgpu_batch_plan *plan, rnpgpu_complex_float *a, rnpgpu_complex_float *tau, double *ms);
int rnpgpu_zgeqrf_batched_tune(rnpgpu_batch_plan *plan, rnpgpu_complex_double *a, rnpgpu_complex_double *tau, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_BATCHED_GB300_H */
