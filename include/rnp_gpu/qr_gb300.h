/* qr_gb300.h — C ABI of the GB300 blocked Householder QR.
 *
 * Drop-in for the QR path of RNP2 (RNP::LA::QR, RNP/LA/QR.hpp).  Every
 * entry point keeps the argument list, meaning and storage convention of the
 * reference routine it replaces:
 *   - column-major matrices with leading dimension lda/ldc, 0-based offsets
 *     are expressed by passing offset pointers, as in the reference;
 *   - R in the upper triangle/trapezoid of A, the reflector vectors v below
 *     the diagonal (v[i] = 1 implicit), tau[i] the reflector scalars, so that
 *     H[i] = I - tau[i] v v^H and Q = H[0] H[1] ... H[k-1];
 *   - caller-owned work blocks with RNP's query: work == NULL or *lwork == 0
 *     stores the optimal length (in elements of the scalar type) in *lwork
 *     and returns.  A smaller *lwork selects smaller splits, then the
 *     level-2 code (which needs n, resp. the reference's length);
 *   - the library never allocates memory.
 * Differences forced by the device:
 *   - a, tau, c and work are DEVICE pointers (cudaMalloc'd or managed);
 *   - calls are asynchronous on the stream set by rnpgpu_set_stream (default
 *     stream 0); results are ready when that stream is synchronized;
 *   - the reference returns void and only prints failed preconditions
 *     (RNP/Debug.hpp:4-17); here every entry point returns an int status:
 *       0   success,
 *      -i   the i-th argument (1-based) is invalid; nothing was enqueued,
 *      >0   a CUDA error (message in rnpgpu_get_last_error()).
 * Complex arguments are (re, im) pairs, layout-compatible with
 * std::complex<T> and C99 _Complex.
 */
#ifndef RNP_GPU_QR_GB300_H
#define RNP_GPU_QR_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float re, im; } rnpgpu_complex_float;
typedef struct { double re, im; } rnpgpu_complex_double;

#define RNPGPU_OK 0
#define RNPGPU_ERR_CUDA 1
#define RNPGPU_ERR_DEVICE 2

/* ---- Factor: RNP::LA::QR::Factor (RNP/LA/QR.hpp:129-197), LAPACK _geqrf ---- */
int rnpgpu_sgeqrf(size_t m, size_t n, float *a, size_t lda, float *tau, size_t *lwork, float *work);
int rnpgpu_dgeqrf(size_t m, size_t n, double *a, size_t lda, double *tau, size_t *lwork, double *work);
int rnpgpu_cgeqrf(size_t m, size_t n, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zgeqrf(size_t m, size_t n, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);

/* ---- Factor without a work block (no counterpart in the reference): the
 *      same factorization as rnpgpu_dgeqrf for callers that cannot allocate
 *      device memory (frameworks that own and pre-budget it, fixed-budget
 *      real-time loops).  It uses an 8 MiB scratch array built into the
 *      library and always factors in the serial order, so n up to 16,000
 *      columns always fits (status -2 past about 16,100, message in
 *      rnpgpu_get_last_error()).  The first call on a device looks up the
 *      array's address and should come before any stream capture; calls that
 *      overlap on the GPU share the array and race. ---- */
int rnpgpu_dgeqrf_noalloc(size_t m, size_t n, double *a, size_t lda, double *tau);

/* ---- Factor_unblocked: RNP::LA::QR::Factor_unblocked (RNP/LA/QR.hpp:78-102), _geqr2; work: n ---- */
int rnpgpu_sgeqr2(size_t m, size_t n, float *a, size_t lda, float *tau, float *work);
int rnpgpu_dgeqr2(size_t m, size_t n, double *a, size_t lda, double *tau, double *work);
int rnpgpu_cgeqr2(size_t m, size_t n, rnpgpu_complex_float *a, size_t lda, rnpgpu_complex_float *tau, rnpgpu_complex_float *work);
int rnpgpu_zgeqr2(size_t m, size_t n, rnpgpu_complex_double *a, size_t lda, rnpgpu_complex_double *tau, rnpgpu_complex_double *work);

/* ---- MultQ: RNP::LA::QR::MultQ (RNP/LA/QR.hpp:337-429), _unmqr/_ormqr.
 *      side "L"/"R", trans "N"/"C" (first character read, as in the reference) ---- */
int rnpgpu_sunmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const float *a, size_t lda, const float *tau, float *c, size_t ldc, size_t *lwork, float *work);
int rnpgpu_dunmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const double *a, size_t lda, const double *tau, double *c, size_t ldc, size_t *lwork, double *work);
int rnpgpu_cunmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zunmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, size_t *lwork, rnpgpu_complex_double *work);

/* ---- MultQ_unblocked: RNP::LA::QR::MultQ_unblocked (RNP/LA/QR.hpp:234-298), _unm2r; work: n ("L") or m ("R") ---- */
int rnpgpu_sunm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const float *a, size_t lda, const float *tau, float *c, size_t ldc, float *work);
int rnpgpu_dunm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const double *a, size_t lda, const double *tau, double *c, size_t ldc, double *work);
int rnpgpu_cunm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *c, size_t ldc, rnpgpu_complex_float *work);
int rnpgpu_zunm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *c, size_t ldc, rnpgpu_complex_double *work);

/* ---- GenerateQ: RNP::LA::QR::GenerateQ (RNP/LA/QR.hpp:509-570), _ungqr/_orgqr; m >= n >= k ---- */
int rnpgpu_sungqr(size_t m, size_t n, size_t k, float *a, size_t lda, const float *tau, size_t *lwork, float *work);
int rnpgpu_dungqr(size_t m, size_t n, size_t k, double *a, size_t lda, const double *tau, size_t *lwork, double *work);
int rnpgpu_cungqr(size_t m, size_t n, size_t k, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, size_t *lwork, rnpgpu_complex_float *work);
int rnpgpu_zungqr(size_t m, size_t n, size_t k, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, size_t *lwork, rnpgpu_complex_double *work);

/* ---- GenerateQ_unblocked: RNP::LA::QR::GenerateQ_unblocked (RNP/LA/QR.hpp:451-485), _ung2r; work: n ---- */
int rnpgpu_sung2r(size_t m, size_t n, size_t k, float *a, size_t lda, const float *tau, float *work);
int rnpgpu_dung2r(size_t m, size_t n, size_t k, double *a, size_t lda, const double *tau, double *work);
int rnpgpu_cung2r(size_t m, size_t n, size_t k, rnpgpu_complex_float *a, size_t lda, const rnpgpu_complex_float *tau, rnpgpu_complex_float *work);
int rnpgpu_zung2r(size_t m, size_t n, size_t k, rnpgpu_complex_double *a, size_t lda, const rnpgpu_complex_double *tau, rnpgpu_complex_double *work);

/* ---- Library context (no counterpart in the reference, which is synchronous) ---- */
/* Stream used by the calling host thread (a cudaStream_t; NULL = default stream). */
int rnpgpu_set_stream(void *stream);
void *rnpgpu_get_stream(void);
/* Message of the last CUDA error seen by the calling thread ("" if none). */
const char *rnpgpu_get_last_error(void);
/* Library version string. */
const char *rnpgpu_version(void);
/* Device-side status of the tensor-core kernels: nonzero if one of their
 * bounded waits gave up (its results are then not valid); reset != 0 clears
 * it.  Synchronous. */
int rnpgpu_device_status(int reset);
/* C = alpha op(A) op(B) + beta C in FP32 on the tensor cores (each operand
 * split into three BF16 terms, six products, FP32 accumulation); op "N" or
 * "T", beta 0 or 1.  No counterpart in the reference: the tensor-core
 * contraction the library uses for short FP32 contractions (K <= 64) that are
 * not a trailing update, exported for checking. */
int rnpgpu_sgemm_tc(const char *transa, const char *transb, size_t m, size_t n, size_t k, float alpha, const float *a, size_t lda, const float *b, size_t ldb, float beta, float *c, size_t ldc);
/* The FP32 factorization the mixed least-squares solvers use internally
 * (rnpgpu_dsgels), exported for checking; no counterpart in the reference.
 * Same storage as rnpgpu_sgeqrf (R, V, tau) and the 32 x 32 T factor of every
 * 32-column block in tstore (block b at tstore + 1024 b, leading dimension
 * 32).  Panels: CholeskyQR2 with Householder reconstruction (Householder
 * panels for the whole matrix when a panel is too ill-conditioned for it;
 * *cqr_failed, if given, reports that, and the call then synchronizes).
 * Trailing matrix: one update per 128 columns on the tensor cores when
 * m >= n > 128, m >= 256, lda % 4 == 0 and a is 16-byte aligned, unless flags
 * bit 1 (RNPGPU_REFINE_RANK32_UPDATES in ls_gb300.h) asks for the rank-32
 * updates after every panel.  Workspace query as rnpgpu_sgeqrf. */
int rnpgpu_sgeqrf_mixed(size_t m, size_t n, float *a, size_t lda, float *tau, float *tstore, int flags, int *cqr_failed, size_t *lwork, float *work);
/* Number of kernels this library has launched in this process. */
unsigned long long rnpgpu_launch_count(void);
/* Per-kernel-class timing with CUDA events on the launching stream, for the
 * calling thread: enable/disable, then read "name count total_ms" lines
 * (since the last report) into buf; returns the report's length. */
int rnpgpu_timing_enable(int on);
int rnpgpu_timing_report(char *buf, size_t len);
/* Measured throughput of the current device in TFLOP/s (kind 0: FP64 FMA,
 * kind 1: FP32 FMA, kind 2: FP64 tensor-core MMA, mma.sync m8n8k4), using
 * scratch (>= SMs*8*256 doubles) for the probe's outputs; synchronous.  Used
 * as the roofline denominator of FP64 work and to re-check that the FP64
 * contractions belong on the FMA pipe.  Kinds 3-5 return SM clock cycles
 * instead: 3 the latency of a dependent FP64 FMA, 4 the interval between FP64
 * instructions of one warp with independent work, 5 the latency of an FP64
 * division (the figures behind keeping FP64 work off serial paths). */
int rnpgpu_probe_peak(int kind, void *scratch, size_t scratch_bytes, double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_QR_GB300_H */
