/* matgen_gb300.h — RNP::MatrixGen::RandomMatrix (RNP/MatrixGen.hpp:120-272,
 * with GenerateDiagonal :31-109) on the GPU, for float and double (the
 * reference's RandomMatrix compiles for real types only).
 *
 *   sym    0 Nonsymmetric, 1 Hermitian (random signs on d), 2 Hermitian
 *          positive definite, 3 Symmetric (1-3: m == n)
 *   dist   RNP::Random::Distribution of d for mode 6: 0 Uniform01,
 *          1 Uniform_11, 2 Normal01, 3 UnitDisc, 4 UnitCircle
 *   mode   RNP::MatrixGen::DiagonalMode: 0 Given (d read), 1 First1RemainingCond,
 *          2 LastCondRemaining1, 3 GradedExponentially, 4 GradedLinearly,
 *          5 RandomExponential, 6 RandomDist
 *   reverse  as the reference's argument; its reversal loop swaps every
 *          pair twice and leaves d unchanged, and so does this one
 *   cond, dmax  condition number (>= 1) and largest |d| (modes 1-5)
 *   d      device, min(m,n): read for mode 0, otherwise written when not NULL
 *   a      device, m x n (lda)
 *   iseed  HOST, 4 ints: the reference's seed, advanced past every number
 *          drawn exactly as the reference leaves it
 * A = U diag(d) V^H with U, V products of Householder reflectors drawn from
 * Normal01 vectors of the reference's generator (every uniform bit-identical
 * to the reference's).  Workspace query as the QR routines (work == NULL or
 * *lwork == 0).  The call synchronizes its stream.  Status 0, -i for
 * argument i, > 0 for a CUDA error. */
#ifndef RNP_GPU_MATGEN_GB300_H
#define RNP_GPU_MATGEN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

int rnpgpu_srandom_matrix(int sym, int dist, int mode, int reverse, float cond, float dmax, float *d, size_t m, size_t n, float *a, size_t lda, int *iseed, size_t *lwork,
                          float *work);
int rnpgpu_drandom_matrix(int sym, int dist, int mode, int reverse, double cond, double dmax, double *d, size_t m, size_t n, double *a, size_t lda, int *iseed,
                          size_t *lwork, double *work);

#ifdef __cplusplus
}
#endif

#endif /* RNP_GPU_MATGEN_GB300_H */
