// ref_driver.cpp — builds the REFERENCE ITSELF into a small shared library
// (oracle/_ref/libref_qr.so) so that golden vectors can be generated from it
// and the oracle restatement (qr_oracle.cpp) can be pinned against it.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile with the reference
// headers on the include path, where they lie (read-only); nothing of the
// reference is copied into this repository.  It needs the reference's source
// tree, so it is built only on a machine that has it; the golden fixtures it
// produces are committed under tests/golden/.
//
// Entry points mirror the reference API:
//   RNP::LA::QR::Factor / Factor_unblocked / MultQ / MultQ_unblocked /
//   GenerateQ / GenerateQ_unblocked   (RNP/LA/QR.hpp:78-570)
//   the same six for RNP::LA::LQ, QL and RQ (RNP/LA/LQ.hpp, QL.hpp, RQ.hpp)
//   RNP::Random::GenerateVector       (RNP/Random.hpp:262-320)
//   RNP::MatrixGen::RandomMatrix      (RNP/MatrixGen.hpp:120-203)
//   RNP::BLAS::SolveTrM               (RNP/BLAS/BLAS_mix.hpp:2096-2113)
//   RNP::LA::Hessenberg::Reduce / MultQ / GenerateQ   (RNP/LA/Hessenberg.hpp:351-590)
//   RNP::LA::Tridiagonal::ReduceHerm / MultQHerm / GenerateQHerm
//                                     (RNP/LA/Tridiagonal.hpp:924-1188)
//   the QR step of ComplexGeneralizedEigensystem, as the reference's own
//   calls in the order of RNP/LA/GeneralizedEigensystems.hpp:457-472
#include <RNP/LA/QR.hpp>
#include <RNP/LA/LQ.hpp>
#include <RNP/LA/QL.hpp>
#include <RNP/LA/RQ.hpp>
#include <RNP/Random.hpp>
#include <RNP/MatrixGen.hpp>
#include <RNP/LA/Hessenberg.hpp>
#include <RNP/LA/Tridiagonal.hpp>
#include <RNP/LA/Triangular.hpp>
#include <RNP/BLAS.hpp>
#include <complex>
#include <cstddef>

typedef std::complex<float> cf;
typedef std::complex<double> cd;

#define REF_DEF(P, T)                                                                                                   \
    extern "C" void ref_##P##geqrf(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {           \
        RNP::LA::QR::Factor<T>(m, n, a, lda, tau, lwork, work);                                                       \
    }                                                                                                                 \
    extern "C" void ref_##P##geqr2(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) {                           \
        RNP::LA::QR::Factor_unblocked<T>(m, n, a, lda, tau, work);                                                    \
    }                                                                                                                 \
    extern "C" void ref_##P##unmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a,     \
                                   size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {              \
        RNP::LA::QR::MultQ<T>(side, trans, m, n, k, a, lda, tau, c, ldc, lwork, work);                                \
    }                                                                                                                 \
    extern "C" void ref_##P##unm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a,     \
                                   size_t lda, const T *tau, T *c, size_t ldc, T *work) {                             \
        RNP::LA::QR::MultQ_unblocked<T>(side, trans, m, n, k, a, lda, tau, c, ldc, work);                             \
    }                                                                                                                 \
    extern "C" void ref_##P##ungqr(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork,      \
                                   T *work) {                                                                         \
        RNP::LA::QR::GenerateQ<T>(m, n, k, a, lda, tau, lwork, work);                                                 \
    }                                                                                                                 \
    extern "C" void ref_##P##ung2r(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) {           \
        RNP::LA::QR::GenerateQ_unblocked<T>(m, n, k, a, lda, tau, work);                                              \
    }                                                                                                                 \
    extern "C" void ref_##P##trsm_lunn(size_t n, size_t nrhs, const T *a, size_t lda, T *b, size_t ldb) {             \
        RNP::BLAS::SolveTrM("L", "U", "N", "N", n, nrhs, T(1), a, lda, b, ldb);                                      \
    }

// LQ / QL / RQ under LAPACK-style names (factor, unblocked factor, MultQ,
// unblocked MultQ, GenerateQ, unblocked GenerateQ)
#define REF_DEF2(P, T, NS, F, F2, M, M2, G, G2)                                                                         \
    extern "C" void ref_##P##F(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {                \
        RNP::LA::NS::Factor<T>(m, n, a, lda, tau, lwork, work);                                                       \
    }                                                                                                                 \
    extern "C" void ref_##P##F2(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) {                              \
        RNP::LA::NS::Factor_unblocked<T>(m, n, a, lda, tau, work);                                                    \
    }                                                                                                                 \
    extern "C" void ref_##P##M(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a,         \
                               size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {                  \
        RNP::LA::NS::MultQ<T>(side, trans, m, n, k, a, lda, tau, c, ldc, lwork, work);                                \
    }                                                                                                                 \
    extern "C" void ref_##P##M2(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a,        \
                                size_t lda, const T *tau, T *c, size_t ldc, T *work) {                                \
        RNP::LA::NS::MultQ_unblocked<T>(side, trans, m, n, k, a, lda, tau, c, ldc, work);                             \
    }                                                                                                                 \
    extern "C" void ref_##P##G(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) { \
        RNP::LA::NS::GenerateQ<T>(m, n, k, a, lda, tau, lwork, work);                                                 \
    }                                                                                                                 \
    extern "C" void ref_##P##G2(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) {              \
        RNP::LA::NS::GenerateQ_unblocked<T>(m, n, k, a, lda, tau, work);                                              \
    }
#define REF_DEF3(P, T)                                                             \
    REF_DEF2(P, T, LQ, gelqf, gelq2, unmlq, unml2, unglq, ungl2)                   \
    REF_DEF2(P, T, QL, geqlf, geql2, unmql, unm2l, ungql, ung2l)                   \
    REF_DEF2(P, T, RQ, gerqf, gerq2, unmrq, unmr2, ungrq, ungr2)

#define REF_RNG(P, T)                                                                                                   \
    extern "C" void ref_##P##larnv(int dist, int *iseed, size_t n, T *x) {                                            \
        RNP::Random::GenerateVector<T>((RNP::Random::Distribution::Distribution)dist, n, x, iseed);                   \
    }

#define REF_MG(P, T, R)                                                                                                 \
    extern "C" void ref_##P##random_matrix(int sym, int dist, int mode, int reverse, R cond, R dmax, R *d, size_t m,   \
                                           size_t n, T *a, size_t lda, int *iseed) {                                  \
        RNP::MatrixGen::RandomMatrix<T>((RNP::MatrixGen::Symmetry::Sym)sym, (RNP::Random::Distribution::Distribution)dist, \
                                        (RNP::MatrixGen::DiagonalMode::Mode)mode, reverse != 0, cond, dmax, d, m, n, a, lda, iseed); \
    }
// RandomMatrix compiles for real types only in the reference
// (RNP/MatrixGen.hpp:175 scales a real vector by a complex 1/wb)
REF_MG(s, float, float)
REF_MG(d, double, double)

REF_DEF(s, float)
REF_DEF(d, double)
REF_DEF(c, cf)
REF_DEF(z, cd)
REF_DEF3(s, float)
REF_DEF3(d, double)
REF_DEF3(c, cf)
REF_DEF3(z, cd)
// GenerateVector<std::complex<float> > does not compile in the reference
// (RNP/Random.hpp:213 mixes double and float), so no "c" generator here.
REF_RNG(s, float)
REF_RNG(d, double)
REF_RNG(z, cd)

// callers of QR / QL (LAPACK names: gehrd, unmhr, unghr, hetrd, unmtr, ungtr)
#define REF_CONS(P, T, R)                                                                                               \
    extern "C" void ref_##P##gehrd(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, T *tau, size_t *lwork, T *work) { \
        RNP::LA::Hessenberg::Reduce<T>(n, ilo, ihi, a, lda, tau, lwork, work);                                        \
    }                                                                                                                 \
    extern "C" void ref_##P##unmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi,  \
                                   const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {  \
        RNP::LA::Hessenberg::MultQ<T>(side, trans, m, n, ilo, ihi, a, lda, tau, c, ldc, lwork, work);                 \
    }                                                                                                                 \
    extern "C" void ref_##P##unghr(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, const T *tau, size_t *lwork,  \
                                   T *work) {                                                                         \
        RNP::LA::Hessenberg::GenerateQ<T>(n, ilo, ihi, a, lda, tau, lwork, work);                                     \
    }                                                                                                                 \
    extern "C" void ref_##P##hetrd(const char *uplo, size_t n, T *a, size_t lda, R *diag, R *offdiag, T *tau,         \
                                   size_t *lwork, T *work) {                                                          \
        RNP::LA::Tridiagonal::ReduceHerm<T>(uplo, n, a, lda, diag, offdiag, tau, lwork, work);                        \
    }                                                                                                                 \
    extern "C" void ref_##P##ungtr(const char *uplo, size_t n, T *a, size_t lda, const T *tau, size_t *lwork,         \
                                   T *work) {                                                                         \
        RNP::LA::Tridiagonal::GenerateQHerm<T>(uplo, n, a, lda, tau, lwork, work);                                    \
    }                                                                                                                 \
    extern "C" void ref_##P##unmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n,         \
                                   const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {  \
        RNP::LA::Tridiagonal::MultQHerm<T>(side, uplo, trans, m, n, a, lda, tau, c, ldc, lwork, work);                \
    }
REF_CONS(s, float, float)
REF_CONS(d, double, double)
REF_CONS(c, cf, float)
REF_CONS(z, cd, double)

// ComplexGeneralizedEigensystem's QR step: the reference's calls of
// RNP/LA/GeneralizedEigensystems.hpp:457-472 in their order, with its
// workspace layout [tau | work] (the driver itself also balances, reduces and
// iterates, none of which calls QR)
#define REF_GG(P, T)                                                                                                    \
    extern "C" void ref_##P##gg_triangularize_b(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, T *b, size_t ldb, \
                                                T *vl, size_t ldvl, T *vr, size_t ldvr, size_t lwork, T *work) {      \
        const T zero(0), one(1);                                                                                      \
        const size_t irows = ihi - ilo;                                                                               \
        const size_t icols = (NULL != vl || NULL != vr) ? n - ilo : irows;                                            \
        T *tau = work;                                                                                                \
        T *work2 = tau + n;                                                                                           \
        size_t lwork2 = lwork - n;                                                                                    \
        RNP::LA::QR::Factor(irows, icols, &b[ilo + ilo * ldb], ldb, tau, &lwork2, work2);                             \
        RNP::LA::QR::MultQ("L", "C", irows, icols, irows, &b[ilo + ilo * ldb], ldb, tau, &a[ilo + ilo * lda], lda,    \
                           &lwork2, work2);                                                                           \
        if (NULL != vl) {                                                                                             \
            RNP::BLAS::Set(n, n, zero, one, vl, ldvl);                                                                \
            if (irows > 1)                                                                                            \
                RNP::LA::Triangular::Copy("L", irows - 1, irows - 1, &b[ilo + 1 + ilo * ldb], ldb,                    \
                                          &vl[ilo + 1 + ilo * ldvl], ldvl);                                           \
            RNP::LA::QR::GenerateQ(irows, irows, irows, &vl[ilo + ilo * ldvl], ldvl, tau, &lwork2, work2);            \
        }                                                                                                             \
        if (NULL != vr) RNP::BLAS::Set(n, n, zero, one, vr, ldvr);                                                    \
    }
REF_GG(c, cf)
REF_GG(z, cd)
