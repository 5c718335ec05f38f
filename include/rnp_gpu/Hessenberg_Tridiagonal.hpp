// Hessenberg_Tridiagonal.hpp — the reference's callers of QR and QL on the
// GB300, with its template signatures: RNP::LA::Hessenberg::MultQ and
// GenerateQ (RNP/LA/Hessenberg.hpp:477-590) and RNP::LA::Tridiagonal::
// GenerateQHerm and MultQHerm (RNP/LA/Tridiagonal.hpp:1037-1188).  The
// reductions themselves (Hessenberg::Reduce, Tridiagonal::ReduceHerm) are not
// provided on the GPU; their output is the input of these routines.
//
//   RNP::LA::Hessenberg::GenerateQ(n, ilo, ihi, a, lda, tau, &lwork, work);
//   RNP::LA::Tridiagonal::MultQHerm("L", "U", "N", m, n, a, lda, tau, c, ldc, &lwork, work);
//
// Device pointers; the calls enqueue on the stream set with
// rnpgpu_set_stream() and return without synchronizing.  Like the reference
// they return void and print failed preconditions; the status of the last
// call is in GPUStatus() of each namespace.
#ifndef RNP_GPU_HESSENBERG_TRIDIAGONAL_HPP_INCLUDED
#define RNP_GPU_HESSENBERG_TRIDIAGONAL_HPP_INCLUDED

#include <complex>
#include <cstddef>
#include <cstdio>

#include "consumers_gb300.h"

namespace RNP {
namespace LA {
namespace consumers_detail {
template <typename T> struct Abi;
template <> struct Abi<float> {
    typedef float C;
    static int mhr(const char *s, const char *tr, size_t m, size_t n, size_t ilo, size_t ihi, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmhr(s, tr, m, n, ilo, ihi, a, lda, t, c, ldc, lw, w); }
    static int ghr(size_t n, size_t ilo, size_t ihi, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sunghr(n, ilo, ihi, a, lda, t, lw, w); }
    static int gtr(const char *u, size_t n, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sungtr(u, n, a, lda, t, lw, w); }
    static int mtr(const char *s, const char *u, const char *tr, size_t m, size_t n, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmtr(s, u, tr, m, n, a, lda, t, c, ldc, lw, w); }
};
template <> struct Abi<double> {
    typedef double C;
    static int mhr(const char *s, const char *tr, size_t m, size_t n, size_t ilo, size_t ihi, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmhr(s, tr, m, n, ilo, ihi, a, lda, t, c, ldc, lw, w); }
    static int ghr(size_t n, size_t ilo, size_t ihi, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dunghr(n, ilo, ihi, a, lda, t, lw, w); }
    static int gtr(const char *u, size_t n, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dungtr(u, n, a, lda, t, lw, w); }
    static int mtr(const char *s, const char *u, const char *tr, size_t m, size_t n, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmtr(s, u, tr, m, n, a, lda, t, c, ldc, lw, w); }
};
template <> struct Abi<std::complex<float>> {
    typedef rnpgpu_complex_float C;
    static int mhr(const char *s, const char *tr, size_t m, size_t n, size_t ilo, size_t ihi, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmhr(s, tr, m, n, ilo, ihi, a, lda, t, c, ldc, lw, w); }
    static int ghr(size_t n, size_t ilo, size_t ihi, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cunghr(n, ilo, ihi, a, lda, t, lw, w); }
    static int gtr(const char *u, size_t n, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cungtr(u, n, a, lda, t, lw, w); }
    static int mtr(const char *s, const char *u, const char *tr, size_t m, size_t n, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmtr(s, u, tr, m, n, a, lda, t, c, ldc, lw, w); }
};
template <> struct Abi<std::complex<double>> {
    typedef rnpgpu_complex_double C;
    static int mhr(const char *s, const char *tr, size_t m, size_t n, size_t ilo, size_t ihi, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmhr(s, tr, m, n, ilo, ihi, a, lda, t, c, ldc, lw, w); }
    static int ghr(size_t n, size_t ilo, size_t ihi, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zunghr(n, ilo, ihi, a, lda, t, lw, w); }
    static int gtr(const char *u, size_t n, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zungtr(u, n, a, lda, t, lw, w); }
    static int mtr(const char *s, const char *u, const char *tr, size_t m, size_t n, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmtr(s, u, tr, m, n, a, lda, t, c, ldc, lw, w); }
};
template <typename T> inline typename Abi<T>::C *cp(T *p) { return reinterpret_cast<typename Abi<T>::C *>(p); }
template <typename T> inline const typename Abi<T>::C *cp(const T *p) { return reinterpret_cast<const typename Abi<T>::C *>(p); }
inline void report(int &status, const char *ns, const char *routine, int rc) {
    status = rc;
    if (rc != 0)
        std::fprintf(stderr, "RNP::LA::%s::%s (GB300) failed: status %d %s\n", ns, routine, rc, rc > 0 ? rnpgpu_get_last_error() : "(bad argument)");
}
} // namespace consumers_detail

namespace Hessenberg {
inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
// RNP/LA/Hessenberg.hpp:477-512
template <typename T>
void MultQ(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    using namespace consumers_detail;
    report(GPUStatus(), "Hessenberg", "MultQ", Abi<T>::mhr(side, trans, m, n, ilo, ihi, cp(a), lda, cp(tau), cp(c), ldc, lwork, cp(work)));
}
// RNP/LA/Hessenberg.hpp:539-590
template <typename T> void GenerateQ(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    using namespace consumers_detail;
    report(GPUStatus(), "Hessenberg", "GenerateQ", Abi<T>::ghr(n, ilo, ihi, cp(a), lda, cp(tau), lwork, cp(work)));
}
} // namespace Hessenberg

namespace Tridiagonal {
inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
// RNP/LA/Tridiagonal.hpp:1037-1097
template <typename T> void GenerateQHerm(const char *uplo, size_t n, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    using namespace consumers_detail;
    report(GPUStatus(), "Tridiagonal", "GenerateQHerm", Abi<T>::gtr(uplo, n, cp(a), lda, cp(tau), lwork, cp(work)));
}
// RNP/LA/Tridiagonal.hpp:1140-1188
template <typename T>
void MultQHerm(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    using namespace consumers_detail;
    report(GPUStatus(), "Tridiagonal", "MultQHerm", Abi<T>::mtr(side, uplo, trans, m, n, cp(a), lda, cp(tau), cp(c), ldc, lwork, cp(work)));
}
} // namespace Tridiagonal

} // namespace LA
} // namespace RNP

#endif
