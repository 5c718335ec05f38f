// QR.hpp — RNP::LA::QR on the GB300, with the reference's template signatures
// (RNP/LA/QR.hpp:41-570).  Include this instead of <RNP/LA/QR.hpp> to run the
// same calls on the GPU:
//
//   RNP::LA::QR::Factor(m, n, a, lda, tau, &lwork, work);           // QR.hpp:129-132
//   RNP::LA::QR::MultQ("L", "C", m, n, k, a, lda, tau, c, ldc, &lwork, work);  // QR.hpp:337-342
//   RNP::LA::QR::GenerateQ(m, n, k, a, lda, tau, &lwork, work);     // QR.hpp:509-513
//   (+ Factor_unblocked, MultQ_unblocked, GenerateQ_unblocked, Tuning<T>)
//
// T is float, double, std::complex<float> or std::complex<double>.  a, tau,
// c and work are device pointers; the calls enqueue on the stream set with
// rnpgpu_set_stream() and return without synchronizing.  The reference's
// routines return void and only print failed preconditions
// (RNP/Debug.hpp:4-17); these do the same (void, message on stderr) and keep
// the status of the last call in RNP::LA::QR::GPUStatus() (0 = ok, -i = bad
// argument i, > 0 = CUDA error).
#ifndef RNP_GPU_QR_HPP_INCLUDED
#define RNP_GPU_QR_HPP_INCLUDED

#include <complex>
#include <cstddef>
#include <cstdio>

#include "qr_gb300.h"

namespace RNP {
namespace LA {
namespace QR {

inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
inline void GPUReport(const char *routine, int rc) {
    GPUStatus() = rc;
    if (rc != 0)
        std::fprintf(stderr, "RNP::LA::QR::%s (GB300) failed: status %d %s\n", routine, rc, rc > 0 ? rnpgpu_get_last_error() : "(bad argument)");
}

// Block sizes are fixed by the GPU kernels (32-column panels); the structure
// is kept so code that specializes it still compiles (RNP/LA/QR.hpp:41-51).
template <typename T> struct Tuning {
    static size_t factor_block_size_opt(size_t, size_t) { return 32; }
    static size_t factor_block_size_min(size_t, size_t) { return 2; }
    static size_t factor_crossover_size(size_t, size_t) { return 0; }
    static size_t multQ_block_size_opt(const char *, const char *, size_t, size_t, size_t) { return 32; }
    static size_t multQ_block_size_min(const char *, const char *, size_t, size_t, size_t) { return 2; }
    static size_t genQ_block_size_opt(size_t, size_t, size_t) { return 32; }
    static size_t genQ_block_size_min(size_t, size_t, size_t) { return 2; }
    static size_t genQ_crossover_size(size_t, size_t, size_t) { return 0; }
};

namespace detail {
template <typename T> struct Abi;
template <> struct Abi<float> {
    typedef float C;
    static int geqrf(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_sgeqrf(m, n, a, lda, t, lw, w); }
    static int geqr2(size_t m, size_t n, C *a, size_t lda, C *t, C *w) { return rnpgpu_sgeqr2(m, n, a, lda, t, w); }
    static int unmqr(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmqr(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int unm2r(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, C *w) { return rnpgpu_sunm2r(s, tr, m, n, k, a, lda, t, c, ldc, w); }
    static int ungqr(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sungqr(m, n, k, a, lda, t, lw, w); }
    static int ung2r(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, C *w) { return rnpgpu_sung2r(m, n, k, a, lda, t, w); }
};
template <> struct Abi<double> {
    typedef double C;
    static int geqrf(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_dgeqrf(m, n, a, lda, t, lw, w); }
    static int geqr2(size_t m, size_t n, C *a, size_t lda, C *t, C *w) { return rnpgpu_dgeqr2(m, n, a, lda, t, w); }
    static int unmqr(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmqr(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int unm2r(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, C *w) { return rnpgpu_dunm2r(s, tr, m, n, k, a, lda, t, c, ldc, w); }
    static int ungqr(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dungqr(m, n, k, a, lda, t, lw, w); }
    static int ung2r(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, C *w) { return rnpgpu_dung2r(m, n, k, a, lda, t, w); }
};
template <> struct Abi<std::complex<float> > {
    typedef rnpgpu_complex_float C;
    static int geqrf(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_cgeqrf(m, n, a, lda, t, lw, w); }
    static int geqr2(size_t m, size_t n, C *a, size_t lda, C *t, C *w) { return rnpgpu_cgeqr2(m, n, a, lda, t, w); }
    static int unmqr(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmqr(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int unm2r(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, C *w) { return rnpgpu_cunm2r(s, tr, m, n, k, a, lda, t, c, ldc, w); }
    static int ungqr(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cungqr(m, n, k, a, lda, t, lw, w); }
    static int ung2r(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, C *w) { return rnpgpu_cung2r(m, n, k, a, lda, t, w); }
};
template <> struct Abi<std::complex<double> > {
    typedef rnpgpu_complex_double C;
    static int geqrf(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_zgeqrf(m, n, a, lda, t, lw, w); }
    static int geqr2(size_t m, size_t n, C *a, size_t lda, C *t, C *w) { return rnpgpu_zgeqr2(m, n, a, lda, t, w); }
    static int unmqr(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmqr(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int unm2r(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, C *w) { return rnpgpu_zunm2r(s, tr, m, n, k, a, lda, t, c, ldc, w); }
    static int ungqr(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zungqr(m, n, k, a, lda, t, lw, w); }
    static int ung2r(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, C *w) { return rnpgpu_zung2r(m, n, k, a, lda, t, w); }
};
template <typename T> inline typename Abi<T>::C *cp(T *p) { return reinterpret_cast<typename Abi<T>::C *>(p); }
template <typename T> inline const typename Abi<T>::C *cp(const T *p) { return reinterpret_cast<const typename Abi<T>::C *>(p); }
} // namespace detail

// RNP/LA/QR.hpp:78-102
template <typename T> void Factor_unblocked(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) {
    GPUReport("Factor_unblocked", detail::Abi<T>::geqr2(m, n, detail::cp(a), lda, detail::cp(tau), detail::cp(work)));
}
// RNP/LA/QR.hpp:129-197
template <typename T> void Factor(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    GPUReport("Factor", detail::Abi<T>::geqrf(m, n, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}
// RNP/LA/QR.hpp:234-298
template <typename T> void MultQ_unblocked(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, T *work) {
    GPUReport("MultQ_unblocked", detail::Abi<T>::unm2r(side, trans, m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(c), ldc, detail::cp(work)));
}
// RNP/LA/QR.hpp:337-429
template <typename T> void MultQ(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    GPUReport("MultQ", detail::Abi<T>::unmqr(side, trans, m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(c), ldc, lwork, detail::cp(work)));
}
// RNP/LA/QR.hpp:451-485
template <class T> void GenerateQ_unblocked(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) {
    GPUReport("GenerateQ_unblocked", detail::Abi<T>::ung2r(m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(work)));
}
// RNP/LA/QR.hpp:509-570
template <class T> void GenerateQ(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    GPUReport("GenerateQ", detail::Abi<T>::ungqr(m, n, k, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}

} // namespace QR
} // namespace LA
} // namespace RNP

#endif // RNP_GPU_QR_HPP_INCLUDED
