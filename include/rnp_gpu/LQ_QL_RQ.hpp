// LQ_QL_RQ.hpp — RNP::LA::LQ, RNP::LA::QL and RNP::LA::RQ on the GB300, with
// the reference's template signatures for Factor, MultQ and GenerateQ
// (RNP/LA/LQ.hpp, QL.hpp, RQ.hpp).  Include this instead of the reference
// headers to run the same calls on the GPU:
//
//   RNP::LA::LQ::Factor(m, n, a, lda, tau, &lwork, work);
//   RNP::LA::QL::MultQ("L", "C", m, n, k, a, lda, tau, c, ldc, &lwork, work);
//   RNP::LA::RQ::GenerateQ(m, n, k, a, lda, tau, &lwork, work);
//
// Device pointers; the calls enqueue on the stream set with
// rnpgpu_set_stream() and return without synchronizing.  Like the reference
// they return void and print failed preconditions; the status of the last
// call is in RNP::LA::<LQ|QL|RQ>::GPUStatus().  The workspace query returns
// the GPU's length (it holds a transformed copy of the reflectors, see
// lqr_gb300.h).  The _unblocked forms are not provided on the GPU.
#ifndef RNP_GPU_LQ_QL_RQ_HPP_INCLUDED
#define RNP_GPU_LQ_QL_RQ_HPP_INCLUDED

#include <complex>
#include <cstddef>
#include <cstdio>

#include "lqr_gb300.h"

namespace RNP {
namespace LA {

namespace LQ {

inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
inline void GPUReport(const char *routine, int rc) {
    GPUStatus() = rc;
    if (rc != 0)
        std::fprintf(stderr, "RNP::LA::LQ::%s (GB300) failed: status %d %s\n", routine, rc, rc > 0 ? rnpgpu_get_last_error() : "(bad argument)");
}
namespace detail {
template <typename T> struct Abi;
template <> struct Abi<float> {
    typedef float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_sgelqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmlq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sunglq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<double> {
    typedef double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_dgelqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmlq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dunglq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<float>> {
    typedef rnpgpu_complex_float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_cgelqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmlq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cunglq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<double>> {
    typedef rnpgpu_complex_double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_zgelqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmlq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zunglq(m, n, k, a, lda, t, lw, w); }
};
template <typename T> inline typename Abi<T>::C *cp(T *p) { return reinterpret_cast<typename Abi<T>::C *>(p); }
template <typename T> inline const typename Abi<T>::C *cp(const T *p) { return reinterpret_cast<const typename Abi<T>::C *>(p); }
} // namespace detail

// RNP/LA/LQ.hpp:127-184
template <typename T> void Factor(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    GPUReport("Factor", detail::Abi<T>::f(m, n, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}
// RNP/LA/LQ.hpp:310-419
template <typename T> void MultQ(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    GPUReport("MultQ", detail::Abi<T>::mq(side, trans, m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(c), ldc, lwork, detail::cp(work)));
}
// RNP/LA/LQ.hpp:492-556
template <typename T> void GenerateQ(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    GPUReport("GenerateQ", detail::Abi<T>::g(m, n, k, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}

} // namespace LQ

namespace QL {

inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
inline void GPUReport(const char *routine, int rc) {
    GPUStatus() = rc;
    if (rc != 0)
        std::fprintf(stderr, "RNP::LA::QL::%s (GB300) failed: status %d %s\n", routine, rc, rc > 0 ? rnpgpu_get_last_error() : "(bad argument)");
}
namespace detail {
template <typename T> struct Abi;
template <> struct Abi<float> {
    typedef float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_sgeqlf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmql(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sungql(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<double> {
    typedef double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_dgeqlf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmql(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dungql(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<float>> {
    typedef rnpgpu_complex_float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_cgeqlf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmql(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cungql(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<double>> {
    typedef rnpgpu_complex_double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_zgeqlf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmql(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zungql(m, n, k, a, lda, t, lw, w); }
};
template <typename T> inline typename Abi<T>::C *cp(T *p) { return reinterpret_cast<typename Abi<T>::C *>(p); }
template <typename T> inline const typename Abi<T>::C *cp(const T *p) { return reinterpret_cast<const typename Abi<T>::C *>(p); }
} // namespace detail

// RNP/LA/QL.hpp:129-208
template <typename T> void Factor(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    GPUReport("Factor", detail::Abi<T>::f(m, n, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}
// RNP/LA/QL.hpp:337-437
template <typename T> void MultQ(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    GPUReport("MultQ", detail::Abi<T>::mq(side, trans, m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(c), ldc, lwork, detail::cp(work)));
}
// RNP/LA/QL.hpp:501-566
template <typename T> void GenerateQ(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    GPUReport("GenerateQ", detail::Abi<T>::g(m, n, k, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}

} // namespace QL

namespace RQ {

inline int &GPUStatus() {
    static thread_local int status = 0;
    return status;
}
inline void GPUReport(const char *routine, int rc) {
    GPUStatus() = rc;
    if (rc != 0)
        std::fprintf(stderr, "RNP::LA::RQ::%s (GB300) failed: status %d %s\n", routine, rc, rc > 0 ? rnpgpu_get_last_error() : "(bad argument)");
}
namespace detail {
template <typename T> struct Abi;
template <> struct Abi<float> {
    typedef float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_sgerqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_sunmrq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_sungrq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<double> {
    typedef double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_dgerqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_dunmrq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_dungrq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<float>> {
    typedef rnpgpu_complex_float C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_cgerqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_cunmrq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_cungrq(m, n, k, a, lda, t, lw, w); }
};
template <> struct Abi<std::complex<double>> {
    typedef rnpgpu_complex_double C;
    static int f(size_t m, size_t n, C *a, size_t lda, C *t, size_t *lw, C *w) { return rnpgpu_zgerqf(m, n, a, lda, t, lw, w); }
    static int mq(const char *s, const char *tr, size_t m, size_t n, size_t k, const C *a, size_t lda, const C *t, C *c, size_t ldc, size_t *lw, C *w) { return rnpgpu_zunmrq(s, tr, m, n, k, a, lda, t, c, ldc, lw, w); }
    static int g(size_t m, size_t n, size_t k, C *a, size_t lda, const C *t, size_t *lw, C *w) { return rnpgpu_zungrq(m, n, k, a, lda, t, lw, w); }
};
template <typename T> inline typename Abi<T>::C *cp(T *p) { return reinterpret_cast<typename Abi<T>::C *>(p); }
template <typename T> inline const typename Abi<T>::C *cp(const T *p) { return reinterpret_cast<const typename Abi<T>::C *>(p); }
} // namespace detail

// RNP/LA/RQ.hpp:131-210
template <typename T> void Factor(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    GPUReport("Factor", detail::Abi<T>::f(m, n, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}
// RNP/LA/RQ.hpp:344-449
template <typename T> void MultQ(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    GPUReport("MultQ", detail::Abi<T>::mq(side, trans, m, n, k, detail::cp(a), lda, detail::cp(tau), detail::cp(c), ldc, lwork, detail::cp(work)));
}
// RNP/LA/RQ.hpp:519-586
template <typename T> void GenerateQ(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    GPUReport("GenerateQ", detail::Abi<T>::g(m, n, k, detail::cp(a), lda, detail::cp(tau), lwork, detail::cp(work)));
}

} // namespace RQ

} // namespace LA
} // namespace RNP

#endif // RNP_GPU_LQ_QL_RQ_HPP_INCLUDED
