// qr_oracle.cpp — CPU ORACLE for the blocked Householder QR path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, the algorithm of
// RNP2's RNP::LA::QR path so that the GPU kernels can be checked against it.
// Only tests, the smoke check and the CPU-baseline leg of the benchmark may
// load it; the product library never links or calls it.
//
// Parity pin: the restatement is checked against golden vectors produced by
// the reference itself (tests/golden/, generated by tests/golden/make_golden.py
// from the reference headers compiled by oracle/Makefile into oracle/_ref/).
//
// Every routine cites the reference file:line it follows (paths relative to
// the RNP2 project root).  Level-2/3 BLAS calls of the reference are written
// here as plain loops with the same mathematical meaning (reference BLAS
// semantics); optionally (CPU baseline only) they are dispatched to an
// external Fortran BLAS loaded with dlopen, which is what the reference
// itself links against (tests/Makefile:3, src/BLAS_mix.cpp).
#include <complex>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <cstdint>
#include <limits>
#include <vector>
#include <utility>
#include <string>
#include <dlfcn.h>

namespace orc {

typedef std::complex<float> cf;
typedef std::complex<double> cd;

template <class T> struct Tr {
    typedef T R;
    static R re(const T &x) { return x; }
    static R im(const T &) { return R(0); }
    static T conj(const T &x) { return x; }
    static R absv(const T &x) { return std::fabs(x); }
};
template <class Rr> struct Tr<std::complex<Rr> > {
    typedef Rr R;
    static R re(const std::complex<Rr> &x) { return x.real(); }
    static R im(const std::complex<Rr> &x) { return x.imag(); }
    static std::complex<Rr> conj(const std::complex<Rr> &x) { return std::complex<Rr>(x.real(), -x.imag()); }
    static R absv(const std::complex<Rr> &x) { return std::abs(x); }
};

// ---------------------------------------------------------------------------
// Optional external BLAS (CPU baseline only).  Fortran ABI with 32-bit ints,
// as RNP/BLAS/FBLAS.hpp:8-14 declares it.
// ---------------------------------------------------------------------------
typedef int fint;
struct ExtBlas {
    void *h = nullptr;
    void (*dgemm)(const char *, const char *, const fint *, const fint *, const fint *, const double *, const double *, const fint *, const double *, const fint *, const double *, double *, const fint *, size_t, size_t) = nullptr;
    void (*zgemm)(const char *, const char *, const fint *, const fint *, const fint *, const cd *, const cd *, const fint *, const cd *, const fint *, const cd *, cd *, const fint *, size_t, size_t) = nullptr;
    void (*sgemm)(const char *, const char *, const fint *, const fint *, const fint *, const float *, const float *, const fint *, const float *, const fint *, const float *, float *, const fint *, size_t, size_t) = nullptr;
    void (*cgemm)(const char *, const char *, const fint *, const fint *, const fint *, const cf *, const cf *, const fint *, const cf *, const fint *, const cf *, cf *, const fint *, size_t, size_t) = nullptr;
    void (*dtrmm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const double *, const double *, const fint *, double *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*ztrmm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const cd *, const cd *, const fint *, cd *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*strmm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const float *, const float *, const fint *, float *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*ctrmm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const cf *, const cf *, const fint *, cf *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*dtrsm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const double *, const double *, const fint *, double *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*ztrsm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const cd *, const cd *, const fint *, cd *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*dgemv)(const char *, const fint *, const fint *, const double *, const double *, const fint *, const double *, const fint *, const double *, double *, const fint *, size_t) = nullptr;
    void (*zgemv)(const char *, const fint *, const fint *, const cd *, const cd *, const fint *, const cd *, const fint *, const cd *, cd *, const fint *, size_t) = nullptr;
    void (*sgemv)(const char *, const fint *, const fint *, const float *, const float *, const fint *, const float *, const fint *, const float *, float *, const fint *, size_t) = nullptr;
    void (*cgemv)(const char *, const fint *, const fint *, const cf *, const cf *, const fint *, const cf *, const fint *, const cf *, cf *, const fint *, size_t) = nullptr;
    void (*dger)(const fint *, const fint *, const double *, const double *, const fint *, const double *, const fint *, double *, const fint *) = nullptr;
    void (*zgerc)(const fint *, const fint *, const cd *, const cd *, const fint *, const cd *, const fint *, cd *, const fint *) = nullptr;
    void (*sger)(const fint *, const fint *, const float *, const float *, const fint *, const float *, const fint *, float *, const fint *) = nullptr;
    void (*cgerc)(const fint *, const fint *, const cf *, const cf *, const fint *, const cf *, const fint *, cf *, const fint *) = nullptr;
    void (*dtrmv)(const char *, const char *, const char *, const fint *, const double *, const fint *, double *, const fint *, size_t, size_t, size_t) = nullptr;
    void (*ztrmv)(const char *, const char *, const char *, const fint *, const cd *, const fint *, cd *, const fint *, size_t, size_t, size_t) = nullptr;
    void (*strmv)(const char *, const char *, const char *, const fint *, const float *, const fint *, float *, const fint *, size_t, size_t, size_t) = nullptr;
    void (*ctrmv)(const char *, const char *, const char *, const fint *, const cf *, const fint *, cf *, const fint *, size_t, size_t, size_t) = nullptr;
    void (*strsm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const float *, const float *, const fint *, float *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*ctrsm)(const char *, const char *, const char *, const char *, const fint *, const fint *, const cf *, const cf *, const fint *, cf *, const fint *, size_t, size_t, size_t, size_t) = nullptr;
    void (*set_threads)(int) = nullptr;
};
static ExtBlas g_ext;
static bool g_use_ext = false;

template <class T> inline bool ext_gemm(const char *ta, const char *tb, size_t m, size_t n, size_t k, T alpha, const T *a, size_t lda, const T *b, size_t ldb, T beta, T *c, size_t ldc);
template <class T> inline bool ext_trmm(const char *side, const char *uplo, const char *ta, const char *diag, size_t m, size_t n, T alpha, const T *a, size_t lda, T *b, size_t ldb);
template <class T> inline bool ext_trsm(const char *side, const char *uplo, const char *ta, const char *diag, size_t m, size_t n, T alpha, const T *a, size_t lda, T *b, size_t ldb);

#define ORC_EXT_GEMM(T, fn)                                                                           \
    template <> inline bool ext_gemm<T>(const char *ta, const char *tb, size_t m, size_t n, size_t k, T alpha, \
                                        const T *a, size_t lda, const T *b, size_t ldb, T beta, T *c, size_t ldc) { \
        if (!g_use_ext || !g_ext.fn) return false;                                                     \
        fint M = (fint)m, N = (fint)n, K = (fint)k, LA = (fint)(lda ? lda : 1), LB = (fint)(ldb ? ldb : 1), LC = (fint)(ldc ? ldc : 1); \
        g_ext.fn(ta, tb, &M, &N, &K, &alpha, a, &LA, b, &LB, &beta, c, &LC, 1, 1);                   \
        return true;                                                                                   \
    }
ORC_EXT_GEMM(double, dgemm)
ORC_EXT_GEMM(cd, zgemm)
ORC_EXT_GEMM(float, sgemm)
ORC_EXT_GEMM(cf, cgemm)
#define ORC_EXT_TR(T, name, fn)                                                                        \
    template <> inline bool name<T>(const char *side, const char *uplo, const char *ta, const char *diag, size_t m, size_t n, \
                                    T alpha, const T *a, size_t lda, T *b, size_t ldb) {               \
        if (!g_use_ext || !g_ext.fn) return false;                                                     \
        fint M = (fint)m, N = (fint)n, LA = (fint)(lda ? lda : 1), LB = (fint)(ldb ? ldb : 1);         \
        g_ext.fn(side, uplo, ta, diag, &M, &N, &alpha, a, &LA, b, &LB, 1, 1, 1, 1);                    \
        return true;                                                                                   \
    }
ORC_EXT_TR(double, ext_trmm, dtrmm)
ORC_EXT_TR(cd, ext_trmm, ztrmm)
ORC_EXT_TR(float, ext_trmm, strmm)
ORC_EXT_TR(cf, ext_trmm, ctrmm)
ORC_EXT_TR(double, ext_trsm, dtrsm)
ORC_EXT_TR(cd, ext_trsm, ztrsm)
ORC_EXT_TR(float, ext_trsm, strsm)
ORC_EXT_TR(cf, ext_trsm, ctrsm)

// level 2: gemv, ger/gerc, trmv (src/BLAS_mix.cpp:112,122,248,256,374,384
// forward the same calls of the reference to the Fortran BLAS)
#define ORC_EXT_GEMV(T, fn)                                                                            \
    inline bool ext_gemv(char trans, size_t m, size_t n, T alpha, const T *a, size_t lda, const T *x, size_t incx, T beta, T *y, size_t incy) { \
        if (!g_use_ext || !g_ext.fn || m == 0 || n == 0) return false;                                 \
        const char t[2] = {trans, 0};                                                                  \
        fint M = (fint)m, N = (fint)n, LA = (fint)(lda ? lda : 1), IX = (fint)incx, IY = (fint)incy;   \
        g_ext.fn(t, &M, &N, &alpha, a, &LA, x, &IX, &beta, y, &IY, 1);                                  \
        return true;                                                                                   \
    }
ORC_EXT_GEMV(double, dgemv)
ORC_EXT_GEMV(cd, zgemv)
ORC_EXT_GEMV(float, sgemv)
ORC_EXT_GEMV(cf, cgemv)
#define ORC_EXT_GER(T, fn)                                                                             \
    inline bool ext_gerc(size_t m, size_t n, T alpha, const T *x, size_t incx, const T *y, size_t incy, T *a, size_t lda) { \
        if (!g_use_ext || !g_ext.fn || m == 0 || n == 0) return false;                                 \
        fint M = (fint)m, N = (fint)n, LA = (fint)(lda ? lda : 1), IX = (fint)incx, IY = (fint)incy;   \
        g_ext.fn(&M, &N, &alpha, x, &IX, y, &IY, a, &LA);                                              \
        return true;                                                                                   \
    }
ORC_EXT_GER(double, dger)
ORC_EXT_GER(cd, zgerc)
ORC_EXT_GER(float, sger)
ORC_EXT_GER(cf, cgerc)
#define ORC_EXT_TRMV(T, fn)                                                                            \
    inline bool ext_trmv_upper(char trans, size_t n, const T *a, size_t lda, T *x) {                   \
        if (!g_use_ext || !g_ext.fn || n == 0) return false;                                           \
        const char t[2] = {trans, 0};                                                                  \
        fint N = (fint)n, LA = (fint)(lda ? lda : 1), IX = 1;                                          \
        g_ext.fn("U", t, "N", &N, a, &LA, x, &IX, 1, 1, 1);                                            \
        return true;                                                                                   \
    }
ORC_EXT_TRMV(double, dtrmv)
ORC_EXT_TRMV(cd, ztrmv)
ORC_EXT_TRMV(float, strmv)
ORC_EXT_TRMV(cf, ctrmv)

// ---------------------------------------------------------------------------
// Level-1/2/3 helpers with reference-BLAS meaning (plain loops).
// ---------------------------------------------------------------------------

// Scaled sum-of-squares 2-norm.  RNP/BLAS/BLAS_mix.hpp:725-760: real and
// imaginary parts are folded in separately, in element order.
template <class T> typename Tr<T>::R norm2(size_t n, const T *x, size_t incx) {
    typedef typename Tr<T>::R R;
    R ssq(1), scale(0);
    for (size_t i = 0; i < n; ++i, x += incx) {
        R parts[2] = {Tr<T>::re(*x), Tr<T>::im(*x)};
        for (int p = 0; p < 2; ++p) {
            if (parts[p] != R(0)) {
                R temp = std::fabs(parts[p]);
                if (scale < temp) {
                    R r = scale / temp;
                    ssq = ssq * r * r + R(1);
                    scale = temp;
                } else {
                    R r = temp / scale;
                    ssq += r * r;
                }
            }
        }
    }
    return scale * std::sqrt(ssq);
}

// RNP/Types.hpp:73-92.
template <class R> R hypot3(R x, R y, R z) {
    R xa = std::fabs(x), ya = std::fabs(y), za = std::fabs(z);
    R w = xa;
    if (ya > w) w = ya;
    if (za > w) w = za;
    if (w == R(0)) return xa + ya + za;
    xa /= w; ya /= w; za /= w;
    return w * std::sqrt(xa * xa + ya * ya + za * za);
}

template <class T> void scal(size_t n, T a, T *x, size_t incx) {
    for (size_t i = 0; i < n; ++i) x[i * incx] *= a;
}

// y := alpha*op(A)*x + beta*y   (gemv)
template <class T> void gemv(char trans, size_t m, size_t n, T alpha, const T *a, size_t lda, const T *x, size_t incx, T beta, T *y, size_t incy) {
    if (ext_gemv(trans, m, n, alpha, a, lda, x, incx, beta, y, incy)) return;
    if (trans == 'N') {
        for (size_t i = 0; i < m; ++i) y[i * incy] = (beta == T(0)) ? T(0) : beta * y[i * incy];
        for (size_t j = 0; j < n; ++j) {
            T t = alpha * x[j * incx];
            for (size_t i = 0; i < m; ++i) y[i * incy] += t * a[i + j * lda];
        }
    } else {
        const bool cj = (trans == 'C');
        for (size_t j = 0; j < n; ++j) {
            T s(0);
            for (size_t i = 0; i < m; ++i) s += (cj ? Tr<T>::conj(a[i + j * lda]) : a[i + j * lda]) * x[i * incx];
            y[j * incy] = (beta == T(0)) ? alpha * s : alpha * s + beta * y[j * incy];
        }
    }
}

// A := A + alpha*x*y^H   (ger / gerc; RNP "ConjugateRank1Update")
template <class T> void gerc(size_t m, size_t n, T alpha, const T *x, size_t incx, const T *y, size_t incy, T *a, size_t lda) {
    if (ext_gerc(m, n, alpha, x, incx, y, incy, a, lda)) return;
    for (size_t j = 0; j < n; ++j) {
        T t = alpha * Tr<T>::conj(y[j * incy]);
        if (t == T(0)) continue;
        for (size_t i = 0; i < m; ++i) a[i + j * lda] += x[i * incx] * t;
    }
}

// x := op(A)*x, A upper triangular, non-unit  (trmv "U", trans, "N")
template <class T> void trmv_upper(char trans, size_t n, const T *a, size_t lda, T *x) {
    if (ext_trmv_upper(trans, n, a, lda, x)) return;
    if (trans == 'N') {
        for (size_t j = 0; j < n; ++j) {
            T t = x[j];
            for (size_t i = 0; i < j; ++i) x[i] += t * a[i + j * lda];
            x[j] *= a[j + j * lda];
        }
    } else {
        const bool cj = (trans == 'C');
        for (size_t jj = n; jj-- > 0;) {
            T s = x[jj] * (cj ? Tr<T>::conj(a[jj + jj * lda]) : a[jj + jj * lda]);
            for (size_t i = 0; i < jj; ++i) s += (cj ? Tr<T>::conj(a[i + jj * lda]) : a[i + jj * lda]) * x[i];
            x[jj] = s;
        }
    }
}

template <class T> inline T opel(char t, const T *a, size_t lda, size_t i, size_t j) {
    // element (i,j) of op(A)
    if (t == 'N') return a[i + j * lda];
    if (t == 'T') return a[j + i * lda];
    return Tr<T>::conj(a[j + i * lda]);
}

// C := alpha*op(A)*op(B) + beta*C   (gemm)
template <class T> void gemm(char ta, char tb, size_t m, size_t n, size_t k, T alpha, const T *a, size_t lda, const T *b, size_t ldb, T beta, T *c, size_t ldc) {
    if (m == 0 || n == 0) return;
    const char sa[2] = {ta, 0}, sb[2] = {tb, 0};
    if (k > 0 && ext_gemm<T>(sa, sb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc)) return;
    std::vector<T> col(m);
    for (size_t j = 0; j < n; ++j) {
        for (size_t i = 0; i < m; ++i) col[i] = T(0);
        for (size_t l = 0; l < k; ++l) {
            T bl = opel(tb, b, ldb, l, j);
            if (bl == T(0)) continue;
            if (ta == 'N') {
                const T *ac = a + l * lda;
                for (size_t i = 0; i < m; ++i) col[i] += ac[i] * bl;
            } else {
                for (size_t i = 0; i < m; ++i) col[i] += opel(ta, a, lda, i, l) * bl;
            }
        }
        for (size_t i = 0; i < m; ++i)
            c[i + j * ldc] = (beta == T(0)) ? alpha * col[i] : alpha * col[i] + beta * c[i + j * ldc];
    }
}

// B := B*op(A), A k-by-k triangular, right side (trmm "R", uplo, trans, diag)
template <class T> void trmm_right(char uplo, char ta, char diag, size_t m, size_t k, const T *a, size_t lda, T *b, size_t ldb) {
    if (m == 0 || k == 0) return;
    const char s1[2] = {'R', 0}, s2[2] = {uplo, 0}, s3[2] = {ta, 0}, s4[2] = {diag, 0};
    if (ext_trmm<T>(s1, s2, s3, s4, m, k, T(1), a, lda, b, ldb)) return;
    // element (l,j) of op(A) with its triangular structure
    auto el = [&](size_t l, size_t j) -> T {
        // storage index of op(A)(l,j)
        size_t r = (ta == 'N') ? l : j, c = (ta == 'N') ? j : l;
        bool lowerstored = (uplo == 'L');
        if (lowerstored ? (r < c) : (r > c)) return T(0);
        if (r == c && diag == 'U') return T(1);
        T v = a[r + c * lda];
        return (ta == 'C') ? Tr<T>::conj(v) : v;
    };
    std::vector<T> row(k);
    for (size_t i = 0; i < m; ++i) {
        for (size_t j = 0; j < k; ++j) {
            T s(0);
            for (size_t l = 0; l < k; ++l) s += b[i + l * ldb] * el(l, j);
            row[j] = s;
        }
        for (size_t j = 0; j < k; ++j) b[i + j * ldb] = row[j];
    }
}

// Solve op(A)*X = alpha*B, A upper triangular non-unit, left side
// (trsm "L","U","N","N"; RNP/BLAS/BLAS_mix.hpp:2096-2113 -> dtrsm_).
template <class T> void trsm_luN(size_t n, size_t nrhs, const T *a, size_t lda, T *b, size_t ldb) {
    if (ext_trsm<T>("L", "U", "N", "N", n, nrhs, T(1), a, lda, b, ldb)) return;
    for (size_t j = 0; j < nrhs; ++j) {
        T *x = b + j * ldb;
        for (size_t kk = n; kk-- > 0;) {
            if (x[kk] != T(0)) {
                x[kk] /= a[kk + kk * lda];
                T t = x[kk];
                for (size_t i = 0; i < kk; ++i) x[i] -= t * a[i + kk * lda];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Reflector primitives (RNP/LA/Reflector.hpp)
// ---------------------------------------------------------------------------

// ila_lc: RNP/LA/Reflector.hpp:36-48
template <class T> size_t last_nonzero_col(size_t m, size_t n, const T *a, size_t lda) {
    if (n == 0 || a[0 + (n - 1) * lda] != T(0) || a[m - 1 + (n - 1) * lda] != T(0)) return n;
    size_t j = n;
    while (j-- > 0) {
        for (size_t i = 0; i < m; ++i)
            if (a[i + j * lda] != T(0)) return j + 1;
    }
    return j + 1;
}
// ila_lr: RNP/LA/Reflector.hpp:63-75
template <class T> size_t last_nonzero_row(size_t m, size_t n, const T *a, size_t lda) {
    if (m == 0 || a[m - 1 + 0 * lda] != T(0) || a[m - 1 + (n - 1) * lda] != T(0)) return m;
    size_t i = m;
    while (i-- > 0) {
        for (size_t j = 0; j < n; ++j)
            if (a[i + j * lda] != T(0)) return i + 1;
    }
    return i + 1;
}

// larfg: RNP/LA/Reflector.hpp:117-158
template <class T> void generate(size_t n, T *alpha, T *x, size_t incx, T *tau) {
    typedef typename Tr<T>::R R;
    if (n == 0) { *tau = T(0); return; }
    R xnorm = norm2(n - 1, x, incx);
    if (xnorm == R(0) && Tr<T>::im(*alpha) == R(0)) {
        *tau = T(0);
        return;
    }
    R beta = hypot3(Tr<T>::re(*alpha), Tr<T>::im(*alpha), xnorm);
    if (Tr<T>::re(*alpha) > R(0)) beta = -beta;
    const R safmin = std::numeric_limits<R>::min() / (2 * std::numeric_limits<R>::epsilon());
    const R rsafmn = R(1) / safmin;
    size_t knt = 0;
    if (std::fabs(beta) < safmin) {
        do {
            ++knt;
            scal(n - 1, T(rsafmn), x, incx);
            beta *= rsafmn;
            *alpha *= rsafmn;
        } while (std::fabs(beta) < safmin);
        xnorm = norm2(n - 1, x, incx);
        beta = hypot3(Tr<T>::re(*alpha), Tr<T>::im(*alpha), xnorm);
        if (Tr<T>::re(*alpha) > R(0)) beta = -beta;
    }
    *tau = (beta - *alpha) / beta;
    *alpha = R(1) / (*alpha - beta);
    scal(n - 1, *alpha, x, incx);
    while (knt-- > 0) beta *= safmin;
    *alpha = beta;
}

// larf with vconj = false: RNP/LA/Reflector.hpp:191-300 (vone = 0 and 1)
template <class T> void apply(char side, int vone, size_t m, size_t n, const T *v, size_t incv, T tau, T *c, size_t ldc, T *work) {
    size_t lenv = 0, lenc = 0;
    if (tau != T(0)) {
        lenv = (side == 'L') ? m : n;
        if (lenv == 0) return;
        size_t i = (lenv - 1) * incv;
        while (lenv > 0 && v[i] == T(0)) { --lenv; i -= incv; }
        if (side == 'L') lenc = last_nonzero_col(lenv, n, c, ldc);
        else lenc = last_nonzero_row(m, lenv, c, ldc);
        if (lenc == 0) return;
    }
    const T one(1);
    if (vone == 0) {
        if (side == 'L') {
            gemv('C', lenv, lenc, T(1), c, ldc, v, incv, T(0), work, 1);
            gerc(lenv, lenc, -tau, v, incv, work, 1, c, ldc);
        } else {
            gemv('N', lenc, lenv, T(1), c, ldc, v, incv, T(0), work, 1);
            gerc(lenc, lenv, -tau, work, 1, v, incv, c, ldc);
        }
    } else {
        if (side == 'L') {
            for (size_t j = 0; j < lenc; ++j) work[j] = Tr<T>::conj(c[0 + j * ldc]);
            if (lenv > 1) gemv('C', lenv - 1, lenc, T(1), c + 1, ldc, v + incv, incv, T(1), work, 1);
            gerc(1, lenc, -tau, &one, incv, work, 1, c, ldc);
            if (lenv > 1) gerc(lenv - 1, lenc, -tau, v + incv, incv, work, 1, c + 1, ldc);
        } else {
            for (size_t i = 0; i < lenc; ++i) work[i] = c[i];
            if (lenv > 1) gemv('N', lenc, lenv - 1, T(1), c + ldc, ldc, v + incv, incv, T(1), work, 1);
            for (size_t i = 0; i < lenc; ++i) c[i] += -tau * work[i];
            if (lenv > 1) gerc(lenc, lenv - 1, -tau, work, 1, v + incv, incv, c + ldc, ldc);
        }
    }
}

// larft, dir = "F", storev = "C": RNP/LA/Reflector.hpp:580-626
template <class T> void block_tr(size_t n, size_t k, const T *v, size_t ldv, const T *tau, T *t, size_t ldt) {
    if (n == 0) return;
    size_t prevlastv = n - 1;
    for (size_t i = 0; i < k; ++i) {
        if (i > prevlastv) prevlastv = i;
        if (tau[i] == T(0)) {
            for (size_t j = 0; j <= i; ++j) t[j + i * ldt] = T(0);
        } else {
            size_t lastv;
            for (lastv = n - 1; lastv > i; --lastv)
                if (v[lastv + i * ldv] != T(0)) break;
            for (size_t j = 0; j < i; ++j) t[j + i * ldt] = -tau[i] * Tr<T>::conj(v[i + j * ldv]);
            size_t jlim = (lastv < prevlastv ? lastv : prevlastv);
            gemv('C', jlim - i, i, -tau[i], v + i + 1, ldv, v + i + 1 + i * ldv, 1, T(1), t + i * ldt, 1);
            trmv_upper('N', i, t, ldt, t + i * ldt);
            t[i + i * ldt] = tau[i];
            if (i > 0) { if (lastv > prevlastv) prevlastv = lastv; }
            else prevlastv = lastv;
        }
    }
}

// larfb, dir = "F", storev = "C": RNP/LA/Reflector.hpp:725-815
template <class T> void apply_block(char side, char trans, size_t m, size_t n, size_t k, const T *v, size_t ldv, const T *t, size_t ldt, T *c, size_t ldc, T *work, size_t ldwork) {
    if (m == 0 || n == 0) return;
    const char transt = (trans == 'N') ? 'C' : 'N';
    if (side == 'L') {
        size_t lastv = last_nonzero_row(m, k, v, ldv);
        if (k > lastv) lastv = k;
        const size_t lastc = last_nonzero_col(lastv, n, c, ldc);
        for (size_t j = 0; j < k; ++j)
            for (size_t i = 0; i < lastc; ++i) work[i + j * ldwork] = Tr<T>::conj(c[j + i * ldc]);
        trmm_right('L', 'N', 'U', lastc, k, v, ldv, work, ldwork);
        if (lastv > k) gemm('C', 'N', lastc, k, lastv - k, T(1), c + k, ldc, v + k, ldv, T(1), work, ldwork);
        trmm_right('U', transt, 'N', lastc, k, t, ldt, work, ldwork);
        if (m > k) gemm('N', 'C', lastv - k, lastc, k, T(-1), v + k, ldv, work, ldwork, T(1), c + k, ldc);
        trmm_right('L', 'C', 'U', lastc, k, v, ldv, work, ldwork);
        for (size_t j = 0; j < k; ++j)
            for (size_t i = 0; i < lastc; ++i) c[j + i * ldc] -= Tr<T>::conj(work[i + j * ldwork]);
    } else {
        size_t lastv = last_nonzero_row(n, k, v, ldv);
        if (k > lastv) lastv = k;
        const size_t lastc = last_nonzero_row(m, lastv, c, ldc);
        for (size_t j = 0; j < k; ++j)
            for (size_t i = 0; i < lastc; ++i) work[i + j * ldwork] = c[i + j * ldc];
        trmm_right('L', 'N', 'U', lastc, k, v, ldv, work, ldwork);
        if (lastv > k) gemm('N', 'N', lastc, k, lastv - k, T(1), c + k * ldc, ldc, v + k, ldv, T(1), work, ldwork);
        trmm_right('U', trans, 'N', lastc, k, t, ldt, work, ldwork);
        if (lastv > k) gemm('N', 'C', lastc, lastv - k, k, T(-1), work, ldwork, v + k, ldv, T(1), c + k * ldc, ldc);
        trmm_right('L', 'C', 'U', lastc, k, v, ldv, work, ldwork);
        for (size_t j = 0; j < k; ++j)
            for (size_t i = 0; i < lastc; ++i) c[i + j * ldc] -= work[i + j * ldwork];
    }
}

// ---------------------------------------------------------------------------
// QR (RNP/LA/QR.hpp) with the reference's default Tuning (QR.hpp:41-51)
// ---------------------------------------------------------------------------
static const size_t kNb = 32, kNbMin = 2, kNx = 128;

// geqr2: RNP/LA/QR.hpp:78-102
template <class T> void factor_unblocked(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) {
    size_t k = m < n ? m : n;
    for (size_t i = 0; i < k; ++i) {
        size_t row = m - 1;
        if (i + 1 < row) row = i + 1;
        generate(m - i, &a[i + i * lda], &a[row + i * lda], 1, &tau[i]);
        if (i < n - 1) {
            T alpha = a[i + i * lda];
            a[i + i * lda] = T(1);
            apply('L', 0, m - i, n - i - 1, &a[i + i * lda], 1, Tr<T>::conj(tau[i]), &a[i + (i + 1) * lda], lda, work);
            a[i + i * lda] = alpha;
        }
    }
}

// geqrf: RNP/LA/QR.hpp:129-197
template <class T> void factor(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    const size_t k = m < n ? m : n;
    if (k == 0) return;
    size_t nb = kNb;
    if (work == nullptr || *lwork == 0) { *lwork = nb * n; return; }
    size_t nbmin = 2, nx = 0, ldwork = n;
    if (nb > 1 && nb < k) {
        nx = kNx;
        if (nx < k) {
            size_t iws = ldwork * nb;
            if (*lwork < iws) { nb = *lwork / ldwork; nbmin = kNbMin; }
        }
    }
    size_t i;
    if (nb >= nbmin && nb < k && nx < k) {
        for (i = 0; i + nx < k; i += nb) {
            const size_t ib = (k - i < nb ? k - i : nb);
            factor_unblocked(m - i, ib, &a[i + i * lda], lda, &tau[i], work);
            if (i + ib < n) {
                block_tr(m - i, ib, &a[i + i * lda], lda, &tau[i], work, ldwork);
                apply_block('L', 'C', m - i, n - i - ib, ib, &a[i + i * lda], lda, work, ldwork, &a[i + (i + ib) * lda], lda, &work[ib], ldwork);
            }
        }
    } else {
        i = 0;
    }
    if (i < k) factor_unblocked(m - i, n - i, &a[i + i * lda], lda, &tau[i], work);
}

// orm2r/unm2r: RNP/LA/QR.hpp:234-298
template <class T> void multq_unblocked(char side, char trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, T *work) {
    const bool left = side == 'L', notran = trans == 'N';
    if (m < 1 || n < 1 || k < 1) return;
    size_t mi = m, ni = n, ic = 0, jc = 0;
    auto step = [&](size_t i) {
        if (left) { mi = m - i; ic = i; } else { ni = n - i; jc = i; }
        T taui = notran ? tau[i] : Tr<T>::conj(tau[i]);
        apply(side, 1, mi, ni, &a[i + i * lda], 1, taui, &c[ic + jc * ldc], ldc, work);
    };
    if ((left && !notran) || (!left && notran)) {
        for (size_t i = 0; i < k; ++i) step(i);
    } else {
        size_t i = k;
        while (i-- > 0) step(i);
    }
}

// ormqr/unmqr: RNP/LA/QR.hpp:337-429
template <class T> void multq(char side, char trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    if (m == 0 || n == 0 || k == 0) return;
    const bool left = side == 'L', notran = trans == 'N';
    const size_t nq = left ? m : n, nw = left ? n : m;
    size_t nb = kNb;
    if (*lwork == 0 || work == nullptr) { *lwork = nb * nw + nb * nb; return; }
    size_t nbmin = 2, ldwork = nw;
    T *t = nullptr;
    size_t ldt = nb;
    if (nb > 1 && nb < k) {
        size_t iws = nw * nb + nb * nb;
        t = work + nb * ldwork;
        if (*lwork < iws) {
            nb = *lwork / (2 * ldwork);
            t = work + nb * ldwork;
            ldt = nb;
            nbmin = kNbMin;
        }
    }
    if (nb < nbmin || nb >= k) {
        multq_unblocked(side, trans, m, n, k, a, lda, tau, c, ldc, work);
        return;
    }
    size_t ni = n, mi = m, ic = 0, jc = 0;
    auto blk = [&](size_t i) {
        size_t ib = (k < nb + i ? k - i : nb);
        block_tr(nq - i, ib, &a[i + i * lda], lda, &tau[i], t, ldt);
        if (left) { mi = m - i; ic = i; } else { ni = n - i; jc = i; }
        apply_block(side, trans, mi, ni, ib, &a[i + i * lda], lda, t, ldt, &c[ic + jc * ldc], ldc, work, ldwork);
    };
    if ((left && !notran) || (!left && notran)) {
        for (size_t i = 0; i < k; i += nb) blk(i);
    } else {
        size_t i = ((k - 1) / nb) * nb + nb;
        do { i -= nb; blk(i); } while (i > 0);
    }
}

// org2r/ung2r: RNP/LA/QR.hpp:451-485
template <class T> void genq_unblocked(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) {
    if (n < 1) return;
    for (size_t j = k; j < n; ++j) {
        for (size_t i = 0; i < m; ++i) a[i + j * lda] = T(0);
        a[j + j * lda] = T(1);
    }
    size_t i = k;
    while (i-- > 0) {
        if (i + 1 < n) {
            a[i + i * lda] = T(1);
            apply('L', 0, m - i, n - i - 1, &a[i + i * lda], 1, tau[i], &a[i + (i + 1) * lda], lda, work);
        }
        if (i + 1 < m) scal(m - i - 1, -tau[i], &a[i + 1 + i * lda], 1);
        a[i + i * lda] = T(1) - tau[i];
        for (size_t l = 0; l < i; ++l) a[l + i * lda] = T(0);
    }
}

// orgqr/ungqr: RNP/LA/QR.hpp:509-570
template <class T> void genq(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    if (n == 0) return;
    size_t nb = kNb;
    if (*lwork == 0 || work == nullptr) { *lwork = n * nb; return; }
    size_t nbmin = 2, nx = 0, ldwork = n;
    if (nb > 1 && nb < k) {
        nx = kNx;
        if (nx < k) {
            size_t iws = ldwork * nb;
            if (*lwork < iws) { nb = *lwork / ldwork; nbmin = kNbMin; }
        }
    }
    size_t ki = 0, kk = 0;
    if (nb >= nbmin && nb < k && nx < k) {
        ki = ((k - nx - 1) / nb) * nb;
        kk = (k < ki + nb ? k : ki + nb);
        for (size_t j = kk; j < n; ++j)
            for (size_t i = 0; i < kk; ++i) a[i + j * lda] = T(0);
    }
    if (kk < n) genq_unblocked(m - kk, n - kk, k - kk, &a[kk + kk * lda], lda, &tau[kk], work);
    if (kk > 0) {
        size_t i = ki + nb;
        do {
            i -= nb;
            const size_t ib = (nb + i < k ? nb : k - i);
            if (i + ib < n) {
                block_tr(m - i, ib, &a[i + i * lda], lda, &tau[i], work, ldwork);
                apply_block('L', 'N', m - i, n - i - ib, ib, &a[i + i * lda], lda, work, ldwork, &a[i + (i + ib) * lda], lda, &work[ib], ldwork);
            }
            genq_unblocked(m - i, ib, ib, &a[i + i * lda], lda, &tau[i], work);
            for (size_t j = i; j < i + ib; ++j)
                for (size_t l = 0; l < i; ++l) a[l + j * lda] = T(0);
        } while (i > 0);
    }
}

// Least squares by QR, composed the way a caller of the reference does it:
// Factor, MultQ("L","C") on B, then the upper-triangular solve
// (BLAS::SolveTrM "L","U","N","N", RNP/BLAS/BLAS_mix.hpp:2096-2113).
template <class T> void gels(size_t m, size_t n, size_t nrhs, T *a, size_t lda, T *tau, T *b, size_t ldb) {
    size_t lw = 0;
    factor(m, n, a, lda, tau, &lw, (T *)nullptr);
    size_t lw2 = 0;
    multq('L', 'C', m, nrhs, n, a, lda, tau, b, ldb, &lw2, (T *)nullptr);
    if (lw2 > lw) lw = lw2;
    std::vector<T> work(lw > 0 ? lw : 1);
    factor(m, n, a, lda, tau, &lw, work.data());
    multq('L', 'C', m, nrhs, n, a, lda, tau, b, ldb, &lw, work.data());
    trsm_luN(n, nrhs, a, lda, b, ldb);
}

// ---------------------------------------------------------------------------
// Seeded inputs: RNP/Random.hpp:45-183 (laruv-style 48-bit multiplicative
// congruential generator, multiplier 33952834046453, modulus 2^48) and
// GenerateVector (Random.hpp:262-320).  The reference walks the sequence
// seed*a^1, seed*a^2, ... in chunks of 128 using a table of powers of a;
// the same sequence is produced here by stepping the 48-bit state directly.
// ---------------------------------------------------------------------------
static const uint64_t kMcgA = 33952834046453ULL;
static const uint64_t kMask48 = (1ULL << 48) - 1;

static uint64_t seed_to_state(const int iseed[4]) {
    uint64_t s = ((uint64_t)(iseed[0] & 4095) << 36) | ((uint64_t)(iseed[1] & 4095) << 24) | ((uint64_t)(iseed[2] & 4095) << 12) | (uint64_t)((iseed[3] | 1) & 4095);
    return s;
}
static void state_to_seed(uint64_t s, int iseed[4]) {
    iseed[0] = (int)((s >> 36) & 4095);
    iseed[1] = (int)((s >> 24) & 4095);
    iseed[2] = (int)((s >> 12) & 4095);
    iseed[3] = (int)(s & 4095);
}
template <class R> static void uniform01(size_t n, R *x, int iseed[4]) {
    if (n == 0) return;
    uint64_t s = seed_to_state(iseed);
    for (size_t j = 0; j < n; ++j) {
        s = (s * kMcgA) & kMask48;
        R it1 = (R)(double)((s >> 36) & 4095), it2 = (R)(double)((s >> 24) & 4095), it3 = (R)(double)((s >> 12) & 4095), it4 = (R)(double)(s & 4095);
        R v = (it1 + (it2 + (it3 + it4 * (R(1) / R(4096))) * (R(1) / R(4096))) * (R(1) / R(4096))) * (R(1) / R(4096));
        x[j] = R(1) - v;
    }
    state_to_seed(s, iseed);
}

// dist: 0 = Uniform01, 1 = Uniform_11, 2 = Normal01 (RNP/Random.hpp:262-289)
template <class R> static void larnv_real(int dist, size_t n, R *x, int iseed[4]) {
    if (dist == 0) { uniform01(n, x, iseed); return; }
    if (dist == 3 || dist == 4) {
        // UnitDisc / UnitCircle for real numbers (RNP/Random.hpp:291-315):
        // a whole chunk of 128 uniforms per 64 outputs, from the even ones
        R pool[128];
        for (size_t i0 = 0; i0 < n; i0 += 64) {
            size_t ilim = 64;
            if (n < i0 + ilim) ilim = n - i0;
            uniform01(128, pool, iseed);
            for (size_t i = 0; i < ilim; ++i) x[i0 + i] = dist == 3 ? R(2) * pool[2 * i] - R(1) : ((R(2) * pool[2 * i] < R(1)) ? R(-1) : R(1));
        }
        return;
    }
    if (dist == 1) {
        uniform01(n, x, iseed);
        for (size_t i = 0; i < n; ++i) x[i] = R(2) * x[i] - R(1);
        return;
    }
    R pool[128];
    for (size_t i0 = 0; i0 < n; i0 += 64) {
        size_t ilim = 64;
        if (n < i0 + ilim) ilim = n - i0;
        uniform01(2 * ilim, pool, iseed);
        for (size_t i = 0; i < ilim; ++i) {
            // The reference's unqualified log1p/sqrt/cos resolve to the C
            // double-precision functions, so the float case is evaluated in
            // double and rounded once on assignment.
            R ang = R(6.28318530717958647692528676656) * pool[2 * i + 1];
            x[i0 + i] = (R)(::sqrt((double)R(-2) * ::log1p(-(double)pool[2 * i])) * ::cos((double)ang));
        }
    }
}
template <class R> static void larnv_cplx(int dist, size_t n, std::complex<R> *x, int iseed[4]) {
    R *xr = reinterpret_cast<R *>(x);
    if (dist == 0) { uniform01(2 * n, xr, iseed); return; }
    if (dist == 1) {
        uniform01(2 * n, xr, iseed);
        for (size_t i = 0; i < n; ++i) x[i] = R(2) * x[i] - std::complex<R>(R(1), R(1));
        return;
    }
    R pool[128];
    for (size_t i0 = 0; i0 < n; i0 += 64) {
        size_t ilim = 64;
        if (n < i0 + ilim) ilim = n - i0;
        uniform01(2 * ilim, pool, iseed);
        for (size_t i = 0; i < ilim; ++i) {
            R ang = R(6.28318530717958647692528676656) * pool[2 * i + 1];
            x[i0 + i] = std::sqrt(R(-2) * std::log1p(-pool[2 * i])) * std::complex<R>(std::cos(ang), std::sin(ang));
        }
    }
}

// ---------------------------------------------------------------------------
// MatrixGen (RNP/MatrixGen.hpp): GenerateDiagonal (:31-109) and RandomMatrix
// (:120-272) for real types (the reference's RandomMatrix does not compile
// for complex types).  sym: 0 Nonsymmetric, 1 Hermitian, 2 Hermitian
// positive definite, 3 Symmetric (the last three are one path for reals).
// ---------------------------------------------------------------------------
template <class T> void gen_diagonal(int dist, int mode, bool reverse, bool randsign, T cond, T dscale, size_t n, T *d, int iseed[4]) {
    if (n == 0) return;
    const T rcond = T(1) / cond;
    switch (mode) {
    case 1:
        d[0] = T(1);
        for (size_t i = 1; i < n; ++i) d[i] = rcond;
        break;
    case 2:
        for (size_t i = 0; i + 1 < n; ++i) d[i] = T(1);
        d[n - 1] = rcond;
        break;
    case 3:
        for (size_t i = 0; i < n; ++i) d[i] = std::pow(rcond, T(i) / T(n - 1));
        break;
    case 4:
        for (size_t i = 0; i < n; ++i) {
            const T t = T(i) / T(n - 1);
            d[i] = (T(1) - t) + t * rcond;
        }
        break;
    case 5:
        uniform01(n, d, iseed);
        for (size_t i = 0; i < n; ++i) d[i] = std::pow(rcond, d[i]);
        break;
    case 6:
        larnv_real(dist, n, d, iseed);
        break;
    default:
        break;
    }
    // RNP/MatrixGen.hpp:79-85 swaps d[i] and d[n-1-i] for every i in [0, n):
    // each pair is swapped twice, so "reverse" leaves d as it was; restated
    // as written
    if (reverse)
        for (size_t i = 0; i < n; ++i) std::swap(d[i], d[n - 1 - i]);
    if (randsign)
        for (size_t i = 0; i < n; ++i) {
            T r;
            uniform01(1, &r, iseed);
            if (T(2) * r > T(1)) d[i] = -d[i];
        }
    if (mode != 0 && mode != 6) {
        T maxabs = std::fabs(d[0]);
        for (size_t i = 1; i < n; ++i) maxabs = std::max(maxabs, std::fabs(d[i]));
        scal(n, dscale / maxabs, d, 1);
    }
}
// the reflector of a Normal01 vector w (length len): u = w / (w0 + wa) with
// u0 = 1, tau = (w0 + wa) / wa, wa = ||w|| sign(w0)  (RNP/MatrixGen.hpp:170-180)
template <class T> T mg_reflector(size_t len, T *w, int iseed[4]) {
    larnv_real(2, len, w, iseed);
    const T wn = norm2(len, w, 1);
    const T wa = (wn / std::fabs(w[0])) * w[0];
    T tau(0);
    if (wn != T(0)) {
        const T wb = w[0] + wa;
        scal(len - 1, T(1) / wb, w + 1, 1);
        w[0] = T(1);
        tau = wb / wa;
    }
    return tau;
}
template <class T> void random_matrix(int sym, int dist, int mode, bool reverse, T cond, T dmax, T *d_, size_t m, size_t n, T *a, size_t lda, int iseed[4]) {
    const size_t k = m < n ? m : n;
    if (k == 0) return;
    std::vector<T> dd(k), work(m + n);
    T *d = d_ ? d_ : dd.data();
    gen_diagonal(dist, mode, reverse, sym == 1, cond, dmax, k, d, iseed);
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i < m; ++i) a[i + j * lda] = (i == j) ? d[i] : T(0);
    T *w = work.data();
    if (sym == 0) {
        for (size_t i = k; i-- > 0;) {
            if (i + 1 < m) {
                const T tau = mg_reflector(m - i, w, iseed);
                gemv('C', m - i, n - i, T(1), &a[i + i * lda], lda, w, 1, T(0), w + m, 1);
                gerc(m - i, n - i, -tau, w, 1, w + m, 1, &a[i + i * lda], lda);
            }
            if (i + 1 < n) {
                const T tau = mg_reflector(n - i, w, iseed);
                gemv('N', m - i, n - i, T(1), &a[i + i * lda], lda, w, 1, T(0), w + n, 1);
                gerc(m - i, n - i, -tau, w + n, 1, w, 1, &a[i + i * lda], lda);
            }
        }
        return;
    }
    for (size_t i = n; i-- > 0;) {
        const size_t len = n - i;
        const T tau = mg_reflector(len, w, iseed);
        T *A = &a[i + i * lda];
        T *y = w + n;
        // y = tau A u (lower triangle of A)
        for (size_t r = 0; r < len; ++r) {
            T acc(0);
            for (size_t c = 0; c < len; ++c) acc += (r >= c ? A[r + c * lda] : A[c + r * lda]) * w[c];
            y[r] = tau * acc;
        }
        T dot(0);
        for (size_t r = 0; r < len; ++r) dot += y[r] * w[r];
        const T alpha = -(T(1) / T(2)) * tau * dot;
        for (size_t r = 0; r < len; ++r) y[r] += alpha * w[r];
        for (size_t c = 0; c < len; ++c)
            for (size_t r = c; r < len; ++r) A[r + c * lda] -= w[r] * y[c] + y[r] * w[c];
    }
    for (size_t j = 0; j < n; ++j)
        for (size_t i = j + 1; i < n; ++i) a[j + i * lda] = a[i + j * lda];
}

// ---------------------------------------------------------------------------
// LQ, QL and RQ (RNP/LA/LQ.hpp, QL.hpp, RQ.hpp) restated through the QR of a
// transformed matrix (J = reversal, X^H = conjugate transpose):
//   LQ(A) = [QR(A^H)]^H,  QL(A) = J QR(J A J) J,  RQ(A) = [J QR(J A^H J) J]^H,
// tau in reverse order for QL and RQ.  The reference's row-wise generation
// of a conjugated row (LQ.hpp:79-97, RQ.hpp:80-112), its bottom-up columns
// (QL.hpp:80-109) and its blocked updates with storev "R" / direction "B"
// (Reflector.hpp:627-676, 816-1062) perform the transformed operations of
// the QR's, so the results agree to rounding; the golden vectors of the
// reference build pin them.  MultQ: LQ and RQ flip trans; QL and RQ apply to
// C with its rows (side L) or columns (side R) reversed.
// ---------------------------------------------------------------------------
enum { kLQ = 0, kQL = 1, kRQ = 2 };
// dst (ldd) = X(src), src rows x cols
template <class T> void xform(int kind, size_t rows, size_t cols, const T *src, size_t lds, T *dst, size_t ldd) {
    for (size_t j = 0; j < cols; ++j)
        for (size_t i = 0; i < rows; ++i) {
            const T v = src[i + j * lds];
            if (kind == kLQ) dst[j + i * ldd] = Tr<T>::conj(v);
            else if (kind == kQL) dst[(rows - 1 - i) + (cols - 1 - j) * ldd] = v;
            else dst[(cols - 1 - j) + (rows - 1 - i) * ldd] = Tr<T>::conj(v);
        }
}
template <class T> void x_factor(int kind, size_t m, size_t n, T *a, size_t lda, T *tau) {
    const size_t k = m < n ? m : n;
    if (k == 0) return;
    const size_t mt = kind == kQL ? m : n, nt = kind == kQL ? n : m;
    std::vector<T> b(mt * nt), t(k);
    xform(kind, m, n, a, lda, b.data(), mt);
    size_t lw = 0;
    factor<T>(mt, nt, b.data(), mt, t.data(), &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    factor<T>(mt, nt, b.data(), mt, t.data(), &lw, w.data());
    xform(kind, mt, nt, b.data(), mt, a, lda);
    for (size_t i = 0; i < k; ++i) tau[i] = kind == kLQ ? t[i] : t[k - 1 - i];
}
template <class T> void x_multq(int kind, char side, char trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc) {
    if (m == 0 || n == 0 || k == 0) return;
    const bool left = side == 'L';
    const size_t nq = left ? m : n;
    std::vector<T> b(nq * k), t(k);
    if (kind == kQL) xform(kind, nq, k, a, lda, b.data(), nq);
    else xform(kind, k, nq, a, lda, b.data(), nq);
    for (size_t i = 0; i < k; ++i) t[i] = kind == kLQ ? tau[i] : tau[k - 1 - i];
    const char tr = kind == kQL ? trans : (trans == 'N' ? 'C' : 'N');
    auto flip = [&]() {
        if (kind == kLQ) return;
        if (left) {
            for (size_t j = 0; j < n; ++j)
                for (size_t i = 0; i < m / 2; ++i) std::swap(c[i + j * ldc], c[(m - 1 - i) + j * ldc]);
        } else {
            for (size_t j = 0; j < n / 2; ++j)
                for (size_t i = 0; i < m; ++i) std::swap(c[i + j * ldc], c[i + (n - 1 - j) * ldc]);
        }
    };
    flip();
    size_t lw = 0;
    multq<T>(side, tr, m, n, k, b.data(), nq, t.data(), c, ldc, &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    multq<T>(side, tr, m, n, k, b.data(), nq, t.data(), c, ldc, &lw, w.data());
    flip();
}
template <class T> void x_genq(int kind, size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau) {
    if (m == 0 || n == 0) return;
    const size_t mt = kind == kQL ? m : n, nt = kind == kQL ? n : m;
    std::vector<T> b(mt * nt), t(k > 0 ? k : 1);
    xform(kind, m, n, a, lda, b.data(), mt);
    for (size_t i = 0; i < k; ++i) t[i] = kind == kLQ ? tau[i] : tau[k - 1 - i];
    size_t lw = 0;
    genq<T>(mt, nt, k, b.data(), mt, t.data(), &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    genq<T>(mt, nt, k, b.data(), mt, t.data(), &lw, w.data());
    xform(kind, mt, nt, b.data(), mt, a, lda);
}

// ---------------------------------------------------------------------------
// Callers of QR / QL: the Q of a Hessenberg reduction and of a Hermitian
// tridiagonal reduction, and the QR step of the complex generalized
// eigensystem driver.  Each is the reference's composition restated over the
// restated QR / QL above.
// ---------------------------------------------------------------------------
template <class T> void q_multq(char side, char trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc) {
    size_t lw = 0;
    multq<T>(side, trans, m, n, k, a, lda, tau, c, ldc, &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    multq<T>(side, trans, m, n, k, a, lda, tau, c, ldc, &lw, w.data());
}
template <class T> void q_genq(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau) {
    size_t lw = 0;
    genq<T>(m, n, k, a, lda, tau, &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    genq<T>(m, n, k, a, lda, tau, &lw, w.data());
}
// Hessenberg::MultQ (RNP/LA/Hessenberg.hpp:477-512): QR MultQ with the nh =
// ihi-ilo-1 reflectors below the subdiagonal of columns ilo.., on rows (left)
// or columns (right) ilo+1 .. ihi-1 of C
template <class T> void hess_multq(char side, char trans, size_t m, size_t n, size_t ilo, size_t ihi, const T *a, size_t lda, const T *tau, T *c, size_t ldc) {
    const bool left = side == 'L';
    const size_t nh = ihi - ilo - 1;
    const size_t mi = left ? nh : m, ni = left ? n : nh;
    const size_t off = left ? ilo + 1 : (ilo + 1) * ldc;
    q_multq<T>(side, trans, mi, ni, nh, a + (ilo + 1) + ilo * lda, lda, tau + ilo, c + off, ldc);
}
// Hessenberg::GenerateQ (Hessenberg.hpp:539-590): reflector vectors moved one
// column right (columns ihi-1 down to ilo+1), the rest of the matrix set to
// the identity, then QR GenerateQ of the nh x nh block at (ilo+1, ilo+1)
template <class T> void hess_genq(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, const T *tau) {
    if (n == 0) return;
    for (size_t j = ihi - 1; j > ilo; --j) {
        T *col = a + j * lda;
        const T *prev = a + (j - 1) * lda;
        for (size_t i = 0; i < j; ++i) col[i] = T(0);
        for (size_t i = j + 1; i < ihi; ++i) col[i] = prev[i];
        for (size_t i = ihi; i < n; ++i) col[i] = T(0);
    }
    for (size_t j = 0; j < n; ++j) {
        if (j > ilo && j < ihi) continue;
        for (size_t i = 0; i < n; ++i) a[i + j * lda] = (i == j) ? T(1) : T(0);
    }
    const size_t nh = ihi - ilo - 1;
    if (nh > 0) q_genq<T>(nh, nh, nh, a + (ilo + 1) * (lda + 1), lda, tau + ilo);
}
// Tridiagonal::GenerateQHerm (Tridiagonal.hpp:1037-1097): "U" moves the
// vectors one column left and generates a QL factor's Q in the leading
// (n-1) x (n-1) block; "L" moves them one column right and generates a QR
// factor's Q in the trailing block
template <class T> void trid_genq(char uplo, size_t n, T *a, size_t lda, const T *tau) {
    if (n == 0) return;
    if (uplo == 'U') {
        for (size_t j = 0; j + 1 < n; ++j) {
            for (size_t i = 0; i < j; ++i) a[i + j * lda] = a[i + (j + 1) * lda];
            a[(n - 1) + j * lda] = T(0);
        }
        for (size_t i = 0; i + 1 < n; ++i) a[i + (n - 1) * lda] = T(0);
        a[(n - 1) + (n - 1) * lda] = T(1);
        if (n > 1) x_genq<T>(kQL, n - 1, n - 1, n - 1, a, lda, tau);
    } else {
        for (size_t j = n - 1; j >= 1; --j) {
            a[j * lda] = T(0);
            for (size_t i = j + 1; i < n; ++i) a[i + j * lda] = a[i + (j - 1) * lda];
        }
        a[0] = T(1);
        for (size_t i = 1; i < n; ++i) a[i] = T(0);
        if (n > 1) q_genq<T>(n - 1, n - 1, n - 1, a + 1 + lda, lda, tau);
    }
}
// Tridiagonal::MultQHerm (Tridiagonal.hpp:1140-1188)
template <class T> void trid_multq(char side, char uplo, char trans, size_t m, size_t n, const T *a, size_t lda, const T *tau, T *c, size_t ldc) {
    const bool left = side == 'L';
    const size_t nq = left ? m : n;
    if (m == 0 || n == 0 || nq == 1) return;
    const size_t mi = left ? m - 1 : m, ni = left ? n : n - 1;
    if (uplo == 'U') x_multq<T>(kQL, side, trans, mi, ni, nq - 1, a + lda, lda, tau, c, ldc);
    else q_multq<T>(side, trans, mi, ni, nq - 1, a + 1, lda, tau, c + (left ? 1 : ldc), ldc);
}
// The QR step of ComplexGeneralizedEigensystem (GeneralizedEigensystems.hpp:
// 457-472): B(ilo:ihi, ilo:ilo+icols) factored, Q^H applied to A's block,
// vl = I with Q generated in its (ilo:ihi, ilo:ihi) block from B's strictly
// lower part, vr = I; tau (n) returned
template <class T> void gg_triangularize_b(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, T *b, size_t ldb, T *vl, size_t ldvl, T *vr, size_t ldvr, T *tau) {
    const size_t irows = ihi - ilo, icols = (vl || vr) ? n - ilo : irows;
    T *bb = b + ilo + ilo * ldb;
    size_t lw = 0;
    factor<T>(irows, icols, bb, ldb, tau, &lw, nullptr);
    std::vector<T> w(lw > 0 ? lw : 1);
    factor<T>(irows, icols, bb, ldb, tau, &lw, w.data());
    q_multq<T>('L', 'C', irows, icols, irows, bb, ldb, tau, a + ilo + ilo * lda, lda);
    if (vl) {
        for (size_t j = 0; j < n; ++j)
            for (size_t i = 0; i < n; ++i) vl[i + j * ldvl] = (i == j) ? T(1) : T(0);
        for (size_t j = 0; j + 1 < irows; ++j)
            for (size_t i = j; i + 1 < irows; ++i) vl[(ilo + 1 + i) + (ilo + j) * ldvl] = b[(ilo + 1 + i) + (ilo + j) * ldb];
        q_genq<T>(irows, irows, irows, vl + ilo + ilo * ldvl, ldvl, tau);
    }
    if (vr)
        for (size_t j = 0; j < n; ++j)
            for (size_t i = 0; i < n; ++i) vr[i + j * ldvr] = (i == j) ? T(1) : T(0);
}

} // namespace orc

// ---------------------------------------------------------------------------
// extern "C" surface for ctypes (tests, smoke check, CPU baseline)
// ---------------------------------------------------------------------------
using namespace orc;
#define ORC_DEF(P, T)                                                                                                  \
    extern "C" void oracle_##P##geqrf(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) { factor<T>(m, n, a, lda, tau, lwork, work); } \
    extern "C" void oracle_##P##geqr2(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) { factor_unblocked<T>(m, n, a, lda, tau, work); } \
    extern "C" void oracle_##P##unmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) { multq<T>(side[0], trans[0], m, n, k, a, lda, tau, c, ldc, lwork, work); } \
    extern "C" void oracle_##P##unm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, T *work) { multq_unblocked<T>(side[0], trans[0], m, n, k, a, lda, tau, c, ldc, work); } \
    extern "C" void oracle_##P##ungqr(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) { genq<T>(m, n, k, a, lda, tau, lwork, work); } \
    extern "C" void oracle_##P##ung2r(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) { genq_unblocked<T>(m, n, k, a, lda, tau, work); } \
    extern "C" void oracle_##P##larfg(size_t n, T *alpha, T *x, size_t incx, T *tau) { generate<T>(n, alpha, x, incx, tau); } \
    extern "C" void oracle_##P##larft(size_t n, size_t k, const T *v, size_t ldv, const T *tau, T *t, size_t ldt) { block_tr<T>(n, k, v, ldv, tau, t, ldt); } \
    extern "C" void oracle_##P##gels(size_t m, size_t n, size_t nrhs, T *a, size_t lda, T *tau, T *b, size_t ldb) { gels<T>(m, n, nrhs, a, lda, tau, b, ldb); }
#define ORC_XDEF(P, T, F, M, G, KIND)                                                                                   \
    extern "C" void oracle_##P##F(size_t m, size_t n, T *a, size_t lda, T *tau) { x_factor<T>(KIND, m, n, a, lda, tau); } \
    extern "C" void oracle_##P##M(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, \
                                  const T *tau, T *c, size_t ldc) { x_multq<T>(KIND, side[0], trans[0], m, n, k, a, lda, tau, c, ldc); } \
    extern "C" void oracle_##P##G(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau) { x_genq<T>(KIND, m, n, k, a, lda, tau); }
#define ORC_XDEF3(P, T)                             \
    ORC_XDEF(P, T, gelqf, unmlq, unglq, kLQ)        \
    ORC_XDEF(P, T, geqlf, unmql, ungql, kQL)        \
    ORC_XDEF(P, T, gerqf, unmrq, ungrq, kRQ)
#define ORC_CONS(P, T)                                                                                                  \
    extern "C" void oracle_##P##unmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const T *a, size_t lda, \
                                      const T *tau, T *c, size_t ldc) { hess_multq<T>(side[0], trans[0], m, n, ilo, ihi, a, lda, tau, c, ldc); } \
    extern "C" void oracle_##P##unghr(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, const T *tau) { hess_genq<T>(n, ilo, ihi, a, lda, tau); } \
    extern "C" void oracle_##P##ungtr(const char *uplo, size_t n, T *a, size_t lda, const T *tau) { trid_genq<T>(uplo[0], n, a, lda, tau); } \
    extern "C" void oracle_##P##unmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const T *a, size_t lda, \
                                      const T *tau, T *c, size_t ldc) { trid_multq<T>(side[0], uplo[0], trans[0], m, n, a, lda, tau, c, ldc); }
ORC_CONS(s, float)
ORC_CONS(d, double)
ORC_CONS(c, cf)
ORC_CONS(z, cd)
extern "C" void oracle_cgg_triangularize_b(size_t n, size_t ilo, size_t ihi, cf *a, size_t lda, cf *b, size_t ldb, cf *vl, size_t ldvl, cf *vr, size_t ldvr, cf *tau) {
    gg_triangularize_b<cf>(n, ilo, ihi, a, lda, b, ldb, vl, ldvl, vr, ldvr, tau);
}
extern "C" void oracle_zgg_triangularize_b(size_t n, size_t ilo, size_t ihi, cd *a, size_t lda, cd *b, size_t ldb, cd *vl, size_t ldvl, cd *vr, size_t ldvr, cd *tau) {
    gg_triangularize_b<cd>(n, ilo, ihi, a, lda, b, ldb, vl, ldvl, vr, ldvr, tau);
}
ORC_XDEF3(s, float)
ORC_XDEF3(d, double)
ORC_XDEF3(c, cf)
ORC_XDEF3(z, cd)
ORC_DEF(s, float)
ORC_DEF(d, double)
ORC_DEF(c, cf)
ORC_DEF(z, cd)

extern "C" void oracle_srandom_matrix(int sym, int dist, int mode, int reverse, float cond, float dmax, float *d, size_t m, size_t n, float *a, size_t lda, int *iseed) {
    random_matrix<float>(sym, dist, mode, reverse != 0, cond, dmax, d, m, n, a, lda, iseed);
}
extern "C" void oracle_drandom_matrix(int sym, int dist, int mode, int reverse, double cond, double dmax, double *d, size_t m, size_t n, double *a, size_t lda, int *iseed) {
    random_matrix<double>(sym, dist, mode, reverse != 0, cond, dmax, d, m, n, a, lda, iseed);
}
extern "C" double oracle_dnrm2(size_t n, const double *x, size_t incx) { return norm2<double>(n, x, incx); }
extern "C" double oracle_dznrm2(size_t n, const cd *x, size_t incx) { return norm2<cd>(n, x, incx); }
extern "C" void oracle_dlarnv(int dist, int *iseed, size_t n, double *x) { larnv_real<double>(dist, n, x, iseed); }
extern "C" void oracle_slarnv(int dist, int *iseed, size_t n, float *x) { larnv_real<float>(dist, n, x, iseed); }
extern "C" void oracle_zlarnv(int dist, int *iseed, size_t n, cd *x) { larnv_cplx<double>(dist, n, x, iseed); }
extern "C" void oracle_clarnv(int dist, int *iseed, size_t n, cf *x) { larnv_cplx<float>(dist, n, x, iseed); }

// CPU baseline only: route the level-2 and level-3 calls (gemv, ger/gerc,
// trmv, gemm, trmm, trsm: every routine the reference forwards to its BLAS)
// through an external Fortran BLAS
// (e.g. an OpenBLAS shared library; symbols looked up as prefix + "dgemm_").
// Returns 0 on success, -1 if the library or a symbol is missing.
extern "C" int oracle_use_blas(const char *path, const char *prefix, int nthreads) {
    if (path == nullptr) { g_use_ext = false; return 0; }
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    std::string p = prefix ? prefix : "";
    auto sym = [&](const char *n) { return dlsym(h, (p + n).c_str()); };
    g_ext.h = h;
    g_ext.dgemm = (decltype(g_ext.dgemm))sym("dgemm_");
    g_ext.zgemm = (decltype(g_ext.zgemm))sym("zgemm_");
    g_ext.sgemm = (decltype(g_ext.sgemm))sym("sgemm_");
    g_ext.cgemm = (decltype(g_ext.cgemm))sym("cgemm_");
    g_ext.dtrmm = (decltype(g_ext.dtrmm))sym("dtrmm_");
    g_ext.ztrmm = (decltype(g_ext.ztrmm))sym("ztrmm_");
    g_ext.strmm = (decltype(g_ext.strmm))sym("strmm_");
    g_ext.ctrmm = (decltype(g_ext.ctrmm))sym("ctrmm_");
    g_ext.dtrsm = (decltype(g_ext.dtrsm))sym("dtrsm_");
    g_ext.ztrsm = (decltype(g_ext.ztrsm))sym("ztrsm_");
    g_ext.strsm = (decltype(g_ext.strsm))sym("strsm_");
    g_ext.ctrsm = (decltype(g_ext.ctrsm))sym("ctrsm_");
    g_ext.dgemv = (decltype(g_ext.dgemv))sym("dgemv_");
    g_ext.zgemv = (decltype(g_ext.zgemv))sym("zgemv_");
    g_ext.sgemv = (decltype(g_ext.sgemv))sym("sgemv_");
    g_ext.cgemv = (decltype(g_ext.cgemv))sym("cgemv_");
    g_ext.dger = (decltype(g_ext.dger))sym("dger_");
    g_ext.zgerc = (decltype(g_ext.zgerc))sym("zgerc_");
    g_ext.sger = (decltype(g_ext.sger))sym("sger_");
    g_ext.cgerc = (decltype(g_ext.cgerc))sym("cgerc_");
    g_ext.dtrmv = (decltype(g_ext.dtrmv))sym("dtrmv_");
    g_ext.ztrmv = (decltype(g_ext.ztrmv))sym("ztrmv_");
    g_ext.strmv = (decltype(g_ext.strmv))sym("strmv_");
    g_ext.ctrmv = (decltype(g_ext.ctrmv))sym("ctrmv_");
    g_ext.set_threads = (decltype(g_ext.set_threads))sym("openblas_set_num_threads");
    if (!g_ext.dgemm || !g_ext.zgemm || !g_ext.dtrmm || !g_ext.ztrmm || !g_ext.dgemv || !g_ext.zgemv || !g_ext.dger || !g_ext.zgerc ||
        !g_ext.dtrmv || !g_ext.ztrmv) { g_use_ext = false; return -1; }
    if (g_ext.set_threads && nthreads > 0) g_ext.set_threads(nthreads);
    g_use_ext = true;
    return 0;
}
extern "C" int oracle_blas_active(void) { return g_use_ext ? 1 : 0; }
