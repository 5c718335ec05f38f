// consumers.cuh — the reference's callers of QR / QL on the GPU: the Q of a
// Hessenberg reduction (RNP::LA::Hessenberg::MultQ / GenerateQ,
// RNP/LA/Hessenberg.hpp:477-590), the Q of a Hermitian tridiagonal reduction
// (RNP::LA::Tridiagonal::GenerateQHerm / MultQHerm, RNP/LA/Tridiagonal.hpp:
// 1037-1188), and the QR step of the complex generalized eigensystem driver
// (RNP/LA/GeneralizedEigensystems.hpp:457-472: B triangularized, its Q^H
// applied to A, the left vectors started from Q).
//
// Each is the reference's composition of QR::MultQ / QR::GenerateQ /
// QL::MultQ / QL::GenerateQ on a sub-block, run on the GPU routines of those
// (qr_driver.cuh, lqr_driver.cuh).  The only new device work is the in-place
// column shift that GenerateQ and GenerateQHerm do before generating Q (the
// reflector vectors moved one column right or left, the border set to the
// identity): one thread per row walks the columns in the order that reads
// every source column before it is overwritten, 8 columns per step so that
// eight loads are in flight.
#pragma once
#include "lqr_driver.cuh"

namespace rnpgpu {

constexpr int kShiftChunk = 8;

// Hessenberg::GenerateQ's shift (Hessenberg.hpp:556-581): for ilo < j < ihi,
// column j takes column j-1's rows j+1 .. ihi-1, rows above j and from ihi on
// become zero and the diagonal entry is kept; columns 0..ilo and ihi..n-1
// become unit columns.
template <class T> __global__ void __launch_bounds__(128) k_hess_shift(int n, int ilo, int ihi, T *A, size_t lda) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T *row = A + i;
    for (int j1 = n; j1 > 0; j1 -= kShiftChunk) {
        const int j0 = max(j1 - kShiftChunk, 0);
        T src[kShiftChunk];
#pragma unroll
        for (int u = 0; u < kShiftChunk; ++u) {
            const int j = j1 - 1 - u;
            const bool mv = j >= j0 && j > ilo && j < ihi && i > j && i < ihi;
            src[u] = mv ? row[(size_t)(j - 1) * lda] : T(0);
        }
#pragma unroll
        for (int u = 0; u < kShiftChunk; ++u) {
            const int j = j1 - 1 - u;
            if (j < j0) continue;
            if (j <= ilo || j >= ihi) row[(size_t)j * lda] = (i == j) ? T(1) : T(0);
            else if (i != j) row[(size_t)j * lda] = src[u];
        }
    }
}

// Tridiagonal::GenerateQHerm's shifts (Tridiagonal.hpp:1059-1094).
// upper: for j < n-1, column j takes column j+1's rows above j and its last
// row becomes zero (rows j .. n-2 kept); the last column becomes e_{n-1}.
// lower: for j >= 1, column j takes column j-1's rows below j and its first
// row becomes zero (rows 1 .. j kept); the first column becomes e_0.
template <class T> __global__ void __launch_bounds__(128) k_trid_shift(int upper, int n, T *A, size_t lda) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T *row = A + i;
    if (upper) {
        for (int j0 = 0; j0 < n - 1; j0 += kShiftChunk) {
            const int j1 = min(j0 + kShiftChunk, n - 1);
            T src[kShiftChunk];
#pragma unroll
            for (int u = 0; u < kShiftChunk; ++u) {
                const int j = j0 + u;
                src[u] = (j < j1 && i < j) ? row[(size_t)(j + 1) * lda] : T(0);
            }
#pragma unroll
            for (int u = 0; u < kShiftChunk; ++u) {
                const int j = j0 + u;
                if (j >= j1) continue;
                if (i < j || i == n - 1) row[(size_t)j * lda] = src[u];
            }
        }
        row[(size_t)(n - 1) * lda] = (i == n - 1) ? T(1) : T(0);
    } else {
        for (int j1 = n; j1 > 1; j1 -= kShiftChunk) {
            const int j0 = max(j1 - kShiftChunk, 1);
            T src[kShiftChunk];
#pragma unroll
            for (int u = 0; u < kShiftChunk; ++u) {
                const int j = j1 - 1 - u;
                src[u] = (j >= j0 && i > j) ? row[(size_t)(j - 1) * lda] : T(0);
            }
#pragma unroll
            for (int u = 0; u < kShiftChunk; ++u) {
                const int j = j1 - 1 - u;
                if (j < j0) continue;
                if (i > j || i == 0) row[(size_t)j * lda] = src[u];
            }
        }
        row[0] = (i == 0) ? T(1) : T(0);
    }
}

// dst(i, j) = src(i, j) for i >= j, i < m, j < n (Triangular::Copy "L",
// RNP/LA/Triangular.hpp:271-281)
template <class T> __global__ void __launch_bounds__(256) k_copy_lower(int m, int n, const T *src, size_t lds, T *dst, size_t ldd) {
    for (int j = blockIdx.y; j < n; j += gridDim.y)
        for (int i = j + blockIdx.x * 256 + threadIdx.x; i < m; i += gridDim.x * 256) dst[i + (size_t)j * ldd] = src[i + (size_t)j * lds];
}

template <class T> int shift_launch(int which, int n, int ilo, int ihi, T *a, size_t lda, cudaStream_t st) {
    if (n <= 0) return kOk;
    KScope ks("q_shift", st);
    const unsigned g = (unsigned)((n + 127) / 128);
    if (which == 0) k_hess_shift<T><<<g, 128, 0, st>>>(n, ilo, ihi, a, lda);
    else k_trid_shift<T><<<g, 128, 0, st>>>(which == 1, n, a, lda);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

inline bool valid_side(const char *s) { return s[0] == 'L' || s[0] == 'R'; }
inline bool valid_trans(const char *t) { return t[0] == 'N' || t[0] == 'T' || t[0] == 'C'; }

// The sub-call's status, renumbered to the caller's argument positions:
// map[i] is the caller's position of the sub-call's argument i+1 (0: none).
inline int remap_status(int rc, std::initializer_list<int> map) {
    if (rc >= 0) return rc;
    const int i = -rc - 1;
    if (i < (int)map.size() && map.begin()[i] > 0) return -map.begin()[i];
    return rc;
}

// ---------------------------------------------------------------------------
// Hessenberg::MultQ (Hessenberg.hpp:477-512), LAPACK _unmhr: C = op(Q) C or
// C op(Q), Q = H[ilo] ... H[ihi-2] from Reduce; the reflectors lie below the
// subdiagonal of columns ilo .. ihi-2.  Arguments: side 1, trans 2, m 3, n 4,
// ilo 5, ihi 6, a 7, lda 8, tau 9, c 10, ldc 11, lwork 12, work 13.
// ---------------------------------------------------------------------------
template <class T> int unmhr(const char *side, const char *trans, size_t m, size_t n, size_t ilo, size_t ihi, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    if (side == nullptr || !valid_side(side)) return -1;
    if (trans == nullptr || !valid_trans(trans)) return -2;
    if (lwork == nullptr) return -12;
    const bool left = side[0] == 'L';
    const size_t nq = left ? m : n;
    if (ilo > nq) return -5;
    if (ihi <= ilo || ihi > nq) return -6;
    if (lda < std::max<size_t>(1, nq)) return -8;
    if (ldc < std::max<size_t>(1, m)) return -11;
    const size_t nh = ihi - ilo - 1;
    const size_t mi = left ? nh : m, ni = left ? n : nh;
    const size_t i1 = left ? ilo + 1 : 0, i2 = left ? 0 : ilo + 1;
    const T *as = a ? a + (ilo + 1) + ilo * lda : nullptr;
    const T *ts = tau ? tau + ilo : nullptr;
    T *cs = c ? c + i1 + i2 * ldc : nullptr;
    const int rc = unmqr<T>(side, trans, mi, ni, nh, as, lda, ts, cs, ldc, lwork, work);
    return remap_status(rc, {1, 2, 3, 4, 0, 7, 8, 9, 10, 11, 12, 13});
}

// ---------------------------------------------------------------------------
// Hessenberg::GenerateQ (Hessenberg.hpp:539-590), LAPACK _unghr: a (the
// reduction) is overwritten by the n x n Q.  Arguments: n 1, ilo 2, ihi 3,
// a 4, lda 5, tau 6, lwork 7, work 8.
// ---------------------------------------------------------------------------
template <class T> int unghr(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    if (lwork == nullptr) return -7;
    if (ilo > n) return -2;
    if (ihi <= ilo || ihi > n) return -3;
    if (lda < std::max<size_t>(1, n)) return -5;
    if (n > (size_t)INT32_MAX) return -1;
    const size_t nh = ihi - ilo - 1;
    if (work == nullptr || *lwork == 0) {
        size_t q = 0;
        int rc = nh > 0 ? ungqr<T>(nh, nh, nh, nullptr, lda, nullptr, &q, nullptr) : kOk;
        if (rc) return remap_status(rc, {0, 0, 0, 4, 5, 6, 7, 8});
        *lwork = std::max<size_t>(q, 1);
        return kOk;
    }
    if (n == 0) return kOk;
    if (a == nullptr) return -4;
    if (tau == nullptr && nh > 0) return -6;
    int rc = shift_launch<T>(0, (int)n, (int)ilo, (int)ihi, a, lda, current_stream());
    if (rc || nh == 0) return rc;
    rc = ungqr<T>(nh, nh, nh, a + (ilo + 1) * (lda + 1), lda, tau + ilo, lwork, work);
    return remap_status(rc, {0, 0, 0, 4, 5, 6, 7, 8});
}

// ---------------------------------------------------------------------------
// Tridiagonal::GenerateQHerm (Tridiagonal.hpp:1037-1097), LAPACK _ungtr:
// uplo "U": Q = H[n-2] ... H[0] from the upper triangle, generated as a QL
// factor's Q; "L": Q = H[0] ... H[n-2] from the lower triangle, as a QR
// factor's Q.  Arguments: uplo 1, n 2, a 3, lda 4, tau 5, lwork 6, work 7.
// ---------------------------------------------------------------------------
template <class T> int ungtr(const char *uplo, size_t n, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    if (uplo == nullptr || (uplo[0] != 'U' && uplo[0] != 'L')) return -1;
    if (lwork == nullptr) return -6;
    if (lda < std::max<size_t>(1, n)) return -4;
    if (n == 0) return kOk;
    if (n > (size_t)INT32_MAX) return -2;
    const bool upper = uplo[0] == 'U';
    const size_t k = n - 1;
    const std::initializer_list<int> map = {0, 0, 0, 3, 4, 5, 6, 7};
    if (work == nullptr || *lwork == 0) {
        size_t q = 0;
        int rc = kOk;
        if (k > 0) rc = upper ? xungqr<T>(kXQL, k, k, k, nullptr, lda, nullptr, &q, nullptr) : ungqr<T>(k, k, k, nullptr, lda, nullptr, &q, nullptr);
        if (rc) return remap_status(rc, map);
        *lwork = std::max<size_t>(q, 1);
        return kOk;
    }
    if (a == nullptr) return -3;
    if (tau == nullptr && k > 0) return -5;
    int rc = shift_launch<T>(upper ? 1 : 2, (int)n, 0, 0, a, lda, current_stream());
    if (rc || k == 0) return rc;
    rc = upper ? xungqr<T>(kXQL, k, k, k, a, lda, tau, lwork, work) : ungqr<T>(k, k, k, a + 1 + lda, lda, tau, lwork, work);
    return remap_status(rc, map);
}

// ---------------------------------------------------------------------------
// Tridiagonal::MultQHerm (Tridiagonal.hpp:1140-1188), LAPACK _unmtr.
// Arguments: side 1, uplo 2, trans 3, m 4, n 5, a 6, lda 7, tau 8, c 9,
// ldc 10, lwork 11, work 12.
// ---------------------------------------------------------------------------
template <class T> int unmtr(const char *side, const char *uplo, const char *trans, size_t m, size_t n, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    if (side == nullptr || !valid_side(side)) return -1;
    if (uplo == nullptr || (uplo[0] != 'U' && uplo[0] != 'L')) return -2;
    if (trans == nullptr || !valid_trans(trans)) return -3;
    if (lwork == nullptr) return -11;
    const bool left = side[0] == 'L', upper = uplo[0] == 'U';
    const size_t nq = left ? m : n;
    if (lda < std::max<size_t>(1, nq)) return -7;
    if (ldc < std::max<size_t>(1, m)) return -10;
    if (m == 0 || n == 0 || nq == 1) return kOk;
    const size_t mi = left ? m - 1 : m, ni = left ? n : n - 1;
    const std::initializer_list<int> map = {1, 3, 4, 5, 0, 6, 7, 8, 9, 10, 11, 12};
    int rc;
    if (upper) {
        const T *as = a ? a + lda : nullptr;
        rc = xunmqr<T>(kXQL, side, trans, mi, ni, nq - 1, as, lda, tau, c, ldc, lwork, work);
    } else {
        const size_t i1 = left ? 1 : 0, i2 = left ? 0 : 1;
        const T *as = a ? a + 1 : nullptr;
        T *cs = c ? c + i1 + i2 * ldc : nullptr;
        rc = unmqr<T>(side, trans, mi, ni, nq - 1, as, lda, tau, cs, ldc, lwork, work);
    }
    return remap_status(rc, map);
}

// ---------------------------------------------------------------------------
// The QR step of ComplexGeneralizedEigensystem (GeneralizedEigensystems.hpp:
// 376-412 workspace, 451-472 the step): with irows = ihi - ilo and icols =
// n - ilo when vl or vr is given (else irows), B(ilo:ihi, ilo:ilo+icols) is
// factored, Q^H is applied to A(ilo:ihi, ilo:ilo+icols), vl (if given) is set
// to I with Q generated in its (ilo:ihi, ilo:ihi) block, vr (if given) to I.
// The workspace is laid out as the reference's: [tau (n) | work].
// Arguments: n 1, ilo 2, ihi 3, a 4, lda 5, b 6, ldb 7, vl 8, ldvl 9, vr 10,
// ldvr 11, lwork 12, work 13.
// ---------------------------------------------------------------------------
template <class T> int gg_triangularize_b(size_t n, size_t ilo, size_t ihi, T *a, size_t lda, T *b, size_t ldb, T *vl, size_t ldvl, T *vr, size_t ldvr, size_t *lwork, T *work) {
    if (lwork == nullptr) return -12;
    if (n == 0) return kOk;
    if (ilo > n) return -2;
    if (ihi <= ilo || ihi > n) return -3;
    if (lda < n) return -5;
    if (ldb < n) return -7;
    if (vl != nullptr && ldvl < n) return -9;
    if (vr != nullptr && ldvr < n) return -11;
    if (n > (size_t)INT32_MAX) return -1;
    const bool vectors = vl != nullptr || vr != nullptr;
    const size_t irows = ihi - ilo, icols = vectors ? n - ilo : irows;
    // sub-workspaces: the reference's query takes them at the full n (its
    // lines 400-407); the call uses the actual irows / icols
    auto sub_need = [&](size_t r, size_t cc, size_t *need) -> int {
        size_t f = 0, mq = 0, g = 0;
        int rc = geqrf<T>(r, cc, nullptr, std::max<size_t>(r, 1), nullptr, &f, nullptr);
        if (!rc) rc = unmqr<T>("L", "C", r, cc, r, nullptr, std::max<size_t>(r, 1), nullptr, nullptr, std::max<size_t>(r, 1), &mq, nullptr);
        if (!rc && vl != nullptr) rc = ungqr<T>(r, r, r, nullptr, std::max<size_t>(r, 1), nullptr, &g, nullptr);
        *need = std::max(std::max(f, mq), std::max<size_t>(g, 1));
        return rc;
    };
    size_t need = 0;
    if (work == nullptr || *lwork == 0) {
        int rc = sub_need(n, n, &need);
        if (rc) return rc;
        *lwork = n + need;
        return kOk;
    }
    if (a == nullptr) return -4;
    if (b == nullptr) return -6;
    if (*lwork <= n) return -12;
    T *tau = work, *work2 = work + n;
    size_t lwork2 = *lwork - n;
    int rc = geqrf<T>(irows, icols, b + ilo + ilo * ldb, ldb, tau, &lwork2, work2);
    if (rc) return remap_status(rc, {0, 0, 6, 7, 13, 12, 13});
    rc = unmqr<T>("L", "C", irows, icols, irows, b + ilo + ilo * ldb, ldb, tau, a + ilo + ilo * lda, lda, &lwork2, work2);
    if (rc) return remap_status(rc, {0, 0, 0, 0, 0, 6, 7, 13, 4, 5, 12, 13});
    cudaStream_t st = current_stream();
    if (vl != nullptr) {
        const dim3 grid((unsigned)std::min<size_t>((n + 255) / 256, 64), (unsigned)std::min<size_t>(n, 4096));
        k_identity_cols<T><<<grid, 256, 0, st>>>((int)n, 0, (int)n, vl, ldvl);
        RNPGPU_CHECK_LAUNCH();
        if (irows > 1) {
            const size_t r = irows - 1;
            const dim3 g2((unsigned)std::min<size_t>((r + 255) / 256, 64), (unsigned)std::min<size_t>(r, 4096));
            k_copy_lower<T><<<g2, 256, 0, st>>>((int)r, (int)r, b + ilo + 1 + ilo * ldb, ldb, vl + ilo + 1 + ilo * ldvl, ldvl);
            RNPGPU_CHECK_LAUNCH();
        }
        rc = ungqr<T>(irows, irows, irows, vl + ilo + ilo * ldvl, ldvl, tau, &lwork2, work2);
        if (rc) return remap_status(rc, {0, 0, 0, 8, 9, 13, 12, 13});
    }
    if (vr != nullptr) {
        const dim3 grid((unsigned)std::min<size_t>((n + 255) / 256, 64), (unsigned)std::min<size_t>(n, 4096));
        k_identity_cols<T><<<grid, 256, 0, st>>>((int)n, 0, (int)n, vr, ldvr);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

} // namespace rnpgpu
