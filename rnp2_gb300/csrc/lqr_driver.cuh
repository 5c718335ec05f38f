// lqr_driver.cuh — LQ, QL and RQ factorizations (RNP::LA::LQ, QL, RQ:
// RNP/LA/LQ.hpp, QL.hpp, RQ.hpp) on the GB300 QR kernels.
//
// Each of the three is the QR factorization of a transformed matrix; with J
// the reversal permutation and X^H the conjugate transpose:
//
//   LQ(A) = [QR(A^H)]^H              tau unchanged
//   QL(A) = J [QR(J A J)] J          tau in reverse order
//   RQ(A) = [J QR(J A^H J) J]^H      tau in reverse order
//
// The identities hold reflector by reflector: the reference's row-wise
// Generate of a conjugated row (LQ.hpp:79-97) and its bottom-up columns (QL)
// make the same beta, tau and v as the QR of the transformed matrix, and its
// blocked updates (GenerateBlockTr / ApplyBlock with storev "R" or direction
// "B", RNP/LA/Reflector.hpp:627-676, 816-1062) are the transformed ones of the
// QR's.  So MultQ and GenerateQ follow too:
//   LQ: MultQ(side, trans) = QR MultQ(side, trans flipped) on A^H's reflectors
//   QL: MultQ(side, trans) = J (QR MultQ(side, trans) on J C) (rows of C for
//       side L, columns for side R)
//   RQ: both of the above (reflectors J A^H J, trans flipped, C reversed)
//   GenerateQ: the QR GenerateQ of the transformed factor, transformed back.
//
// Here the caller's matrix is transformed into the workspace (a tiled,
// coalesced transpose / reversal), the blocked QR routines run on it, and the
// result is transformed back.  The workspace query adds the transformed copy
// (and the reversed tau) to the QR routine's own workspace.
#pragma once
#include "qr_driver.cuh"

namespace rnpgpu {

enum : int { kXLQ = 0, kXQL = 1, kXRQ = 2 };

// dst = X(src) for src rows x cols:  LQ: dst = src^H (cols x rows);
// QL: dst = J src J (rows x cols);  RQ: dst = J src^H J (cols x rows).
// 32 x 32 tiles through shared memory (reads and writes coalesced).
template <class T> __global__ void __launch_bounds__(256) k_xform(int kind, int rows, int cols, const T *src, size_t lds, T *dst, size_t ldd) {
    __shared__ T tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    for (int yy = ty; yy < 32; yy += 8) {
        const int i = i0 + tx, j = j0 + yy;
        if (i < rows && j < cols) {
            const T v = src[i + (size_t)j * lds];
            if (kind == kXQL) dst[(size_t)(rows - 1 - i) + (size_t)(cols - 1 - j) * ldd] = v;
            else tile[yy][tx] = v;
        }
    }
    if (kind == kXQL) return;
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {
        const int j = j0 + tx, i = i0 + yy;
        if (i < rows && j < cols) {
            const T v = Tr<T>::conj(tile[tx][yy]);
            if (kind == kXLQ) dst[(size_t)j + (size_t)i * ldd] = v;
            else dst[(size_t)(cols - 1 - j) + (size_t)(rows - 1 - i) * ldd] = v;
        }
    }
}

// out[i] = in[n - 1 - i]
template <class T> __global__ void k_reverse_copy(int n, const T *in, T *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[n - 1 - i];
}

// reverse the rows (dim 0) or the columns (dim 1) of C (rows x cols) in place
template <class T> __global__ void k_flip(int dim, int rows, int cols, T *C, size_t ldc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (dim == 0) {
        if (r >= rows / 2) return;
        for (int c = blockIdx.y; c < cols; c += gridDim.y) {
            T &a = C[r + (size_t)c * ldc], &b = C[(rows - 1 - r) + (size_t)c * ldc];
            const T t = a;
            a = b;
            b = t;
        }
    } else {
        if (r >= rows) return;
        for (int c = blockIdx.y; c < cols / 2; c += gridDim.y) {
            T &a = C[r + (size_t)c * ldc], &b = C[r + (size_t)(cols - 1 - c) * ldc];
            const T t = a;
            a = b;
            b = t;
        }
    }
}

template <class T> int xform_launch(int kind, size_t rows, size_t cols, const T *src, size_t lds, T *dst, size_t ldd, cudaStream_t st) {
    if (rows == 0 || cols == 0) return kOk;
    const dim3 grid((unsigned)((rows + 31) / 32), (unsigned)std::min<size_t>((cols + 31) / 32, 65535));
    if ((cols + 31) / 32 > 65535) return kErrDevice;
    KScope ks("lqr_transform", st);
    k_xform<T><<<grid, 256, 0, st>>>(kind, (int)rows, (int)cols, src, lds, dst, ldd);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}
template <class T> int reverse_copy(size_t n, const T *in, T *out, cudaStream_t st) {
    if (n == 0) return kOk;
    k_reverse_copy<T><<<(unsigned)std::min<size_t>((n + 255) / 256, 1024), 256, 0, st>>>((int)n, in, out);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}
template <class T> int flip_launch(int dim, size_t rows, size_t cols, T *C, size_t ldc, cudaStream_t st) {
    if (rows == 0 || cols == 0) return kOk;
    const size_t r = dim == 0 ? rows / 2 : rows;
    if (r == 0) return kOk;
    const dim3 grid((unsigned)((r + 255) / 256), (unsigned)std::min<size_t>(dim == 0 ? cols : std::max<size_t>(cols / 2, 1), 4096));
    k_flip<T><<<grid, 256, 0, st>>>(dim, (int)rows, (int)cols, C, ldc);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

inline size_t xbytes(size_t elems, size_t esz) { return (elems * esz + 255) / 256 * 256; }

// ---------------------------------------------------------------------------
// Factor: LQ.hpp:127-184, QL.hpp:129-208, RQ.hpp:131-210 (the same argument
// list as QR::Factor).  lwork: the transformed copy plus the QR workspace.
// ---------------------------------------------------------------------------
template <class T> int xgeqrf(int kind, size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work) {
    if (lwork == nullptr) return -6;
    const size_t k = std::min(m, n);
    if (k == 0) return kOk;
    if (lda < std::max<size_t>(1, m)) return -4;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -1;
    const size_t mt = kind == kXQL ? m : n, nt = kind == kXQL ? n : m;
    size_t qf = 0;
    int rc = geqrf<T>(mt, nt, nullptr, mt, nullptr, &qf, nullptr);
    if (rc) return rc;
    const size_t bb = xbytes(mt * nt, sizeof(T)), tb = xbytes(k, sizeof(T));
    const size_t need = elems_for<T>(bb + tb) + qf;
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -3;
    if (tau == nullptr) return -5;
    if (*lwork < need) return -6;
    cudaStream_t st = current_stream();
    Carver cv(work);
    T *B = cv.take<T>(mt * nt);
    T *tq = cv.take<T>(k);
    T *wrest = cv.take<T>(0);
    size_t lw = *lwork - (size_t)(wrest - work);
    if ((rc = xform_launch<T>(kind, m, n, a, lda, B, mt, st))) return rc;
    if ((rc = geqrf<T>(mt, nt, B, mt, kind == kXLQ ? tau : tq, &lw, wrest))) return rc < 0 ? -6 : rc;
    if ((rc = xform_launch<T>(kind, mt, nt, B, mt, a, lda, st))) return rc;
    if (kind != kXLQ && (rc = reverse_copy<T>(k, tq, tau, st))) return rc;
    return kOk;
}

// ---------------------------------------------------------------------------
// MultQ: LQ.hpp:310-419, QL.hpp:337-437, RQ.hpp:344-449.  The reflectors:
// LQ and RQ k x nq (rows of a), QL nq x k (columns of a).
// ---------------------------------------------------------------------------
template <class T> int xunmqr(int kind, const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work) {
    if (lwork == nullptr) return -11;
    if (side == nullptr) return -1;
    if (trans == nullptr) return -2;
    const bool left = side[0] == 'L';
    const size_t nq = left ? m : n;
    if (m == 0 || n == 0 || k == 0) {
        if (work == nullptr || *lwork == 0) *lwork = 1;
        return kOk;
    }
    if (k > nq) return -5;
    if (lda < (kind == kXQL ? std::max<size_t>(1, nq) : std::max<size_t>(1, k))) return -7;
    if (ldc < std::max<size_t>(1, m)) return -10;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -3;
    const char *tr = (kind == kXQL) ? trans : (trans[0] == 'N' ? "C" : "N");
    size_t qm = 0;
    int rc = unmqr<T>(side, tr, m, n, k, nullptr, nq, nullptr, nullptr, m, &qm, nullptr);
    if (rc) return rc;
    const size_t bb = xbytes(nq * k, sizeof(T)), tb = xbytes(k, sizeof(T));
    const size_t need = elems_for<T>(bb + tb) + qm;
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -6;
    if (tau == nullptr) return -8;
    if (c == nullptr) return -9;
    if (*lwork < need) return -11;
    cudaStream_t st = current_stream();
    Carver cv(work);
    T *B = cv.take<T>(nq * k);
    T *tq = cv.take<T>(k);
    T *wrest = cv.take<T>(0);
    size_t lw = *lwork - (size_t)(wrest - work);
    // the reflector block, transformed to QR storage (nq x k)
    if (kind == kXQL) rc = xform_launch<T>(kind, nq, k, a, lda, B, nq, st);
    else rc = xform_launch<T>(kind, k, nq, a, lda, B, nq, st);
    if (rc) return rc;
    if (kind != kXLQ && (rc = reverse_copy<T>(k, tau, tq, st))) return rc;
    const int dim = left ? 0 : 1;
    if (kind != kXLQ && (rc = flip_launch<T>(dim, m, n, c, ldc, st))) return rc;
    if ((rc = unmqr<T>(side, tr, m, n, k, B, nq, kind == kXLQ ? tau : tq, c, ldc, &lw, wrest))) return rc < 0 ? -11 : rc;
    if (kind != kXLQ && (rc = flip_launch<T>(dim, m, n, c, ldc, st))) return rc;
    return kOk;
}

// ---------------------------------------------------------------------------
// GenerateQ: LQ.hpp:492-556 (m <= n), QL.hpp:501-566 (m >= n), RQ.hpp:519-586
// (m <= n); k reflectors.
// ---------------------------------------------------------------------------
template <class T> int xungqr(int kind, size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    if (lwork == nullptr) return -7;
    if (kind == kXQL ? (n > m) : (m > n)) return -2;
    if (k > std::min(m, n)) return -3;
    if (m == 0 || n == 0) {
        if (work == nullptr || *lwork == 0) *lwork = 1;
        return kOk;
    }
    if (lda < std::max<size_t>(1, m)) return -5;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -1;
    const size_t mt = kind == kXQL ? m : n, nt = kind == kXQL ? n : m;
    size_t qg = 0;
    int rc = ungqr<T>(mt, nt, k, nullptr, mt, nullptr, &qg, nullptr);
    if (rc) return rc;
    const size_t bb = xbytes(mt * nt, sizeof(T)), tb = xbytes(std::max<size_t>(k, 1), sizeof(T));
    const size_t need = elems_for<T>(bb + tb) + qg;
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -4;
    if (tau == nullptr && k > 0) return -6;
    if (*lwork < need) return -7;
    cudaStream_t st = current_stream();
    Carver cv(work);
    T *B = cv.take<T>(mt * nt);
    T *tq = cv.take<T>(std::max<size_t>(k, 1));
    T *wrest = cv.take<T>(0);
    size_t lw = *lwork - (size_t)(wrest - work);
    if ((rc = xform_launch<T>(kind, m, n, a, lda, B, mt, st))) return rc;
    if (kind != kXLQ && (rc = reverse_copy<T>(k, tau, tq, st))) return rc;
    if ((rc = ungqr<T>(mt, nt, k, B, mt, kind == kXLQ ? tau : tq, &lw, wrest))) return rc < 0 ? -7 : rc;
    return xform_launch<T>(kind, mt, nt, B, mt, a, lda, st);
}

} // namespace rnpgpu
