// ls_driver.cuh — least squares on the QR path.
//
//  gels<T>          min ||A x - b|| by Factor, MultQ("L","C") and the upper
//                   triangular solve, the composition a caller of the
//                   reference writes (RNP/LA/QR.hpp:129-197, 337-429;
//                   BLAS::SolveTrM, RNP/BLAS/BLAS_mix.hpp:2096-2113)
//  gels_refine<H,L> the mixed form: Factor in the low precision L (FP32),
//                   then refinement  x += R^{-1} Q^H (b - A x)  with the
//                   residual, the solution and the error metrics in H
//                   (FP64).  Loop shape and stop rule follow the reference's
//                   LU::RefineSolution (RNP/LA/LU.hpp:244-311): stop when the
//                   backward error is small enough or the correction stops
//                   halving, at most max_iter steps.
#pragma once
#include "ls_kernels.cuh"
#include "qr_driver.cuh"
#include "oz_gemm.cuh"
#include <cmath>
#include <vector>

namespace rnpgpu {

struct RefineInfo {
    int iterations;
    int converged;
    double backward_error;   // max_j ||R^{-H} A^H r_j|| / ||x_j||  (LS backward error bound)
    double normal_residual;  // max_j ||A^H r_j|| / (||A||_F (||A||_F ||x_j|| + ||b_j||))
    double correction;       // max_j ||d_j|| / ||x_j|| of the last step
    double anorm;            // ||A||_F
};

// dinv (optional, n <= kTrsmSmallMax): the inverted diagonal blocks of R
// (k_trinv_diag), formed once per factorization
template <class T> int trsm_upper(size_t n, size_t nrhs, const T *a, size_t lda, T *b, size_t ldb, cudaStream_t st, const T *dinv = nullptr) {
    if (n == 0 || nrhs == 0) return kOk;
    KScope ks("trsm", st);
    bool small = false;
    if constexpr (sizeof(T) <= 8) {
        if (n <= (size_t)kTrsmSmallMax) {
            k_trsm_small<T, false><<<(unsigned)std::min<size_t>(nrhs, 65535), 512, 0, st>>>((int)n, (int)nrhs, a, lda, b, ldb, dinv);
            small = true;
        }
    }
    if (!small) k_trsm_upper<T><<<(unsigned)std::min<size_t>(nrhs, 65535), 512, 0, st>>>((int)n, (int)nrhs, a, lda, b, ldb);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> int trsm_upper_ct(size_t n, size_t nrhs, const T *a, size_t lda, T *b, size_t ldb, cudaStream_t st, const T *dinv = nullptr) {
    if (n == 0 || nrhs == 0) return kOk;
    KScope ks("trsm", st);
    bool small = false;
    if constexpr (sizeof(T) <= 8) {
        if (n <= (size_t)kTrsmSmallMax) {
            k_trsm_small<T, true><<<(unsigned)std::min<size_t>(nrhs, 65535), 512, 0, st>>>((int)n, (int)nrhs, a, lda, b, ldb, dinv);
            small = true;
        }
    }
    if (!small) k_trsm_upper_ct<T><<<(unsigned)std::min<size_t>(nrhs, 65535), 512, 0, st>>>((int)n, (int)nrhs, a, lda, b, ldb);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> int trsm_lunn(size_t n, size_t nrhs, const T *a, size_t lda, T *b, size_t ldb) {
    if (n == 0 || nrhs == 0) return kOk;
    if (lda < n) return -4;
    if (ldb < n) return -6;
    if (a == nullptr) return -3;
    if (b == nullptr) return -5;
    if (n > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX) return -1;
    return trsm_upper<T>(n, nrhs, a, lda, b, ldb, current_stream());
}

// ---------------------------------------------------------------------------
// plain least squares
// ---------------------------------------------------------------------------
template <class T> size_t tstore_bytes(size_t n) { return ((n + GpuTuning::nb - 1) / GpuTuning::nb) * t_bytes<T>(); }

template <class T> size_t gels_bytes(size_t m, size_t n, size_t nrhs) {
    size_t f = geqrf_bytes<T>(m, n, smax_for<T>(m));
    size_t q = unmqr_bytes<T>(m, nrhs, n, smax_for<T>(m), smax_for<T>(m));
    return std::max(f, q) + tstore_bytes<T>(n) + 512;
}

template <class T> int gels(size_t m, size_t n, size_t nrhs, T *a, size_t lda, T *tau, T *b, size_t ldb, size_t *lwork, T *work) {
    if (lwork == nullptr) return -9;
    if (n > m) return -2;
    if (m == 0 || n == 0 || nrhs == 0) return kOk;
    if (lda < m) return -5;
    if (ldb < m) return -8;
    if (m > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX) return -1;
    const size_t need = elems_for<T>(gels_bytes<T>(m, n, nrhs));
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -4;
    if (tau == nullptr) return -6;
    if (b == nullptr) return -7;
    if (*lwork < need) return -9;
    // the T factors of the factorization are kept for MultQ
    Carver cv(work);
    T *Ts = cv.take<T>(tstore_bytes<T>(n) / sizeof(T));
    T *wrest = cv.take<T>(0);
    size_t lw = *lwork - (size_t)(wrest - work);
    int rc = geqrf<T>(m, n, a, lda, tau, &lw, wrest, Ts);
    if (rc) return rc < 0 ? -9 : rc;
    lw = *lwork - (size_t)(wrest - work);
    rc = unmqr<T>("L", "C", m, nrhs, n, a, lda, tau, b, ldb, &lw, wrest, Ts);
    if (rc) return rc < 0 ? -9 : rc;
    return trsm_upper<T>(n, nrhs, a, lda, b, ldb, current_stream());
}

// ---------------------------------------------------------------------------
// mixed precision least squares with iterative refinement
// ---------------------------------------------------------------------------
template <class TH, class TL> struct RefinePlan {
    size_t af, tauf, ts, wq, r, rf, p, g, norms, ozw, cqrw, widew, t128, dinv, total;
    int split;
    // the FP64 products r = b - A x and A^T r on the tensor cores (exact
    // integer slices) for real FP64 data; other types use FP64 FMA
    static constexpr bool kOz = std::is_same<TH, double>::value;
    RefinePlan(size_t m, size_t n, size_t nrhs) {
        auto al = [](size_t b) { return (b + 255) / 256 * 256; };
        af = al(m * n * sizeof(TL));
        tauf = al(n * sizeof(TL));
        ts = al(tstore_bytes<TL>(n));
        wq = al(std::max(geqrf_bytes<TL>(m, n, smax_for<TL>(m)), unmqr_bytes<TL>(m, nrhs, n, smax_for<TL>(m), smax_for<TL>(m))) + 256);
        r = al(m * nrhs * sizeof(TH));
        rf = al(m * nrhs * sizeof(TL));
        split = smax_for<TL>(m);
        p = al((size_t)split * n * nrhs * sizeof(TH));
        g = al(n * nrhs * sizeof(TH));
        norms = al((n + 6 * nrhs) * sizeof(double));
        rf = std::max(rf, al(n * nrhs * sizeof(TL)));
        ozw = kOz ? OzWork::bytes(m, n, nrhs) : 0;
        cqrw = std::is_same<TL, float>::value ? cqr_ws_bytes() : 0;
        widew = (std::is_same<TL, float>::value && wide::usable(m, n, reinterpret_cast<const float *>(256), m)) ? wide::ws_bytes(m, n) : 0;
        // the wide blocks' T factors, kept for the Q^T r steps
        t128 = widew > 0 ? al((n / wide::kNb) * wide::kNb * wide::kNb * sizeof(float)) : 0;
        if (widew > 0 && nrhs <= (size_t)kQtcMaxCols) wq = std::max(wq, al(qtc_ws_bytes(nrhs) + 256));
        // the inverted 32 x 32 diagonal blocks of R for the small triangular solves
        dinv = (sizeof(TL) <= 8 && n <= (size_t)kTrsmSmallMax) ? al((n + 31) / 32 * 1024 * sizeof(TL)) : 0;
        total = af + tauf + ts + wq + r + rf + p + g + norms + ozw + cqrw + widew + t128 + dinv;
    }
};

// Host staging of A (gels_refine_host): A's device copy arrives in ranges of
// kStageCols columns on a copy stream, ev_copy[c] recorded after range c.
constexpr int kStageCols = 128;
struct HostStage {
    cudaStream_t prep;        // converts each range to FP32 once it has landed
    cudaStream_t dig;         // (lower priority) the packed digits and norms of each range
    const cudaEvent_t *ev_copy;
    const cudaEvent_t *ev_prep;  // range c prepared (recorded by the staging)
    int nchunk;
    cudaEvent_t ev_all;       // every range prepared
    unsigned char *vcache;    // per-block V slice images of the left-looking factor (or null)
    size_t vstride;
};
// the left-looking factor's per-block V slice images (every 128-column block
// but the last)
inline size_t stage_vcache_stride(size_t m) { return wide::al256(wide::va_bytes((int)m)) + wide::al256(wide::vb_bytes((int)m)); }
inline size_t stage_vcache_bytes(size_t m, size_t n) {
    if (!wide::usable(m, n, reinterpret_cast<const float *>(256), m)) return 0;
    const size_t nblk = (n + wide::kNb - 1) / wide::kNb;
    return nblk > 1 ? (nblk - 1) * stage_vcache_stride(m) : 0;
}

template <class TH, class TL>
int gels_refine(size_t m, size_t n, size_t nrhs, const TH *a, size_t lda, const TH *b, size_t ldb, TH *x, size_t ldx, int max_iter, int flags, RefineInfo *info, size_t *lwork, TH *work,
                const HostStage *hs = nullptr) {
    if (lwork == nullptr) return -13;
    if (n > m) return -2;
    if (m == 0 || n == 0 || nrhs == 0) return kOk;
    if (lda < m) return -5;
    if (ldb < m) return -7;
    if (ldx < n) return -9;
    if (m > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX) return -1;
    RefinePlan<TH, TL> plan(m, n, nrhs);
    const size_t need = elems_for<TH>(plan.total);
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -4;
    if (b == nullptr) return -6;
    if (x == nullptr) return -8;
    if (*lwork < need) return -13;
    const bool forward = (flags & 1) != 0;
    if (max_iter <= 0) max_iter = forward ? 30 : 10;
    cudaStream_t st = current_stream();
    Carver cv(work);
    TL *Af = cv.take<TL>(plan.af / sizeof(TL));
    TL *tauf = cv.take<TL>(plan.tauf / sizeof(TL));
    TL *Tf = cv.take<TL>(plan.ts / sizeof(TL));
    TL *wq = cv.take<TL>(plan.wq / sizeof(TL));
    TH *r = cv.take<TH>(plan.r / sizeof(TH));
    TL *rf = cv.take<TL>(plan.rf / sizeof(TL));
    TH *P = cv.take<TH>(plan.p / sizeof(TH));
    TH *g = cv.take<TH>(plan.g / sizeof(TH));
    double *dn = cv.take<double>(plan.norms / sizeof(double));
    constexpr bool use_oz = RefinePlan<TH, TL>::kOz;
    OzWork ow{};
    if (use_oz) ow.carve(cv, m, n, nrhs);
    CqrWs cw;
    if (std::is_same<TL, float>::value) cw = carve_cqr(cv);
    if (plan.widew > 0) {
        cw.wide = wide::carve(cv, m, n);
        cw.use_wide = (flags & 2) == 0;  // flag 2: rank-32 trailing updates only
        if (plan.t128 > 0) cw.t128 = cv.take<float>(plan.t128 / sizeof(float));
    }
    TL *dinv = plan.dinv > 0 ? cv.take<TL>(plan.dinv / sizeof(TL)) : nullptr;
    const size_t lwq = plan.wq / sizeof(TL);
    const dim3 gmn((unsigned)std::min<size_t>((m + 255) / 256, 2048), (unsigned)std::min<size_t>(n, 65535));
    const dim3 gmr((unsigned)std::min<size_t>((m + 255) / 256, 2048), (unsigned)std::min<size_t>(nrhs, 65535));
    const dim3 gnr((unsigned)std::min<size_t>((n + 255) / 256, 2048), (unsigned)std::min<size_t>(nrhs, 65535));
    const unsigned cb = (unsigned)std::min<size_t>(std::max(n, nrhs), 4096);
    int rc;

    // low-precision working copy and its factorization (for real FP64 data the
    // same pass writes the packed digits of A for the residual products)
    if constexpr (use_oz) {
        KScope ks("prepare_digits", st);
        if (hs != nullptr) {
            // A arrives range by range: each range is prepared on the staging
            // stream once its copy has landed; the factor starts after the
            // first range and waits for the rest before it updates columns
            // past its first block
            // the factor needs only the FP32 copy of a range: it is made first,
            // on its own stream; the digits of the residual products and the
            // column norms follow on a lower-priority stream, done long before
            // the refinement reads them
            for (int c = 0; c < hs->nchunk; ++c) {
                const int c0 = c * kStageCols, w = (int)std::min<size_t>(kStageCols, n - (size_t)c0);
                RNPGPU_CHECK(cudaStreamWaitEvent(hs->prep, hs->ev_copy[c], 0));
                k_convert<TH, TL><<<dim3((unsigned)std::min<size_t>((m + 255) / 256, 2048), (unsigned)w), 256, 0, hs->prep>>>((int)m, w, a + (size_t)c0 * lda, lda,
                                                                                                                    Af + (size_t)c0 * m, m);
                RNPGPU_CHECK_LAUNCH();
                RNPGPU_CHECK(cudaEventRecord(hs->ev_prep[c], hs->prep));
                RNPGPU_CHECK(cudaStreamWaitEvent(hs->dig, hs->ev_prep[c], 0));
                if ((rc = oz_prepare_cols((int)m, (int)n, c0, w, a, lda, ow, nullptr, nullptr, m, hs->dig))) return rc;
                oz::k_col_sumsq_f32<0><<<(unsigned)std::min(w, 8192), 256, 0, hs->dig>>>((int)m, w, Af + (size_t)c0 * m, m, dn + c0);
                RNPGPU_CHECK_LAUNCH();
            }
            RNPGPU_CHECK(cudaEventRecord(hs->ev_all, hs->dig));
            RNPGPU_CHECK(cudaStreamWaitEvent(st, hs->ev_prep[0], 0));
            if constexpr (std::is_same<TL, float>::value) {
                cw.range_ready = hs->ev_prep;
                cw.nranges = hs->nchunk;
                cw.vcache = hs->vcache;
                cw.vcache_stride = hs->vstride;
            } else {
                RNPGPU_CHECK(cudaStreamWaitEvent(st, hs->ev_all, 0));
            }
        } else {
            if ((rc = oz_prepare_a((int)m, (int)n, a, lda, ow, dn, Af, m, st))) return rc;
        }
    } else {
        k_convert<TH, TL><<<gmn, 256, 0, st>>>((int)m, (int)n, a, lda, Af, m);
        RNPGPU_CHECK_LAUNCH();
    }
    size_t lw = lwq;
    std::vector<double> h(n + 6 * nrhs);
    if constexpr (!use_oz) {
        k_col_sumsq<TH><<<cb, 256, 0, st>>>((int)m, (int)n, a, lda, dn);
        RNPGPU_CHECK_LAUNCH();
    }
    k_col_sumsq<TH><<<cb, 256, 0, st>>>((int)m, (int)nrhs, b, ldb, dn + n);
    RNPGPU_CHECK_LAUNCH();
    if constexpr (std::is_same<TL, float>::value) {
        // FP32 factor with CholeskyQR2 panels; a panel whose Gram matrix is
        // too ill-conditioned for them sends the whole factorization back to
        // Householder panels
        RNPGPU_CHECK(cudaMemsetAsync(cw.fail, 0, sizeof(int), st));
        if ((rc = geqrf<TL>(m, n, Af, m, tauf, &lw, wq, Tf, &cw))) return rc < 0 ? -13 : rc;
        // everything after (the flag, a refactorization, the residuals) reads
        // all of A's preparation
        if (hs != nullptr) RNPGPU_CHECK(cudaStreamWaitEvent(st, hs->ev_all, 0));
        int failed = 0;
        RNPGPU_CHECK(cudaMemcpyAsync(&failed, cw.fail, sizeof(int), cudaMemcpyDeviceToHost, st));
        RNPGPU_CHECK(cudaStreamSynchronize(st));
        if (failed) {
            cw.nwide = 0;  // the Householder refactorization keeps no wide T's
            k_convert<TH, TL><<<gmn, 256, 0, st>>>((int)m, (int)n, a, lda, Af, m);
            RNPGPU_CHECK_LAUNCH();
            lw = lwq;
            if ((rc = geqrf<TL>(m, n, Af, m, tauf, &lw, wq, Tf))) return rc < 0 ? -13 : rc;
        }
    } else {
        if ((rc = geqrf<TL>(m, n, Af, m, tauf, &lw, wq, Tf))) return rc < 0 ? -13 : rc;
    }
    if (hs != nullptr) RNPGPU_CHECK(cudaStreamWaitEvent(st, hs->ev_all, 0));
    if (dinv) {
        k_trinv_diag<TL><<<(unsigned)((n + 31) / 32), 32, 0, st>>>((int)n, Af, m, dinv);
        RNPGPU_CHECK_LAUNCH();
    }

    // ||A||_F (real FP64 data: from the FP32 working copy, which only scales
    // the stopping test) and ||b_j|| in FP64: computed before the factor, read
    // back after it (one wait for the factor's flag and the norms)
    RNPGPU_CHECK(cudaMemcpyAsync(h.data(), dn, (n + nrhs) * sizeof(double), cudaMemcpyDeviceToHost, st));
    RNPGPU_CHECK(cudaStreamSynchronize(st));
    double asq = 0.0;
    for (size_t j = 0; j < n; ++j) asq += h[j];
    const double anorm = std::sqrt(asq);
    std::vector<double> bn(nrhs);
    for (size_t j = 0; j < nrhs; ++j) bn[j] = std::sqrt(h[n + j]);

    // x = 0, r = b
    RNPGPU_CHECK(cudaMemset2DAsync(x, ldx * sizeof(TH), 0, n * sizeof(TH), nrhs, st));
    RNPGPU_CHECK(cudaMemcpy2DAsync(r, m * sizeof(TH), b, ldb * sizeof(TH), m * sizeof(TH), nrhs, cudaMemcpyDeviceToDevice, st));

    const double eps = 0x1p-52;
    const double tol = 10.0 * (double)n * eps;  // 10 n eps
    TL *gf = rf;                                // n x nrhs low-precision copy of A^H r
    auto correction_size = [&](double &corr_out) -> int {
        RNPGPU_CHECK(cudaMemcpyAsync(h.data() + n + nrhs, dn + n + nrhs, 2 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
        RNPGPU_CHECK(cudaStreamSynchronize(st));
        corr_out = 0.0;
        for (size_t j = 0; j < nrhs; ++j) {
            double xs = h[n + 2 * nrhs + j], ds = h[n + nrhs + j];
            // a non-finite x or correction (Inf or NaN in A or b, or a
            // broken-down factor) makes the size NaN, which ends the steps
            if (!std::isfinite(xs) || !std::isfinite(ds)) {
                corr_out = std::nan("");
                return kOk;
            }
            corr_out = std::max(corr_out, xs > 0.0 ? std::sqrt(ds / xs) : (ds > 0.0 ? HUGE_VAL : 0.0));
        }
        return kOk;
    };
    // g = A^H r (FP64); y = R_f^{-H} g (low precision, in gf);
    // eta = max_j ||g_j|| / (||A||_F (||A||_F ||x_j|| + ||b_j||)),
    // mu  = max_j ||y_j|| / ||x_j||   (an upper bound of the Karlson-Walden
    //                                   estimate of the LS backward error)
    double eta = HUGE_VAL, mu = HUGE_VAL;
    auto check = [&]() -> int {
        int rc2;
        if constexpr (use_oz) {
            if ((rc2 = oz_normal((int)m, (int)n, (int)nrhs, ow, r, m, g, n, st))) return rc2;
        } else {
            const int S = choose_splits((int)m, ((int)n + 127) / 128, plan.split);
            const int kchunk = (((int)m + S - 1) / S + 15) / 16 * 16;
            const int nsplit = ((int)m + kchunk - 1) / kchunk;
            GemmArgs<TH> ga = gemm_args<TH>(a, lda, kOpC, 0, r, m, kOpN, 0, P, n, (int)n, (int)nrhs, (int)m, TH(1), kBetaZero);
            ga.kchunk = kchunk;
            ga.dstride = n * nrhs;
            if ((rc2 = launch_gemm(ga, nsplit, st, "normal_eq_fp64"))) return rc2;
            k_sum_partials<TH><<<gnr, 256, 0, st>>>(P, n, n * nrhs, nsplit, (int)n, (int)nrhs, g, n);
            RNPGPU_CHECK_LAUNCH();
        }
        k_col_sumsq<TH><<<(unsigned)std::min<size_t>(nrhs, 4096), 256, 0, st>>>((int)n, (int)nrhs, g, n, dn + n + 3 * nrhs);
        RNPGPU_CHECK_LAUNCH();
        k_convert<TH, TL><<<gnr, 256, 0, st>>>((int)n, (int)nrhs, g, n, gf, n);
        RNPGPU_CHECK_LAUNCH();
        if ((rc2 = trsm_upper_ct<TL>(n, nrhs, Af, m, gf, n, st, dinv))) return rc2;
        k_col_sumsq<TL><<<(unsigned)std::min<size_t>(nrhs, 4096), 256, 0, st>>>((int)n, (int)nrhs, gf, n, dn + n + 4 * nrhs);
        RNPGPU_CHECK_LAUNCH();
        RNPGPU_CHECK(cudaMemcpyAsync(h.data() + n + 3 * nrhs, dn + n + 3 * nrhs, 2 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
        RNPGPU_CHECK(cudaStreamSynchronize(st));
        eta = 0.0;
        mu = 0.0;
        bool finite = std::isfinite(anorm);
        for (size_t j = 0; j < nrhs; ++j) {
            const double xn = std::sqrt(h[n + 2 * nrhs + j]);
            const double den = anorm * (anorm * xn + bn[j]);
            const double gn = std::sqrt(h[n + 3 * nrhs + j]), yn = std::sqrt(h[n + 4 * nrhs + j]);
            finite = finite && std::isfinite(xn) && std::isfinite(bn[j]) && std::isfinite(gn) && std::isfinite(yn);
            eta = std::max(eta, den > 0.0 ? gn / den : 0.0);
            mu = std::max(mu, xn > 0.0 ? yn / xn : 0.0);
        }
        // non-finite data never passes the stopping test (std::max would
        // drop a NaN)
        if (!finite) eta = mu = std::nan("");
        return kOk;
    };

    // Steps: "Q" steps d = R^{-1} (Q^H r)(0:n) until the LS backward error
    // bound mu reaches 10 n eps; in forward mode then "CSNE" steps
    // d = R^{-1} R^{-H} A^H r (corrected seminormal equations, whose fixed
    // point satisfies A^H r = 0 exactly) until the correction stops shrinking.
    bool csne = false, checked = false;
    double prev_corr = HUGE_VAL, corr = 0.0;
    int it = 0, converged = 0;
    for (it = 0; it < max_iter;) {
        if (!csne) {
            k_convert<TH, TL><<<gmr, 256, 0, st>>>((int)m, (int)nrhs, r, m, rf, m);
            RNPGPU_CHECK_LAUNCH();
            lw = lwq;
            bool done = false;
            if constexpr (std::is_same<TL, float>::value) {
                // Q^T r with the wide blocks' T's: 2 grid barriers per
                // 128-column block instead of per 32-column panel
                if (qtc_usable(m, nrhs, n, Af, m, cw.nwide) && lwq * sizeof(TL) >= qtc_ws_bytes(nrhs)) {
                    if ((rc = qtc_blocks(m, nrhs, n, Af, m, Tf, cw.t128, cw.nwide, rf, m, wq, st))) return rc;
                    done = true;
                }
            }
            if (!done && (rc = unmqr<TL>("L", "C", m, nrhs, n, Af, m, tauf, rf, m, &lw, wq, Tf))) return rc < 0 ? -13 : rc;
            if ((rc = trsm_upper<TL>(n, nrhs, Af, m, rf, m, st, dinv))) return rc;
        } else {
            // gf already holds R^{-H} A^H r from the last check
            if ((rc = trsm_upper<TL>(n, nrhs, Af, m, gf, n, st, dinv))) return rc;
        }
        const size_t ldd = csne ? n : m;
        k_add_correction<TL, TH><<<gnr, 256, 0, st>>>((int)n, (int)nrhs, rf, ldd, x, ldx);
        RNPGPU_CHECK_LAUNCH();
        k_col_sumsq<TL><<<(unsigned)std::min<size_t>(nrhs, 4096), 256, 0, st>>>((int)n, (int)nrhs, rf, ldd, dn + n + nrhs);
        RNPGPU_CHECK_LAUNCH();
        k_col_sumsq<TH><<<(unsigned)std::min<size_t>(nrhs, 4096), 256, 0, st>>>((int)n, (int)nrhs, x, ldx, dn + n + 2 * nrhs);
        RNPGPU_CHECK_LAUNCH();
        // r = b - A x in FP64
        if constexpr (use_oz) {
            if ((rc = oz_residual((int)m, (int)n, (int)nrhs, ow, x, ldx, b, ldb, r, m, st))) return rc;
        } else {
            RNPGPU_CHECK(cudaMemcpy2DAsync(r, m * sizeof(TH), b, ldb * sizeof(TH), m * sizeof(TH), nrhs, cudaMemcpyDeviceToDevice, st));
            GemmArgs<TH> gr = gemm_args<TH>(a, lda, kOpN, 0, x, ldx, kOpN, 0, r, m, (int)m, (int)nrhs, (int)n, TH(-1), kBetaOne);
            if ((rc = launch_gemm(gr, 1, st, "residual_fp64"))) return rc;
        }
        ++it;
        if (it == 1 && max_iter > 1) {
            // from x = 0 the first correction is x itself (size 1): nothing
            // to decide yet, so no read-back (and no host wait) here
            prev_corr = corr = 1.0;
            continue;
        }
        if ((rc = correction_size(corr))) return rc;
        if (std::isnan(corr)) {
            if ((rc = check())) return rc;
            checked = true;
            converged = 0;
            break;
        }
        // Q steps contract fast, so failing to halve means they have stalled;
        // CSNE steps contract more slowly and count as stalled only when the
        // correction no longer shrinks noticeably
        const bool stagnated = (it >= 2 && corr > (csne ? 0.9 : 0.5) * prev_corr);
        const bool last = (it == max_iter);
        prev_corr = corr;
        checked = false;
        if (corr <= 1e-5 || stagnated || last || csne) {
            if ((rc = check())) return rc;
            checked = true;
            const bool backward_ok = (mu <= tol) && (eta <= tol);
            converged = backward_ok ? 1 : 0;
            if (last) break;
            if (!csne) {
                // Q steps converge to the point where Q_f^H r = 0 for the FP32
                // factor's Q_f; when that stalls above the bound (or forward
                // accuracy is asked for) switch to the CSNE steps, whose
                // fixed point is the least-squares solution itself.
                if (backward_ok && !forward) break;
                if (backward_ok || stagnated) {
                    csne = true;
                    prev_corr = HUGE_VAL;
                }
            } else {
                if (backward_ok && !forward) break;
                if (stagnated || corr <= 2.0 * eps) break;
            }
        }
    }
    if (!checked && (rc = check())) return rc;
    if (info) {
        info->iterations = it;
        info->converged = converged;
        info->backward_error = mu;
        info->normal_residual = eta;
        info->correction = corr;
        info->anorm = anorm;
    }
    return kOk;
}


// ---------------------------------------------------------------------------
// The mixed solve from host buffers (real FP64 data): A is copied to the
// device in ranges of kStageCols columns on a copy stream while the ranges
// already landed are prepared and the factor's first block runs; b, then the
// solution x, travel on the caller's stream.  Pinned host buffers let the
// copies run asynchronously (pageable ones still give the same result).
// Workspace: A, b and x on the device, then gels_refine's.
// ---------------------------------------------------------------------------
struct StageCtx {
    cudaStream_t copy = nullptr, prep = nullptr, dig = nullptr;
    cudaEvent_t ev_start = nullptr, ev_all = nullptr;
    std::vector<cudaEvent_t> ev_copy, ev_prep;
};
inline StageCtx *stage_ctx(int nchunk) {
    constexpr int kMaxDev = 16;
    static thread_local StageCtx ctx[kMaxDev];
    static thread_local int state[kMaxDev] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
    StageCtx &c = ctx[dev];
    if (state[dev] == 0) {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
            cudaGetLastError();
            least = greatest = 0;
        }
        const bool ok = cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking) == cudaSuccess && cudaStreamCreateWithFlags(&c.prep, cudaStreamNonBlocking) == cudaSuccess &&
                        cudaStreamCreateWithPriority(&c.dig, cudaStreamNonBlocking, least) == cudaSuccess &&
                        cudaEventCreateWithFlags(&c.ev_start, cudaEventDisableTiming) == cudaSuccess && cudaEventCreateWithFlags(&c.ev_all, cudaEventDisableTiming) == cudaSuccess;
        state[dev] = ok ? 1 : 2;
        if (!ok) cudaGetLastError();
    }
    if (state[dev] != 1) return nullptr;
    for (std::vector<cudaEvent_t> *v : {&c.ev_copy, &c.ev_prep}) {
        while ((int)v->size() < nchunk) {
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            v->push_back(e);
        }
    }
    return &c;
}

template <class TH, class TL>
int gels_refine_host(size_t m, size_t n, size_t nrhs, const TH *a, size_t lda, const TH *b, size_t ldb, TH *x, size_t ldx, int max_iter, int flags, RefineInfo *info, size_t *lwork,
                     TH *work) {
    if (lwork == nullptr) return -13;
    if (n > m) return -2;
    if (m == 0 || n == 0 || nrhs == 0) return kOk;
    if (lda < m) return -5;
    if (ldb < m) return -7;
    if (ldx < n) return -9;
    if (m > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX) return -1;
    auto al = [](size_t bytes) { return (bytes + 255) / 256 * 256; };
    const size_t da = al(m * n * sizeof(TH)), db = al(m * nrhs * sizeof(TH)), dx = al(n * nrhs * sizeof(TH));
    const size_t dvc = std::is_same<TL, float>::value ? al(stage_vcache_bytes(m, n)) : 0;
    size_t inner = 0;
    int rc = gels_refine<TH, TL>(m, n, nrhs, nullptr, m, nullptr, m, nullptr, n, max_iter, flags, nullptr, &inner, nullptr);
    if (rc) return rc;
    const size_t need = elems_for<TH>(da + db + dx + dvc) + inner;
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (a == nullptr) return -4;
    if (b == nullptr) return -6;
    if (x == nullptr) return -8;
    if (*lwork < need) return -13;
    const int nchunk = (int)((n + kStageCols - 1) / kStageCols);
    StageCtx *sc = stage_ctx(nchunk);
    if (sc == nullptr) return kErrCuda;
    cudaStream_t st = current_stream();
    Carver cv(work);
    TH *dA = cv.take<TH>(da / sizeof(TH));
    TH *dB = cv.take<TH>(db / sizeof(TH));
    TH *dX = cv.take<TH>(dx / sizeof(TH));
    unsigned char *vcache = dvc ? cv.take<unsigned char>(dvc) : nullptr;
    TH *wrest = cv.take<TH>(0);
    size_t lw = *lwork - (size_t)(wrest - work);
    // the staging streams start after the caller's earlier work on this
    // workspace
    RNPGPU_CHECK(cudaEventRecord(sc->ev_start, st));
    RNPGPU_CHECK(cudaStreamWaitEvent(sc->copy, sc->ev_start, 0));
    RNPGPU_CHECK(cudaStreamWaitEvent(sc->prep, sc->ev_start, 0));
    RNPGPU_CHECK(cudaStreamWaitEvent(sc->dig, sc->ev_start, 0));
    RNPGPU_CHECK(cudaMemcpy2DAsync(dB, m * sizeof(TH), b, ldb * sizeof(TH), m * sizeof(TH), nrhs, cudaMemcpyHostToDevice, st));
    for (int c = 0; c < nchunk; ++c) {
        const size_t c0 = (size_t)c * kStageCols, w = std::min<size_t>(kStageCols, n - c0);
        RNPGPU_CHECK(cudaMemcpy2DAsync(dA + c0 * m, m * sizeof(TH), a + c0 * lda, lda * sizeof(TH), m * sizeof(TH), w, cudaMemcpyHostToDevice, sc->copy));
        RNPGPU_CHECK(cudaEventRecord(sc->ev_copy[c], sc->copy));
    }
    HostStage hs{sc->prep, sc->dig, sc->ev_copy.data(), sc->ev_prep.data(), nchunk, sc->ev_all, vcache, stage_vcache_stride(m)};
    rc = gels_refine<TH, TL>(m, n, nrhs, dA, m, dB, m, dX, n, max_iter, flags, info, &lw, wrest, &hs);
    // the caller's stream also waits for every copy (a failed call may have
    // returned before it waited for them)
    RNPGPU_CHECK(cudaEventRecord(sc->ev_start, sc->copy));
    RNPGPU_CHECK(cudaStreamWaitEvent(st, sc->ev_start, 0));
    RNPGPU_CHECK(cudaEventRecord(sc->ev_start, sc->prep));
    RNPGPU_CHECK(cudaStreamWaitEvent(st, sc->ev_start, 0));
    RNPGPU_CHECK(cudaEventRecord(sc->ev_start, sc->dig));
    RNPGPU_CHECK(cudaStreamWaitEvent(st, sc->ev_start, 0));
    if (rc) return rc;
    RNPGPU_CHECK(cudaMemcpy2DAsync(x, ldx * sizeof(TH), dX, n * sizeof(TH), n * sizeof(TH), nrhs, cudaMemcpyDeviceToHost, st));
    return kOk;
}

} // namespace rnpgpu
