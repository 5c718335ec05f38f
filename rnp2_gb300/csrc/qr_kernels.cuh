// qr_kernels.cuh — device kernels of the blocked Householder QR path.
//
//   k_panel        panel factorization (geqr2 on an M x ib panel) across a
//                  cooperative grid, reflector generation with safe-scaled
//                  norms (RNP/LA/Reflector.hpp:117-158, Generate), the
//                  in-panel applications (Reflector.hpp:191-236, Apply) and
//                  the compact-WY T factor (Reflector.hpp:580-626,
//                  GenerateBlockTr "F","C"), all in one launch
//   k_gemm         tiled contraction  D = alpha*op(A)*op(B) (+ D | + I),
//                  split-K capable; every step of ApplyBlock
//                  (Reflector.hpp:725-815) and the Gram matrix of
//                  GenerateBlockTr is one call of it
//   k_sum_times_t  W = (sum of split-K partials) * op(T)
//   k_build_t      T recurrence from a Gram matrix and tau
//   k_larfg / k_larf_*   level-2 kernels for the *_unblocked entry points
#pragma once
#include <cooperative_groups.h>
#include "rnp_common.cuh"

namespace rnpgpu {

constexpr int kPanelMaxCols = 32;
constexpr int kPanelThreads = 512;
constexpr int kBuildTThreads = 256;
constexpr int kBuildTWarps = 4;  // warps of k_build_t's recurrence

template <class T> __device__ __forceinline__ T ldcg(const T *p) { return *(volatile const T *)p; }
__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ cf64 ldcg(const cf64 *p) { double2 v = __ldcg((const double2 *)p); return cf64(v.x, v.y); }
__device__ __forceinline__ cf32 ldcg(const cf32 *p) { float2 v = __ldcg((const float2 *)p); return cf32(v.x, v.y); }

template <class T> __device__ __forceinline__ T tzero() { return T(0); }
template <class T> __device__ __forceinline__ T tone() { return T(1); }

// ---------------------------------------------------------------------------
// Reflector scalars from (alpha, ||x||):  beta = -sign(Re alpha)*||[alpha;x]||,
// tau = (beta-alpha)/beta, scal = 1/(alpha-beta), including the safmin
// rescaling of Reflector.hpp:133-148.  Computed in FP64 for every type.
// ---------------------------------------------------------------------------
template <class T> struct ReflScalars {
    T tau, scal;      // scal multiplies x after 'knt' multiplications by rsafmn
    double sr, si;    // scal in FP64
    float sr_hi, sr_lo, si_hi, si_lo;  // FP32 forms: scal = (hi + lo) * 2^sh
    int sh;
    double beta;      // final beta (already scaled back)
    int knt;
    bool identity;    // tau == 0: H = I, x and alpha untouched
};

// FP32 hi/lo parts of the FP64 scale factor, with a power-of-two shift when
// its magnitude leaves [2^-100, 2^100] (columns of extreme magnitude), so
// that neither part overflows or loses bits in the FP32 range
template <class T> __device__ __forceinline__ void set_f32_scale(ReflScalars<T> &s, double sr, double si) {
    const double mx = fmax(fabs(sr), fabs(si));
    int e = 0;
    if (mx > 0x1p100 || (mx < 0x1p-100 && mx > 0.0)) {
        frexp(mx, &e);
        sr = ldexp(sr, -e);
        si = ldexp(si, -e);
    }
    s.sh = e;
    s.sr_hi = (float)sr;
    s.sr_lo = (float)(sr - (double)s.sr_hi);
    s.si_hi = (float)si;
    s.si_lo = (float)(si - (double)s.si_hi);
}

// FP64 reciprocal square root and reciprocal by Newton-Raphson iteration
// from the FP32 hardware approximations (y <- y (3 - x y^2) / 2 and
// y <- y (2 - d y), two steps each: the seed's 2^-22 relative error squares
// twice), and the square root s = x y with one Newton correction
// s <- s + y (x - s^2) / 2 (Markstein, "Computation of elementary functions
// on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).
// On this GPU a dependent FP64 operation takes about 64 cycles and a
// division or square root about 600, so these short chains shorten the
// reflector's serial path.  x and d must lie in the normal FP32 range.
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y = (double)rsqrtf((float)x);
    const double h = 0.5 * x;
    y = fma(y, fma(-h * y, y, 0.5), y);
    y = fma(y, fma(-h * y, y, 0.5), y);
    return y;
}
__device__ __forceinline__ double sqrt_from_rsqrt(double x, double y) {
    const double s = x * y;
    return fma(fma(-s, s, x), 0.5 * y, s);
}
__device__ __forceinline__ double rcp_nr(double d) {
    double y = (double)__frcp_rn((float)d);
    y = fma(y, fma(-d, y, 1.0), y);
    y = fma(y, fma(-d, y, 1.0), y);
    return y;
}

template <class T> __device__ ReflScalars<T> reflector_scalars(T alpha, const NormAcc &nacc) {
    typedef typename Tr<T>::R R;
    ReflScalars<T> s;
    double ar = (double)Tr<T>::re(alpha), ai = (double)Tr<T>::im(alpha);
    s.knt = 0;
    if (sizeof(R) == 8 && nacc.sml == 0.0 && nacc.big == 0.0) {
        // FP64 data, squared norm of x in med: when |alpha|^2 + ||x||^2 lies
        // well inside the FP32 range the scalars come from the short
        // Newton chains (no rescaling can be needed there)
        const double q = fma(ar, ar, fma(ai, ai, nacc.med));
        if (q >= 0x1p-120 && q <= 0x1p120 && (nacc.med > 0.0 || ai != 0.0)) {
            const double y = rsqrt_nr(q);
            const double sq = sqrt_from_rsqrt(q, y);
            const double beta = ar > 0.0 ? -sq : sq, invb = ar > 0.0 ? -y : y;
            const double d = ar - beta;  // |d| = |ar| + |beta|: no cancellation
            double tr, ti = 0.0, sr, si = 0.0;
            tr = fma(-ar, invb, 1.0);
            if (Tr<T>::is_complex) {
                ti = -ai * invb;
                const double inv = rcp_nr(fma(d, d, ai * ai));
                sr = d * inv;
                si = -ai * inv;
            } else {
                sr = rcp_nr(d);
            }
            s.identity = false;
            s.tau = Tr<T>::make((R)tr, (R)ti);
            s.scal = Tr<T>::make((R)sr, (R)si);
            s.sr = sr;
            s.si = si;
            s.sr_hi = 0.0f; s.sr_lo = 0.0f; s.si_hi = 0.0f; s.si_lo = 0.0f;
            s.sh = 0;
            s.beta = beta;
            return s;
        }
    }
    const double xnorm = nacc.result();
    if (xnorm == 0.0 && ai == 0.0) {
        s.identity = true;
        s.tau = T(0);
        s.scal = T(1);
        s.sr = 1.0;
        s.si = 0.0;
        s.sr_hi = 1.0f; s.sr_lo = 0.0f; s.si_hi = 0.0f; s.si_lo = 0.0f;
        s.sh = 0;
        s.beta = ar;
        return s;
    }
    s.identity = false;
    double beta = hypot3(ar, ai, xnorm);
    if (ar > 0.0) beta = -beta;
    // The FP32 forms carry beta in FP64, where FP32 magnitudes never reach the
    // safmin region; the rescaling only ever triggers for FP64 data.
    const bool is64 = sizeof(R) == 8;
    if (is64) {
        const double safmin = 0x1p-1022 / (2.0 * 0x1p-52);
        const double rsafmn = 1.0 / safmin;
        if (fabs(beta) < safmin) {
            // as the reference, rescale x and alpha by 1/safmin until beta is
            // representable accurately; the norm of the rescaled x comes from
            // the accumulators scaled by the same power of two
            double mult = 1.0;
            do {
                ++s.knt;
                beta *= rsafmn;
                ar *= rsafmn;
                ai *= rsafmn;
                mult *= rsafmn;
            } while (fabs(beta) < safmin && s.knt < 1);
            const double xn = nacc.result_scaled(mult);
            beta = hypot3(ar, ai, xn);
            if (ar > 0.0) beta = -beta;
        }
    }
    double tr, ti = 0.0, sr, si;
    if (Tr<T>::is_complex) {
        const double rb = 1.0 / beta;
        tr = (beta - ar) * rb;
        ti = -ai * rb;
        crecip(ar - beta, ai, sr, si);
    } else {
        tr = (beta - ar) / beta;
        sr = 1.0 / (ar - beta);
        si = 0.0;
    }
    s.tau = Tr<T>::make((R)tr, (R)ti);
    s.scal = Tr<T>::make((R)sr, (R)si);
    s.sr = sr;
    s.si = si;
    set_f32_scale(s, sr, si);
    if (s.knt) {
        const double safmin = 0x1p-1022 / (2.0 * 0x1p-52);
        for (int q = 0; q < s.knt; ++q) beta *= safmin;
    }
    s.beta = beta;
    return s;
}

template <class T> __device__ __forceinline__ T scale_x(T x, const ReflScalars<T> &s) {
    typedef typename Tr<T>::R R;
    if (sizeof(R) == 8) {
        for (int q = 0; q < s.knt; ++q) x = x * (R)(1.0 / (0x1p-1022 / (2.0 * 0x1p-52)));
        return x * s.scal;
    }
    return x * s.scal;
}
// FP32 types: v = x/(alpha-beta) with the FP64 scale factor applied as an
// FP32 hi + lo pair (FP32 pipe; within an ulp of the FP64 product rounded),
// then the power-of-two shift in two exact steps
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }  // |e| <= 126
__device__ __forceinline__ float shift_f32(float v, int sh) {
    if (sh == 0) return v;
    const int h = sh / 2;
    return (v * pow2f(h)) * pow2f(sh - h);
}
// (an upward shift goes first, so that tiny x are scaled out of the
// subnormal range before the product; a downward one last)
__device__ __forceinline__ float scale_x(float x, const ReflScalars<float> &s) {
    if (s.sh > 0) x = shift_f32(x, s.sh);
    const float v = fmaf(x, s.sr_lo, x * s.sr_hi);
    return s.sh < 0 ? shift_f32(v, s.sh) : v;
}
__device__ __forceinline__ cf32 scale_x(cf32 x, const ReflScalars<cf32> &s) {
    if (s.sh > 0) x = cf32(shift_f32(x.x, s.sh), shift_f32(x.y, s.sh));
    const float re = fmaf(x.x, s.sr_lo, x.x * s.sr_hi) - fmaf(x.y, s.si_lo, x.y * s.si_hi);
    const float im = fmaf(x.x, s.si_lo, x.x * s.si_hi) + fmaf(x.y, s.sr_lo, x.y * s.sr_hi);
    return s.sh < 0 ? cf32(shift_f32(re, s.sh), shift_f32(im, s.sh)) : cf32(re, im);
}

// ---------------------------------------------------------------------------
// Panel factorization across a cooperative grid.
// Rows [b*R, min(M,(b+1)*R)) of the panel belong to block b.  One grid
// barrier per column j: after it every block holds the combined partial sums
// of the previous phase and
//   1. (one thread) forms ||x|| of column j below the diagonal by downdating
//      ||a - c v||^2 = s1 - 2 Re(c conj(s2)) + |c|^2 s3  (c = conj(tau) w_j)
//      from the sums gathered in the previous phase, and from it beta, tau
//      and 1/(alpha-beta) (identical in every block); when the downdating
//      would cancel (result < s1 / 2) or the column holds magnitudes outside
//      the safe squaring range, an extra barrier recomputes the norm exactly
//      with the three-accumulator scheme (FP64);
//   2. (all threads, meanwhile) applies H[j-1]^H (tau[j-1], v[j-1],
//      w[j-1] = v^H A) to its rows of the panel columns right of j-1;
//   3. scales its rows of x into v;
//   4. accumulates over its rows w_c = v^H A[:,c] (c > j), the Gram column
//      g_c = V[:,c]^H v (c < j) and the downdating sums of column j+1, and
//      writes them into the partial record of the next phase; while the
//      following barrier settles, one warp of block 0 extends T by column j
//      from the Gram column.
// FP32 panels accumulate the downdating sums error-free in FP32 (hi + lo
// pairs, about 2^-48 relative), downdate and form the reflector scalars in
// FP32 pair arithmetic, and use FP64 only on the exact path.
// Records are double-buffered by phase parity and combined by all threads in
// a fixed order with all loads of a thread in flight at once: the result is
// deterministic for a given grid size.
// ---------------------------------------------------------------------------
constexpr int kRecT = kPanelMaxCols + 2;  // w/g[32], alpha of the next column, v at its row
constexpr int kRecD = 6;                  // s1, s3, unsafe, Re s2, Im s2 | exact: sml, med, big
template <class T> struct PanelRec {
    T v[kRecT];
    double d[kRecD];  // FP64 sums (FP64 data, and exact norms of every type)
    float fh[kRecD];  // FP32 data: the downdating sums as hi + lo pairs
    float fl[kRecD];
};

template <class T> struct PanelArgs {
    T *A;
    size_t lda;
    int M, N;            // panel rows and columns, N <= kPanelMaxCols, M >= N
    T *tau;              // N
    T *Tm;               // N x N upper triangular T factor (ldt); may be null
    int ldt;
    PanelRec<T> *rec;    // [2][gridDim.x]
    unsigned *counter;   // zeroed before launch
    int *err;            // zeroed before launch
    int *status;         // library-wide status word
    int rows_per_cta;
};

__device__ __forceinline__ double re_of(double v) { return v; }
__device__ __forceinline__ double re_of(float v) { return v; }
template <class R> __device__ __forceinline__ double re_of(cplx<R> v) { return v.x; }
__device__ __forceinline__ double im_of(double) { return 0.0; }
__device__ __forceinline__ double im_of(float) { return 0.0; }
template <class R> __device__ __forceinline__ double im_of(cplx<R> v) { return v.y; }
__device__ __forceinline__ float re_f(float v) { return v; }
__device__ __forceinline__ float re_f(cf32 v) { return v.x; }
__device__ __forceinline__ float im_f(float) { return 0.f; }
__device__ __forceinline__ float im_f(cf32 v) { return v.y; }
template <class T> __device__ __forceinline__ float re_f(T v) { return (float)re_of(v); }
template <class T> __device__ __forceinline__ float im_f(T v) { return (float)im_of(v); }

// pairwise sum of N values in a fixed order
template <class U, int N> __device__ __forceinline__ U tree_sum(U (&v)[N]) {
#pragma unroll
    for (int w = N / 2; w >= 1; w /= 2)
#pragma unroll
        for (int i = 0; i < w; ++i) v[i] = v[i] + v[i + w];
    return v[0];
}

// FP32 data whose downdated squared norm n2 is an FP32 pair and whose
// magnitudes lie in the safe range [2^-40, 2^48] (squares and their sums stay
// normal FP32 numbers): beta = -sign(Re alpha) sqrt(|alpha|^2 + n2) rounded
// once from the pair, tau = (beta - alpha)/beta and 1/(alpha - beta) in FP32
template <class T> __device__ ReflScalars<T> reflector_scalars_f32(T alpha, F2 n2) {
    typedef typename Tr<T>::R R;
    ReflScalars<T> s;
    const float ar = re_f(alpha), ai = im_f(alpha);
    s.knt = 0;
    s.sh = 0;
    s.sr_lo = 0.0f;
    s.si_lo = 0.0f;
    if (n2.h == 0.0f && n2.l == 0.0f && ai == 0.0f) {
        s.identity = true;
        s.tau = T(0);
        s.scal = T(1);
        s.sr = 1.0;
        s.si = 0.0;
        s.sr_hi = 1.0f;
        s.si_hi = 0.0f;
        s.beta = ar;
        return s;
    }
    s.identity = false;
    const F2 q = f2_add(f2_add(f2_sq(ar), f2_sq(ai)), n2);
    float beta = sqrtf(q.h + q.l);
    if (ar > 0.0f) beta = -beta;
    const float d = ar - beta;  // |d| = |ar| + |beta|: no cancellation
    const float tr = (beta - ar) / beta, ti = -ai / beta;
    float sr, si;
    if (Tr<T>::is_complex) {
        const float z2 = fmaf(d, d, ai * ai);
        sr = d / z2;
        si = -ai / z2;
    } else {
        sr = 1.0f / d;
        si = 0.0f;
    }
    s.tau = Tr<T>::make((R)tr, (R)ti);
    s.scal = Tr<T>::make((R)sr, (R)si);
    s.sr = sr;
    s.si = si;
    s.sr_hi = sr;
    s.si_hi = si;
    s.beta = beta;
    return s;
}

// m = max(|x|, |y|) >= 2^486 or 0 < m < 2^-511 (outside the range where
// squares and their sums stay normal FP64 numbers), from the exponent bits
// (integer pipe); non-finite values count as unsafe
__device__ __forceinline__ bool exp_unsafe64(double x, double y = 0.0) {
    const int ex = (__double2hiint(x) >> 20) & 0x7ff, ey = (__double2hiint(y) >> 20) & 0x7ff;  // biased exponents
    const int e = max(ex, ey);
    const bool nonzero = ((__double_as_longlong(x) | __double_as_longlong(y)) << 1) != 0;
    return e >= 1023 + 486 || (e < 1023 - 511 && nonzero);
}

// cluster barrier (all threads of every block of the cluster arrive; the
// release / acquire pair carries each thread's prior shared-memory writes to
// the other blocks)
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// SMEM = true: the block's rows of the panel live in dynamic shared memory
// for the whole launch (loaded once, written back at the end); SMEM = false:
// they are read and written in place in global memory (panels too tall for
// shared memory).
// CL = true: the grid is one thread-block cluster (up to 16 blocks, short
// panels): the partial records live in each block's shared memory and are
// read by the others through distributed shared memory, and the grid barrier
// is the cluster's hardware barrier (no global-memory round trip, no spin).
template <class T, bool SMEM, bool CL = false, int NT = kPanelThreads> __global__ void __launch_bounds__(NT) k_panel(PanelArgs<T> p) {
    typedef typename Tr<T>::R R;
    constexpr bool is64 = sizeof(R) == 8;
    constexpr int nwarps = NT / 32;
    constexpr int kSlots = kRecT + kRecD;            // one thread per record entry ...
    constexpr int kGroups = NT / kSlots;  // ... and kGroups subsets of the records
    // records summed per thread, unrolled; a cluster has at most 16 blocks
    // over the kGroups subsets, and every FP64 add is a 64-cycle instruction
    constexpr int UNR = CL ? 8 : ((sizeof(T) <= 4) ? 32 : (sizeof(T) <= 8 ? 16 : 8));
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = b * p.rows_per_cta;
    const int r1 = min(p.M, r0 + p.rows_per_cta);
    const size_t lda = p.lda;
    T *A = p.A;
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;
    auto bar_arrive = [&]() {
        if (CL) cluster_arrive();
        else bar.arrive();
    };
    auto bar_wait = [&]() -> bool {
        if (CL) {
            cluster_wait();
            return true;
        }
        return bar.wait();
    };
    auto bar_sync = [&]() -> bool {
        bar_arrive();
        return bar_wait();
    };

    __shared__ PanelRec<T> s_rec[CL ? 2 : 1];  // CL: this block's records of the two phase parities
    constexpr bool kColLanes = CL && is64;       // FP64 short panels: lanes over columns (below)
    __shared__ T s_part[kColLanes ? nwarps : 1][kPanelMaxCols];  // per-warp record partials
    __shared__ T s_cvr[kColLanes ? 1024 : 1];                   // -conj(tau) v of the last reflector, own rows
    __shared__ T s_T[kPanelMaxCols][kPanelMaxCols + 1];
    __shared__ T s_cv[kRecT];          // combined record
    __shared__ double s_cd[kRecD];     // combined FP64 sums
    __shared__ float s_ch[kRecD], s_cl[kRecD];  // combined FP32 pair sums
    __shared__ T s_pv[kGroups][kRecT];
    __shared__ double s_pd[kGroups][kRecD];
    __shared__ float s_ph[kGroups][kRecD], s_pl[kGroups][kRecD];
    __shared__ double s_red[nwarps][6];
    __shared__ float s_rh[nwarps][6], s_rl[nwarps][6];
    __shared__ ReflScalars<T> s_refl;
    __shared__ int s_exact;
    __shared__ T s_g[kPanelMaxCols];   // block 0: Gram column of the last reflector
    __shared__ T s_gtau;
    __shared__ int s_gid, s_gcol;
    extern __shared__ __align__(16) unsigned char s_dyn[];
    T *sP = reinterpret_cast<T *>(s_dyn);
    // cluster panels read rows across columns (lanes over columns): an odd
    // leading dimension keeps those loads free of bank conflicts
    const int ldp = CL ? (p.rows_per_cta | 1) : p.rows_per_cta;
    auto at = [&](int r, int c) -> T & {
        if (SMEM) return sP[(size_t)c * ldp + (r - r0)];
        return A[r + (size_t)c * lda];
    };
    if (SMEM) {
        for (int c = 0; c < p.N; ++c)
            for (int r = r0 + tid; r < r1; r += NT) sP[(size_t)c * ldp + (r - r0)] = A[r + (size_t)c * lda];
    }
    __syncthreads();

    int phase = 0;  // records of phase k live in buffer k & 1
    auto my_rec = [&]() -> PanelRec<T> & {
        if (CL) return s_rec[phase & 1];
        return p.rec[(size_t)(phase & 1) * G + b];
    };
    // block q's record of the current phase (CL: in block q's shared memory)
    auto rec_of = [&](int q) -> const PanelRec<T> * {
        if (CL) return cooperative_groups::this_cluster().map_shared_rank(&s_rec[phase & 1], q);
        return p.rec + (size_t)(phase & 1) * G + q;
    };
    auto ldr = [](const auto *ptr) {
        if (CL) return *ptr;
        return ldcg(ptr);
    };
    // combine the records of the current phase into s_cv and s_cd (FP64
    // sums) or s_ch/s_cl (FP32 pair sums)
    auto combine = [&](bool pairs) {
        const int slot = tid % kSlots, grp = tid / kSlots;
        if (grp < kGroups) {
            if (slot < kRecT) {
                T a = T(0);
                for (int base = grp; base < G; base += UNR * kGroups) {
                    T v[UNR];
#pragma unroll
                    for (int u = 0; u < UNR; ++u) {
                        const int q = base + u * kGroups;
                        v[u] = (q < G) ? ldr(&rec_of(q)->v[slot]) : T(0);
                    }
                    a = a + tree_sum(v);
                }
                s_pv[grp][slot] = a;
            } else if (pairs) {
                const int d = slot - kRecT;
                float h = 0.f, l = 0.f;
                for (int base = grp; base < G; base += 16 * kGroups) {
                    float vh[16], vl[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        const int q = base + u * kGroups;
                        vh[u] = (q < G) ? ldr(&rec_of(q)->fh[d]) : 0.f;
                        vl[u] = (q < G) ? ldr(&rec_of(q)->fl[d]) : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        df_add(h, l, vh[u]);
                        l += vl[u];
                    }
                }
                s_ph[grp][d] = h;
                s_pl[grp][d] = l;
            } else {
                const int d = slot - kRecT;
                double a = 0.0;
                for (int base = grp; base < G; base += 16 * kGroups) {
                    double v[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        const int q = base + u * kGroups;
                        v[u] = (q < G) ? ldr(&rec_of(q)->d[d]) : 0.0;
                    }
                    a += tree_sum(v);
                }
                s_pd[grp][d] = a;
            }
        }
        __syncthreads();
        if (tid < kRecT) {
            T a = s_pv[0][tid];
            for (int g = 1; g < kGroups; ++g) a = a + s_pv[g][tid];
            s_cv[tid] = a;
        } else if (tid < kSlots) {
            const int d = tid - kRecT;
            if (pairs) {
                float h = s_ph[0][d], l = s_pl[0][d];
                for (int g = 1; g < kGroups; ++g) {
                    df_add(h, l, s_ph[g][d]);
                    l += s_pl[g][d];
                }
                s_ch[d] = h;
                s_cl[d] = l;
            } else {
                double a = s_pd[0][d];
                for (int g = 1; g < kGroups; ++g) a += s_pd[g][d];
                s_cd[d] = a;
            }
        }
        __syncthreads();
    };
    // exact norm record of column col (rows > col) and its diagonal element
    auto exact_record = [&](int col) {
        NormAcc acc;
        acc.zero();
        for (int r = max(r0, col + 1) + tid; r < r1; r += NT) acc.add(at(r, col));
        acc.warp_reduce();
        if (lane == 0) {
            s_red[warp][0] = acc.sml;
            s_red[warp][1] = acc.med;
            s_red[warp][2] = acc.big;
        }
        __syncthreads();
        ++phase;
        PanelRec<T> &rc = my_rec();
        if (tid < kRecT) rc.v[tid] = (tid == kPanelMaxCols && col >= r0 && col < r1) ? at(col, col) : T(0);
        if (tid < kRecD) {
            double t = 0.0;
            if (tid < 3)
                for (int w = 0; w < nwarps; ++w) t += s_red[w][tid];
            rc.d[tid] = t;
        }
    };
    // thread 0: reflector scalars from the combined exact record
    auto scalars_from_exact = [&]() {
        if (tid == 0) {
            NormAcc nacc;
            nacc.sml = s_cd[0];
            nacc.med = s_cd[1];
            nacc.big = s_cd[2];
            s_refl = reflector_scalars<T>(s_cv[kPanelMaxCols], nacc);
        }
        __syncthreads();
    };

    // block 0, one warp: T(0:jc, jc) = -tau_jc T(0:jc, 0:jc) g(0:jc),
    // T(jc, jc) = tau_jc, for the column jc saved after the last combine
    // (GenerateBlockTr "F","C", Reflector.hpp:588-622)
    auto t_column = [&]() {
        const int jc = s_gcol;
        if (jc < 0) return;
        if (lane < jc) {
            T acc = T(0);
            for (int l = lane; l < jc; ++l) acc = fmac(s_T[lane][l], s_g[l], acc);
            s_T[lane][jc] = s_gid ? T(0) : (-s_gtau) * acc;
        }
        if (lane == 0) s_T[jc][jc] = s_gtau;
        __syncwarp();
    };
    if (tid == 0) s_gcol = -1;

    // prologue: exact norm of column 0
    exact_record(0);
    if (!bar_sync()) return;
    combine(false);
    scalars_from_exact();
    ReflScalars<T> prev;
    prev.identity = true;
    prev.tau = T(0);

    for (int j = 0; j < p.N; ++j) {
        if (j > 0) {
            // 1. one thread of the last warp (which owns no rows to update
            //    when the block holds fewer rows than threads) forms the
            //    downdated norm of column j and its reflector scalars
            if (tid == NT - 1) {
                const T a_pre = s_cv[kPanelMaxCols], vn = s_cv[kPanelMaxCols + 1];
                T alpha = a_pre, c = T(0);
                if (!prev.identity) {
                    const T ctau = Tr<T>::conj(prev.tau);
                    const T wj = s_cv[j];
                    alpha = fmac(-(ctau * vn), wj, a_pre);
                    c = ctau * wj;
                }
                if (is64) {
                    const double s1 = s_cd[0], s3 = s_cd[1], unsafe = s_cd[2], s2r = s_cd[3], s2i = s_cd[4];
                    double n2 = s1;
                    if (!prev.identity) {
                        const double cr = re_of(c), ci = im_of(c);
                        // Re(c * conj(s2)) = cr*s2r + ci*s2i
                        n2 = s1 - 2.0 * (cr * s2r + ci * s2i) + (cr * cr + ci * ci) * s3;
                    }
                    const int exact = (unsafe != 0.0 || !(n2 >= 0.5 * s1) || !(n2 < 1e300)) ? 1 : 0;
                    s_exact = exact;
                    if (!exact) {
                        NormAcc nacc;
                        nacc.zero();
                        nacc.med = n2;
                        s_refl = reflector_scalars<T>(alpha, nacc);
                    }
                } else {
                    // FP32 data: the same downdating in FP32 pair arithmetic
                    const F2 s1{s_ch[0], s_cl[0]}, s3{s_ch[1], s_cl[1]}, s2r{s_ch[3], s_cl[3]}, s2i{s_ch[4], s_cl[4]};
                    F2 n2 = s1;
                    if (!prev.identity) {
                        const float cr = re_f(c), ci = im_f(c);
                        const F2 u = f2_add(f2_mul(s2r, cr), f2_mul(s2i, ci));
                        const F2 cc = f2_add(f2_sq(cr), f2_sq(ci));
                        n2 = f2_add(f2_add(s1, f2_mul(u, -2.0f)), f2_mul(cc, s3));
                    }
                    const float ma = fmaxf(fabsf(re_f(alpha)), fabsf(im_f(alpha)));
                    const bool bad_alpha = ma > 0x1p48f || (ma < 0x1p-40f && ma != 0.0f);
                    const int exact = (s_ch[2] != 0.0f || bad_alpha || !(n2.h >= 0.5f * s1.h) || !(n2.h < 0x1p120f)) ? 1 : 0;
                    s_exact = exact;
                    if (!exact) s_refl = reflector_scalars_f32<T>(alpha, n2);
                }
            }
            // 2. apply H[j-1]^H to own rows r >= j-1 of columns j..N-1
            if (!prev.identity) {
                if constexpr (kColLanes) {
                    // one FP64 FMA per (row, column) pair, the pairs spread
                    // over all warps but the last (whose last thread forms
                    // the scalars meanwhile); row factors from s_cvr
                    constexpr int NA = NT - 32;
                    const int rs2 = max(r0, j - 1), nr = r1 - rs2;
                    if (tid < NA && nr > 0) {
                        // pair e = (row rs2 + e % nr, column j + e / nr), stepped
                        // by NA with a carry instead of a division per pair
                        const int dq = NA / nr, dr = NA % nr;
                        int r = rs2 + tid % nr, c = j + tid / nr;
                        while (c < p.N) {
                            at(r, c) = fmac(s_cvr[r - r0], s_cv[c], at(r, c));
                            r += dr;
                            c += dq;
                            if (r >= r1) {
                                r -= nr;
                                ++c;
                            }
                        }
                    }
                } else {
                    const T ctau = Tr<T>::conj(prev.tau);
                    for (int r = max(r0, j - 1) + tid; r < r1; r += NT) {
                        const T v = (r == j - 1) ? T(1) : at(r, j - 1);
                        const T cv = ctau * v;
                        for (int c = j; c < p.N; ++c) at(r, c) = fmac(-cv, s_cv[c], at(r, c));
                    }
                }
            }
            __syncthreads();
            if (s_exact) {
                exact_record(j);
                if (!bar_sync()) return;
                combine(false);
                scalars_from_exact();
            }
        }
        // 3. scale x into v
        const ReflScalars<T> rs = s_refl;
        if (!rs.identity) {
            for (int r = max(r0, j + 1) + tid; r < r1; r += NT) at(r, j) = scale_x(at(r, j), rs);
            if (tid == 0 && j >= r0 && j < r1) at(j, j) = Tr<T>::make((R)rs.beta, 0);
        }
        if (b == 0 && tid == 0) p.tau[j] = rs.tau;
        __syncthreads();
        // 4. partial record of this phase
        ++phase;
        PanelRec<T> &rc = my_rec();
        T anext = T(0), vnext = T(0);
        if constexpr (kColLanes) {
            // FP64 short panels: lane c accumulates record entry c over the
            // warp's chunk of rows >= j (no shuffle reductions: an FP64 warp
            // instruction costs the same for one lane as for 32).  Lane j,
            // which has no entry, sums |v|^2 and lane j+1 skips rows j and
            // j+1: over rows >= j+2 they are s3 and s2 of the downdating;
            // w_{j+1} gets rows j and j+1 back after the warps are summed.
            const int rs4 = max(r0, j), nr = max(0, r1 - rs4);
            const int per = (nr + nwarps - 1) / nwarps;
            const int ra = rs4 + warp * per, rb = min(r1, ra + per);
            const int c = lane;
            T acc = T(0);
            if (c < p.N) {
                const bool tail = (c == j || c == j + 1);
                for (int r = ra; r < rb; ++r) {
                    const T v = (r == j) ? T(1) : at(r, j);
                    const T a = at(r, c);
                    if (!tail || r >= j + 2) acc = (c >= j) ? fmac(Tr<T>::conj(v), a, acc) : fmac(Tr<T>::conj(a), v, acc);
                }
            }
            s_part[warp][c] = acc;
            if (c == j) s_red[warp][1] = re_of(acc);
            if (c == j + 1) {
                s_red[warp][3] = re_of(acc);
                s_red[warp][4] = im_of(acc);
            }
            // s1 and the magnitude flag of column j+1: lanes over rows
            double e1 = 0.0;
            bool unsafe = false;
            if (j + 1 < p.N) {
                for (int r = max(r0, j + 2) + tid; r < r1; r += NT) {
                    const T a = at(r, j + 1);
                    const double ar = re_of(a);
                    if (Tr<T>::is_complex) {
                        const double ai = im_of(a);
                        unsafe |= exp_unsafe64(ar, ai);
                        e1 = fma(ar, ar, fma(ai, ai, e1));
                    } else {
                        unsafe |= exp_unsafe64(ar);
                        e1 = fma(ar, ar, e1);
                    }
                }
            }
            const bool any_unsafe = __any_sync(0xffffffffu, unsafe);
            e1 = warp_sum(e1);
            if (lane == 0) {
                s_red[warp][0] = e1;
                s_red[warp][2] = any_unsafe ? 1.0 : 0.0;
                if (j + 1 >= p.N) {
                    s_red[warp][1] = 0.0;
                    s_red[warp][3] = 0.0;
                    s_red[warp][4] = 0.0;
                }
            }
        } else {
            // two columns per warp at a time, two rows per step (four
            // independent chains)
            for (int c0 = warp; c0 < p.N; c0 += 2 * nwarps) {
                const int c1 = c0 + nwarps;
                const bool u0 = (c0 != j), u1 = (c1 < p.N && c1 != j);
                T a00 = T(0), a01 = T(0), a10 = T(0), a11 = T(0);
                auto step = [&](int r, T &x0, T &x1) {
                    const T v = (r == j) ? T(1) : at(r, j);
                    if (u0) {
                        const T a = at(r, c0);
                        x0 = (c0 > j) ? fmac(Tr<T>::conj(v), a, x0) : fmac(Tr<T>::conj(a), v, x0);
                    }
                    if (u1) {
                        const T a = at(r, c1);
                        x1 = (c1 > j) ? fmac(Tr<T>::conj(v), a, x1) : fmac(Tr<T>::conj(a), v, x1);
                    }
                };
                int r = max(r0, j) + lane;
                for (; r + 32 < r1; r += 64) {
                    step(r, a00, a10);
                    step(r + 32, a01, a11);
                }
                if (r < r1) step(r, a00, a10);
                const T acc0 = warp_sum(a00 + a01), acc1 = warp_sum(a10 + a11);
                if (lane == 0) {
                    rc.v[c0] = acc0;
                    if (c1 < p.N) rc.v[c1] = acc1;
                }
            }
            for (int c = p.N + tid; c < kPanelMaxCols; c += NT) rc.v[c] = T(0);
            if (is64) {
                // FP64 instructions share one slow pipe per SM here, so the
                // real case skips the imaginary parts, the magnitude test reads
                // the exponent bits (integer pipe) and the flag is a warp vote
                double e1 = 0.0, e3 = 0.0, e2r = 0.0, e2i = 0.0;
                bool unsafe = false;
                if (j + 1 < p.N) {
                    for (int r = max(r0, j + 2) + tid; r < r1; r += NT) {
                        const T a = at(r, j + 1), v = at(r, j);
                        const double ar = re_of(a), vr = re_of(v);
                        if (Tr<T>::is_complex) {
                            const double ai = im_of(a), vi = im_of(v);
                            unsafe |= exp_unsafe64(ar, ai);
                            e1 = fma(ar, ar, fma(ai, ai, e1));
                            e3 = fma(vr, vr, fma(vi, vi, e3));
                            // conj(v) a
                            e2r = fma(vr, ar, fma(vi, ai, e2r));
                            e2i = fma(vr, ai, fma(-vi, ar, e2i));
                        } else {
                            unsafe |= exp_unsafe64(ar);
                            e1 = fma(ar, ar, e1);
                            e3 = fma(vr, vr, e3);
                            e2r = fma(vr, ar, e2r);
                        }
                    }
                }
                const double eu = __any_sync(0xffffffffu, unsafe) ? 1.0 : 0.0;
                e1 = warp_sum(e1);
                e3 = warp_sum(e3);
                e2r = warp_sum(e2r);
                if (Tr<T>::is_complex) e2i = warp_sum(e2i);
                if (lane == 0) {
                    s_red[warp][0] = e1;
                    s_red[warp][1] = e3;
                    s_red[warp][2] = eu;
                    s_red[warp][3] = e2r;
                    s_red[warp][4] = e2i;
                }
            } else {
                // FP32 data: error-free FP32 accumulation; magnitudes outside
                // [2^-40, 2^48] (squares that could leave the FP32 range or lose
                // their low parts) send the column to the exact FP64 norm
                float h1 = 0.f, l1 = 0.f, h3 = 0.f, l3 = 0.f, h2r = 0.f, l2r = 0.f, h2i = 0.f, l2i = 0.f, eu = 0.f;
                if (j + 1 < p.N) {
                    for (int r = max(r0, j + 2) + tid; r < r1; r += NT) {
                        const T a = at(r, j + 1), v = at(r, j);
                        const float ar = re_f(a), vr = re_f(v), ai = im_f(a), vi = im_f(v);
                        const float m = fmaxf(fabsf(ar), fabsf(ai));
                        if (m > 0x1p48f || (m < 0x1p-40f && m != 0.f)) eu = 1.f;
                        df_add_prod(h1, l1, ar, ar);
                        df_add_prod(h3, l3, vr, vr);
                        df_add_prod(h2r, l2r, vr, ar);
                        if (Tr<T>::is_complex) {
                            df_add_prod(h1, l1, ai, ai);
                            df_add_prod(h3, l3, vi, vi);
                            df_add_prod(h2r, l2r, vi, ai);
                            df_add_prod(h2i, l2i, vr, ai);
                            df_add_prod(h2i, l2i, -vi, ar);
                        }
                    }
                }
                df_warp_sum(h1, l1);
                df_warp_sum(h3, l3);
                df_warp_sum(h2r, l2r);
                if (Tr<T>::is_complex) df_warp_sum(h2i, l2i);
                eu = warp_sum(eu);
                if (lane == 0) {
                    s_rh[warp][0] = h1; s_rl[warp][0] = l1;
                    s_rh[warp][1] = h3; s_rl[warp][1] = l3;
                    s_rh[warp][2] = eu; s_rl[warp][2] = 0.f;
                    s_rh[warp][3] = h2r; s_rl[warp][3] = l2r;
                    s_rh[warp][4] = h2i; s_rl[warp][4] = l2i;
                }
            }
        }
        if (j + 1 < p.N && j + 1 >= r0 && j + 1 < r1 && tid == 0) {
            anext = at(j + 1, j + 1);
            vnext = at(j + 1, j);
        }
        __syncthreads();
        if (tid < 5) {
            if (is64) {
                double t = 0.0;
                for (int w = 0; w < nwarps; ++w) t += s_red[w][tid];
                rc.d[tid] = t;
            } else {
                float h = s_rh[0][tid], l = s_rl[0][tid];
                for (int w = 1; w < nwarps; ++w) {
                    df_add(h, l, s_rh[w][tid]);
                    l += s_rl[w][tid];
                }
                rc.fh[tid] = h;
                rc.fl[tid] = l;
            }
        }
        if (tid == 5) {
            rc.d[5] = 0.0;
            rc.fh[5] = 0.f;
            rc.fl[5] = 0.f;
        }
        if constexpr (kColLanes) {
            // the warps' partials of every entry (fixed order); w_{j+1}
            // adds back rows j and j+1 where this block holds them
            if (tid < p.N) {
                T w = s_part[0][tid];
                for (int q = 1; q < nwarps; ++q) w = w + s_part[q][tid];
                if (tid == j) w = T(0);  // no entry for the reflector's own column
                if (tid == j + 1) {
                    if (j >= r0 && j < r1) w = w + at(j, j + 1);
                    if (j + 1 >= r0 && j + 1 < r1) w = fmac(Tr<T>::conj(at(j + 1, j)), at(j + 1, j + 1), w);
                }
                rc.v[tid] = w;
            } else if (tid < kPanelMaxCols) {
                rc.v[tid] = T(0);
            }
        }
        if (tid == 0) {
            rc.v[kPanelMaxCols] = anext;
            rc.v[kPanelMaxCols + 1] = vnext;
        }
        // block 0 extends T by the previous column while the barrier settles
        bar_arrive();
        if (b == 0 && warp == 1) t_column();
        if (!bar_wait()) return;
        combine(!is64);
        if (b == 0) {
            if (tid < kPanelMaxCols) s_g[tid] = s_cv[tid];
            if (tid == 0) {
                s_gtau = rs.tau;
                s_gid = rs.identity ? 1 : 0;
                s_gcol = j;
            }
        }
        prev = rs;
        if constexpr (kColLanes) {
            // row factors of the next apply step: -conj(tau_j) v_r, own rows >= j
            if (!rs.identity && j + 1 < p.N) {
                const T mct = -Tr<T>::conj(rs.tau);
                for (int r = max(r0, j) + tid; r < r1; r += NT) s_cvr[r - r0] = (r == j) ? mct : mct * at(r, j);
            }
            __syncthreads();
        }
    }
    // CL: no block leaves while another may still read its records
    if (CL) bar_sync();
    __syncthreads();
    if (b == 0 && warp == 1) t_column();
    __syncthreads();
    if (SMEM) {
        for (int c = 0; c < p.N; ++c)
            for (int r = r0 + tid; r < r1; r += NT) A[r + (size_t)c * lda] = sP[(size_t)c * ldp + (r - r0)];
    }
    if (b == 0 && p.Tm != nullptr) {
        for (int idx = tid; idx < p.N * p.N; idx += NT) {
            int r = idx % p.N, c = idx / p.N;
            if (r <= c) p.Tm[r + (size_t)c * p.ldt] = s_T[r][c];
        }
    }
}

// ---------------------------------------------------------------------------
// Generic tiled contraction on CUDA cores.
//   D(m,n) = alpha * sum_k opA(m,k) * opB(k,n)  [+ D(m,n) | + delta(m,n)]
// op: 0 = N, 1 = T, 2 = C (conjugate transpose).  An operand flagged
// "vunit" is a Householder block V read in its stored coordinates (row,col):
// zero above the diagonal, one on it (RNP/LA/Reflector.hpp:530-545).
// blockIdx.z splits K into chunks of 'kchunk'; chunk z writes D + z*dstride.
// ---------------------------------------------------------------------------
enum { kOpN = 0, kOpT = 1, kOpC = 2 };
enum { kBetaZero = 0, kBetaOne = 1, kBetaIdentity = 2 };

template <class T> struct GemmArgs {
    const T *A;
    size_t lda;
    const T *B;
    size_t ldb;
    T *D;
    size_t ldd;
    int M, N, K;
    int opA, opB;
    int vunitA, vunitB;
    T alpha;
    int beta_mode;
    int kchunk;
    size_t dstride;
};

template <class T> __device__ __forceinline__ T load_op(const T *X, size_t ldx, int op, int vunit, int i, int k) {
    // element (i,k) of op(X): stored coordinates (row, col)
    int row = (op == kOpN) ? i : k, col = (op == kOpN) ? k : i;
    T v;
    if (vunit && row <= col) v = (row == col) ? T(1) : T(0);
    else v = X[row + (size_t)col * ldx];
    return (op == kOpC) ? Tr<T>::conj(v) : v;
}

template <class T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_gemm(GemmArgs<T> g) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int TX = BN / TN;  // threads along n
    constexpr int LA = (BM * BK + NT - 1) / NT, LB = (BN * BK + NT - 1) / NT;
    __shared__ T sA[BK][BM + 1];
    __shared__ T sB[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * g.kchunk;
    const int kend = min(g.K, kbeg + g.kchunk);
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

    // the next tile is fetched into registers while the current one is used
    T ra[LA], rb[LB];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int idx = tid + u * NT;
            int mi, ki;
            if (g.opA == kOpN) { mi = idx % BM; ki = idx / BM; }
            else { ki = idx % BK; mi = idx / BK; }
            const int gm = m0 + mi, gk = k0 + ki;
            ra[u] = (idx < BM * BK && gm < g.M && gk < kend) ? load_op(g.A, g.lda, g.opA, g.vunitA, gm, gk) : T(0);
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int idx = tid + u * NT;
            int ni, ki;
            if (g.opB == kOpN) { ki = idx % BK; ni = idx / BK; }
            else { ni = idx % BN; ki = idx / BN; }
            const int gn = n0 + ni, gk = k0 + ki;
            rb[u] = (idx < BN * BK && gn < g.N && gk < kend) ? load_op(g.B, g.ldb, g.opB, g.vunitB, gk, gn) : T(0);
        }
    };
    auto stash = [&]() {
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int idx = tid + u * NT;
            if (idx < BM * BK) {
                int mi, ki;
                if (g.opA == kOpN) { mi = idx % BM; ki = idx / BM; }
                else { ki = idx % BK; mi = idx / BK; }
                sA[ki][mi] = ra[u];
            }
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int idx = tid + u * NT;
            if (idx < BN * BK) {
                int ni, ki;
                if (g.opB == kOpN) { ki = idx % BK; ni = idx / BK; }
                else { ni = idx % BN; ki = idx / BN; }
                sB[ki][ni] = rb[u];
            }
        }
    };
    if (kbeg < kend) fetch(kbeg);
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        stash();
        __syncthreads();
        if (k0 + BK < kend) fetch(k0 + BK);
#pragma unroll 4
        for (int kk = 0; kk < BK; ++kk) {
            T a[TM], bb[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = sA[kk][ty + i * (BM / TM)];
#pragma unroll
            for (int j = 0; j < TN; ++j) bb[j] = sB[kk][tx + j * TX];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fmac(a[i], bb[j], acc[i][j]);
        }
        __syncthreads();
    }
    T *D = g.D + (size_t)blockIdx.z * g.dstride;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int gm = m0 + ty + i * (BM / TM);
        if (gm >= g.M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            int gn = n0 + tx + j * TX;
            if (gn >= g.N) continue;
            T v = g.alpha * acc[i][j];
            T *dp = &D[gm + (size_t)gn * g.ldd];
            if (g.beta_mode == kBetaOne) v = v + *dp;
            else if (g.beta_mode == kBetaIdentity && gm == gn) v = v + T(1);
            *dp = v;
        }
    }
}

// ---------------------------------------------------------------------------
// W(r, :) = (sum_s P_s(r, :)) * op(T), T upper triangular k x k.
// op 0: T, op 2: T^H.   P_s has leading dimension ldp, stride pstride.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_sum_times_t(const T *P, size_t ldp, size_t pstride, int nsplit, int rows, int k, const T *Tm, int ldt, int opT, T *W, size_t ldw) {
    __shared__ T sT[kPanelMaxCols][kPanelMaxCols + 1];
    __shared__ T sW[8][kPanelMaxCols + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < k * k; idx += 256) {
        int r = idx % k, c = idx / k;
        sT[r][c] = (r <= c) ? Tm[r + (size_t)c * ldt] : T(0);
    }
    const int rl = tid / kPanelMaxCols, j = tid % kPanelMaxCols;
    const int row = blockIdx.x * 8 + rl;
    T s = T(0);
    if (row < rows && j < k) {
        T a[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) a[u] = T(0);
        int q = 0;
        for (; q + 8 <= nsplit; q += 8) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = a[u] + P[(size_t)(q + u) * pstride + row + (size_t)j * ldp];
        }
        for (int u = 0; q < nsplit; ++q, ++u) a[u] = a[u] + P[(size_t)q * pstride + row + (size_t)j * ldp];
        s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    }
    sW[rl][j] = s;
    __syncthreads();
    if (row < rows && j < k) {
        T acc = T(0);
        if (opT == kOpN) {
            for (int l = 0; l <= j; ++l) acc = fmac(sW[rl][l], sT[l][j], acc);
        } else {
            for (int l = j; l < k; ++l) acc = fmac(sW[rl][l], Tr<T>::conj(sT[j][l]), acc);
        }
        W[row + (size_t)j * ldw] = acc;
    }
}

// ---------------------------------------------------------------------------
// The same product when there are many partials: W(r, :) = (sum_s P_s(r, :))
// op(T) in one launch.  Block: one row of W, 256 threads = 8 split lanes x 32
// columns (one block per row: every SM has loads in flight, and each thread
// has at most a few batches of eight); lane q sums partials q, q + 8, ... in
// independent batches of eight loads, the eight lane sums are added in a
// fixed order, then the row is multiplied by op(T) as above (T's loads go out
// with the partials').
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_reduce_times_t(const T *P, size_t ldp, size_t pstride, int nsplit, int rows, int k, const T *Tm, int ldt, int opT, T *W, size_t ldw) {
    __shared__ T sT[kPanelMaxCols][kPanelMaxCols + 1];
    __shared__ T sP[8][kPanelMaxCols + 1];
    const int tid = threadIdx.x, q = tid >> 5, j = tid & 31, row = blockIdx.x;
    for (int idx = tid; idx < k * k; idx += blockDim.x) {
        const int r = idx % k, c = idx / k;
        sT[r][c] = (r <= c) ? Tm[r + (size_t)c * ldt] : T(0);
    }
    T a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = T(0);
    if (row < rows && j < k) {
        const T *base = P + row + (size_t)j * ldp;
        int sp = q;
        for (; sp + 56 < nsplit; sp += 64) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = a[u] + base[(size_t)(sp + 8 * u) * pstride];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (sp + 8 * u < nsplit) a[u] = a[u] + base[(size_t)(sp + 8 * u) * pstride];
    }
    sP[q][j] = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    __syncthreads();
    if (q == 0) {
        sP[0][j] = ((sP[0][j] + sP[1][j]) + (sP[2][j] + sP[3][j])) + ((sP[4][j] + sP[5][j]) + (sP[6][j] + sP[7][j]));
        __syncwarp();
        if (row < rows && j < k) {
            T acc = T(0);
            if (opT == kOpN) {
                for (int l = 0; l <= j; ++l) acc = fmac(sP[0][l], sT[l][j], acc);
            } else {
                for (int l = j; l < k; ++l) acc = fmac(sP[0][l], Tr<T>::conj(sT[j][l]), acc);
            }
            W[row + (size_t)j * ldw] = acc;
        }
    }
}

// ---------------------------------------------------------------------------
// out(r, c) = sum over s < nsplit of P_s(r, c): four threads per entry, each
// over every fourth partial in independent batches of eight loads, then the
// four sums in a fixed order (one long chain of dependent loads per entry
// would leave the sum latency bound).  Grid: ((rows + 63) / 64, cols).
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_reduce_splits(const T *P, size_t ldp, size_t pstride, int nsplit, int rows, T *out, size_t ldo) {
    __shared__ T s_part[4][64];
    const int tid = threadIdx.x, rl = tid % 64, q = tid / 64;
    const int r = blockIdx.x * 64 + rl, c = blockIdx.y;
    T a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = T(0);
    if (r < rows) {
        const T *base = P + r + (size_t)c * ldp;
        int sp = q;
        for (; sp + 28 < nsplit; sp += 32) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = a[u] + base[(size_t)(sp + 4 * u) * pstride];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (sp + 4 * u < nsplit) a[u] = a[u] + base[(size_t)(sp + 4 * u) * pstride];
    }
    s_part[q][rl] = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    __syncthreads();
    if (q == 0 && r < rows) out[r + (size_t)c * ldo] = (s_part[0][rl] + s_part[1][rl]) + (s_part[2][rl] + s_part[3][rl]);
}

// ---------------------------------------------------------------------------
// T factors from Gram matrices (GenerateBlockTr "F","C" recurrence,
// RNP/LA/Reflector.hpp:588-622):  for i = 0..k-1,
//   T(0:i, i) = -tau_i * T(0:i,0:i) * G(0:i, i),  T(i,i) = tau_i
// with G = V^H V (sum of nsplit partials).  One block per reflector block.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kBuildTThreads) k_build_t(const T *P, size_t pstride_split, size_t pstride_blk, int nsplit, const T *tau, int nb, int k_total, T *Tout, size_t tstride, int ldt) {
    __shared__ T sG[kPanelMaxCols][kPanelMaxCols + 1];
    __shared__ T sT[kPanelMaxCols][kPanelMaxCols + 1];
    const int blk = blockIdx.x, tid = threadIdx.x;
    const int i0 = blk * nb;
    const int k = min(nb, k_total - i0);
    const T *Pb = P + (size_t)blk * pstride_blk;
    // the split partials of the strictly upper Gram entries, summed by all
    // threads of the block (one entry per thread, a fixed order)
    for (int e = tid; e < kPanelMaxCols * kPanelMaxCols; e += blockDim.x) {
        const int r = e % kPanelMaxCols, c = e / kPanelMaxCols;
        if (r < c && c < k) {
            T s = T(0);
            for (int q = 0; q < nsplit; ++q) s = s + Pb[(size_t)q * pstride_split + r + (size_t)c * kPanelMaxCols];
            sG[r][c] = s;
        }
    }
    __syncthreads();
    // the recurrence: each step's products T(r, l) G(l, i) split over the
    // first kBuildTWarps warps by l (a warp issues an FP64 instruction only
    // every 64 cycles), the partials summed by warp 0
    __shared__ T sP4[kBuildTWarps][kPanelMaxCols];
    const int w = tid / kPanelMaxCols, r = tid % kPanelMaxCols;
    constexpr int kChunk = kPanelMaxCols / kBuildTWarps;
    for (int i = 0; i < k; ++i) {
        if (w < kBuildTWarps) {
            T acc = T(0);
            const int l0 = max(r, w * kChunk), l1 = min(i, (w + 1) * kChunk);
            for (int l = l0; l < l1; ++l) acc = fmac(sT[r][l], sG[l][i], acc);
            sP4[w][r] = acc;
        }
        __syncthreads();
        if (tid < kPanelMaxCols) {
            const T ti = tau[i0 + i];
            if (r < i) {
                T acc = sP4[0][r];
#pragma unroll
                for (int q = 1; q < kBuildTWarps; ++q) acc = acc + sP4[q][r];
                sT[r][i] = (ti == T(0)) ? T(0) : (-ti) * acc;
            }
            if (r == 0) sT[i][i] = ti;
        }
        __syncthreads();
    }
    T *To = Tout + (size_t)blk * tstride;
    if (tid < kPanelMaxCols)
        for (int c = 0; c < k; ++c)
            if (tid <= c) To[tid + (size_t)c * ldt] = sT[tid][c];
}

// Y = T * V1^H (k x k) with V1 the unit lower triangular top of V (stored at
// v with leading dimension ldv).  k blocks of kPanelMaxCols threads.
template <class T>
__global__ void __launch_bounds__(kPanelMaxCols) k_t_v1h(const T *Tm, int ldt, const T *v, size_t ldv, int k, T *Y, int ldy) {
    // one warp per column of Y: the FP64 chains spread over k SMs
    const int r = threadIdx.x, c = blockIdx.x;
    if (r >= k || c >= k) return;
    // Y(r,c) = sum_l T(r,l) * conj(V1(c,l)),  T(r,l)=0 for l<r, V1(c,l)=0 for l>c, V1(c,c)=1
    T acc = T(0);
    for (int l = r; l <= c; ++l) {
        T vcl = (l == c) ? T(1) : v[c + (size_t)l * ldv];
        acc = fmac(Tm[r + (size_t)l * ldt], Tr<T>::conj(vcl), acc);
    }
    Y[r + (size_t)c * ldy] = acc;
}

// ---------------------------------------------------------------------------
// Level-2 kernels for the *_unblocked entry points
// ---------------------------------------------------------------------------

// larfg on one column: alpha = *alpha_p, x = x[0..n-1) with stride 1.
template <class T> __global__ void __launch_bounds__(256) k_larfg(int n, T *alpha_p, T *x, T *tau_p) {
    __shared__ NormAcc s_nacc[8];
    __shared__ ReflScalars<T> s_refl;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (n <= 0) {
        if (tid == 0) *tau_p = T(0);
        return;
    }
    NormAcc acc;
    acc.zero();
    for (int r = tid; r < n - 1; r += 256) acc.add(x[r]);
    acc.warp_reduce();
    if (lane == 0) s_nacc[warp] = acc;
    __syncthreads();
    if (tid == 0) {
        NormAcc t = s_nacc[0];
        for (int w = 1; w < 8; ++w) t.merge(s_nacc[w]);
        s_refl = reflector_scalars<T>(*alpha_p, t);
    }
    __syncthreads();
    const ReflScalars<T> rs = s_refl;
    if (!rs.identity)
        for (int r = tid; r < n - 1; r += 256) x[r] = scale_x(x[r], rs);
    if (tid == 0) {
        *tau_p = rs.tau;
        if (!rs.identity) *alpha_p = Tr<T>::make((typename Tr<T>::R)rs.beta, 0);
    }
}

// side L:  w_c = sum_r conj(v_r) C[r,c]   (v_0 = 1), c < nc, r < mc
// side R:  w_r = sum_c C[r,c] v_c         (v_0 = 1), r < mc, c < nc
template <class T> __global__ void __launch_bounds__(256) k_larf_w(int left, int mc, int nc, const T *v, const T *C, size_t ldc, T *w) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (left) {
        int c = blockIdx.x * 8 + warp;
        if (c >= nc) return;
        T acc = T(0);
        for (int r = lane; r < mc; r += 32) {
            T vr = (r == 0) ? T(1) : v[r];
            acc = fmac(Tr<T>::conj(vr), C[r + (size_t)c * ldc], acc);
        }
        acc = warp_sum(acc);
        if (lane == 0) w[c] = acc;
    } else {
        int r = blockIdx.x * 256 + tid;
        if (r >= mc) return;
        T acc = T(0);
        for (int c = 0; c < nc; ++c) {
            T vc = (c == 0) ? T(1) : v[c];
            acc = fmac(C[r + (size_t)c * ldc], vc, acc);
        }
        w[r] = acc;
    }
}

// side L:  C[r,c] -= tau * v_r * w_c ;  side R:  C[r,c] -= tau * w_r * conj(v_c)
// tau = *taup, conjugated when conj_tau is set
template <class T> __global__ void __launch_bounds__(256) k_larf_update(int left, int mc, int nc, const T *v, const T *w, const T *taup, int conj_tau, T *C, size_t ldc) {
    const int r = blockIdx.x * 256 + threadIdx.x;
    if (r >= mc) return;
    const T tau = conj_tau ? Tr<T>::conj(*taup) : *taup;
    if (tau == T(0)) return;
    for (int c = blockIdx.y; c < nc; c += gridDim.y) {
        T upd;
        if (left) {
            T vr = (r == 0) ? T(1) : v[r];
            upd = tau * vr * w[c];
        } else {
            T vc = (c == 0) ? T(1) : v[c];
            upd = tau * w[r] * Tr<T>::conj(vc);
        }
        C[r + (size_t)c * ldc] = C[r + (size_t)c * ldc] - upd;
    }
}

// GenerateQ_unblocked column finish (RNP/LA/QR.hpp:475-483):
// A[i+1:m, i] *= -tau_i;  A[i,i] = 1 - tau_i;  A[0:i, i] = 0
template <class T> __global__ void __launch_bounds__(256) k_ung2r_col(int m, int i, T *A, size_t lda, const T *tau) {
    const T t = tau[i];
    T *col = A + (size_t)i * lda;
    for (int r = blockIdx.x * 256 + threadIdx.x; r < m; r += gridDim.x * 256) {
        if (r < i) col[r] = T(0);
        else if (r == i) col[r] = T(1) - t;
        else col[r] = (-t) * col[r];
    }
}

// columns [j0, j1) of an m-row matrix set to the identity's columns
template <class T> __global__ void __launch_bounds__(256) k_identity_cols(int m, int j0, int j1, T *A, size_t lda) {
    for (int c = j0 + blockIdx.y; c < j1; c += gridDim.y)
        for (int r = blockIdx.x * 256 + threadIdx.x; r < m; r += gridDim.x * 256) A[r + (size_t)c * lda] = (r == c) ? T(1) : T(0);
}

// rows [0, r1) of columns [c0, c1) set to zero
template <class T> __global__ void __launch_bounds__(256) k_zero_rows(int r1, int c0, int c1, T *A, size_t lda) {
    for (int c = c0 + blockIdx.y; c < c1; c += gridDim.y)
        for (int r = blockIdx.x * 256 + threadIdx.x; r < r1; r += gridDim.x * 256) A[r + (size_t)c * lda] = T(0);
}

} // namespace rnpgpu
