// panel_cqr.cuh — FP32 panel factorization for the internal FP32 factor of
// the mixed least-squares solver (not the drop-in Factor, whose output must
// be the reference's Householder QR): CholeskyQR2 (its first Gram matrix in
// double-float when the panel needs it), then Householder reconstruction of
// the orthonormal factor.
//
//   G1 = A^T A, R1 = chol(G1), Q1 = A R1^-1 (FP32 first; double-float sums and
//   factor when Q1 comes out too far from orthonormal);
//   G2 = Q1^T Q1, R2 = chol(G2), Q = Q1 R2^-1, R = R2 R1   (both in FP32)
//   (Yamamoto, Nakatsukasa, Yanagisawa and Fukaya, "Roundoff error analysis
//   of the CholeskyQR2 algorithm", ETNA 44, 2015: the second pass restores
//   orthogonality to working precision when kappa(Q1) is modest; the
//   double-float first pass keeps kappa(Q1) modest for kappa(A) up to about
//   10^5 — Yamazaki, Tomov and Dongarra, "Mixed-precision Cholesky QR
//   factorization and its case studies on multicore CPU with multiple GPUs",
//   SIAM J. Sci. Comput. 37(3), 2015);
//   then the Householder form of Q (Ballard, Demmel, Grigori, Jacquelin,
//   Knight and Nguyen, "Reconstructing Householder vectors from tall-skinny
//   QR", J. Parallel Distrib. Comput. 85, 2015): the LU factorization
//   Q - S = L U without pivoting, with s_j = -sign of the j-th pivot of Q's
//   top block (so that |u_jj| >= 1), gives V = L (unit lower trapezoidal),
//   T = -U S L1^-T and the R of the Householder QR, S R.  Below the top block
//   V = Q U^-1 = Q1 (U R2)^-1: one triangular solve per row.
//
// Every block keeps its rows in shared memory (row-major, 36 floats a row).
// A Gram matrix is formed as 36 upper-triangle tiles of 4 x 4 entries, one
// warp per tile with the rows split across its lanes, summed across the lanes
// by a butterfly; the per-block partials are then summed across blocks by
// all blocks at once (one warp per entry), and every block reads the total
// back and factors it itself, identically — four grid barriers in all (eight
// when the first pass is redone in double-float).  The 32 x 32 factors are
// formed four columns a step: one warp factors the diagonal block and
// publishes the block's rows, then all warps update their entries.  Block 0
// holds the top 32 rows and forms T at the end from two triangular inverses.
// Panels narrower than 32 columns are padded with zero columns and a unit
// Gram diagonal, which carries an identity through every step.
//
// The first pass runs in FP32; a pivot of it below 2^-20 of its column's
// squared norm, or ||G2 - I||_F > 0.1 after it, sends the panel through both
// passes again with the first in double-float.  A double-float pivot that is
// not positive or below 2^-38 of its column's squared norm, or a second-pass
// pivot below 2^-14 of its diagonal (Q1 far from orthonormal), marks the panel
// as failed before anything is written; the caller then refactors it with
// Householder panels.  That happens for panels with condition numbers near
// 10^5 and above, zero columns and non-finite data.
#pragma once
#include "qr_kernels.cuh"

namespace rnpgpu {

constexpr int kCqrThreads = 512;
constexpr int kPanelMaxBlocksCqr = 256;
constexpr int kCqrLd = 36;                     // floats per row of a block's rows in shared memory
constexpr int kCqrTiles = 36;                  // 4 x 4 tiles of a 32 x 32 upper triangle
constexpr int kCqrEntries = kCqrTiles * 16;    // entries of a Gram partial (tile-major)
constexpr int kCqrStaticSmem = 40 * 1024;      // bound on the kernel's static shared memory
constexpr int kCqrMaxDynSmem = 227 * 1024 - kCqrStaticSmem;

struct CqrArgs {
    float *A;
    size_t lda;
    int M, N;             // N <= 32, every block holds >= 32 rows
    float *tau;           // N
    float *Tm;            // N x N upper triangular T (ldt), may be null
    int ldt;
    float2 *gpart;        // [gridDim.x][kCqrEntries] per-block Gram partials (hi, lo)
    float2 *gfin;         // [kCqrEntries] the summed Gram matrix
    float *qtop;          // 32 x 32 row-major: the top rows of Q1
    unsigned *counter;    // zeroed before the launch
    int *err;             // zeroed before the launch
    int *status;          // library-wide status word
    int *fail;            // set when a Cholesky factorization fails
    int rows_per_cta;
};

// double-float helper beyond rnp_common.cuh: a - b c with the sum left
// unnormalized
__device__ __forceinline__ F2 f2_fms(F2 a, F2 b, F2 c) {
    const float p = b.h * c.h;
    const float e = fmaf(b.h, c.l, fmaf(b.l, c.h, fmaf(b.h, c.h, -p)));
    const float s = a.h - p, bp = s - a.h;
    const float err = (a.h - (s - bp)) + (-p - bp);
    return F2{s, (a.l + err) - e};
}
// tile t of the 8 x 8 grid of 4 x 4 tiles over the upper triangle, row-major
__device__ __forceinline__ void cqr_tile(int t, int &ti, int &tj) {
    int i = 0;
    while (t >= 8 - i) {
        t -= 8 - i;
        ++i;
    }
    ti = i;
    tj = i + t;
}
// a warp's 16 sums (h, l per lane) -> each even lane holds the total of one
// entry, whose index it returns (a butterfly that halves the entries at each
// of four steps, then adds lane pairs)
__device__ __forceinline__ int cqr_warp_reduce16(float (&h)[16], float (&l)[16], int lane) {
#pragma unroll
    for (int lvl = 0; lvl < 4; ++lvl) {
        const int o = 16 >> lvl, n = 8 >> lvl;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const F2 a{h[i], l[i]}, c{h[i + n], l[i + n]};
            const F2 send = up ? a : c, keep = up ? c : a;
            const F2 recv{__shfl_xor_sync(0xFFFFFFFFu, send.h, o), __shfl_xor_sync(0xFFFFFFFFu, send.l, o)};
            const F2 s = f2_add(keep, recv);
            h[i] = s.h;
            l[i] = s.l;
        }
    }
    const F2 recv{__shfl_xor_sync(0xFFFFFFFFu, h[0], 1), __shfl_xor_sync(0xFFFFFFFFu, l[0], 1)};
    const F2 s = f2_add(F2{h[0], l[0]}, recv);
    h[0] = s.h;
    l[0] = s.l;
    return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

// packed FP32x2 arithmetic (two independent lanes per instruction)
__device__ __forceinline__ float2 cqr_neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 cqr_dup(float a) { return make_float2(a, a); }
// (h, l) += a c for two entries at once: TwoProduct by FMA and TwoSum, as
// df_add_prod, on packed pairs
__device__ __forceinline__ void df_add_prod2(float2 &h, float2 &l, float2 a, float2 c) {
    const float2 p = __fmul2_rn(a, c);
    const float2 e = __ffma2_rn(a, c, cqr_neg2(p));
    const float2 s = __fadd2_rn(h, p);
    const float2 bp = __fadd2_rn(s, cqr_neg2(h));
    const float2 err = __fadd2_rn(__fadd2_rn(h, cqr_neg2(__fadd2_rn(s, cqr_neg2(bp)))), __fadd2_rn(p, cqr_neg2(bp)));
    l = __fadd2_rn(l, __fadd2_rn(err, e));
    h = s;
}

// x (one row, 32 entries as 16 pairs) <- x Rf^-1 for Rf upper triangular in
// shared memory (rows of kCqrLd floats, 16-byte aligned) with reciprocal
// diagonal rinv
__device__ __forceinline__ void cqr_row_solve(float2 (&x)[16], const float (*Rf)[kCqrLd], const float *rinv) {
#pragma unroll
    for (int l = 0; l < 32; ++l) {
        float xl = ((l & 1) ? x[l >> 1].y : x[l >> 1].x) * rinv[l];
        if (l & 1) x[l >> 1].y = xl;
        else x[l >> 1].x = xl;
        const float2 nx = cqr_dup(-xl);
#pragma unroll
        for (int q = (l + 1) / 4; q < 8; ++q) {
            const float4 r = *reinterpret_cast<const float4 *>(&Rf[l][4 * q]);
            if (4 * q > l) x[2 * q] = __ffma2_rn(nx, make_float2(r.x, r.y), x[2 * q]);
            else if (4 * q + 1 > l) x[2 * q].y = fmaf(-xl, r.y, x[2 * q].y);
            if (4 * q + 2 > l) x[2 * q + 1] = __ffma2_rn(nx, make_float2(r.z, r.w), x[2 * q + 1]);
            else if (4 * q + 3 > l) x[2 * q + 1].y = fmaf(-xl, r.w, x[2 * q + 1].y);
        }
    }
}
__device__ __forceinline__ void cqr_row_load(float2 (&x)[16], const float *row) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 v = *reinterpret_cast<const float4 *>(row + 4 * q);
        x[2 * q] = make_float2(v.x, v.y);
        x[2 * q + 1] = make_float2(v.z, v.w);
    }
}
__device__ __forceinline__ void cqr_row_store(float *row, const float2 (&x)[16]) {
#pragma unroll
    for (int q = 0; q < 8; ++q) *reinterpret_cast<float4 *>(row + 4 * q) = make_float4(x[2 * q].x, x[2 * q].y, x[2 * q + 1].x, x[2 * q + 1].y);
}

// 1 / sqrt(a) for a > 0: the hardware approximation and one Newton step
// y + y (1 - a y^2) / 2, the residual formed with the exact product a.h y
// (about 2^-43 relative in double-float; FP32 to about an ulp)
__device__ __forceinline__ F2 f2_rsqrt(F2 a) {
    const float y = rsqrtf(a.h);
    const float p = a.h * y, pe = fmaf(a.h, y, -p);
    const float r = fmaf(-p, y, 1.0f) - fmaf(pe, y, a.l * y * y);
    return f2_norm(y, 0.5f * y * r);
}
__device__ __forceinline__ float f32_rsqrt(float a) {
    const float y = rsqrtf(a);
    return fmaf(0.5f * y, fmaf(-a * y, y, 1.0f), y);
}

// arithmetic of the blocked Cholesky: double-float (kDF) or FP32 in the
// same F2 carrier (lo stays zero)
template <bool kDF> struct CqrArith {
    static __device__ __forceinline__ F2 from(float2 v) { return kDF ? F2{v.x, v.y} : F2{v.x + v.y, 0.f}; }
    static __device__ __forceinline__ F2 fms(F2 a, F2 b, F2 c) { return kDF ? f2_fms(a, b, c) : F2{fmaf(-b.h, c.h, a.h), 0.f}; }
    static __device__ __forceinline__ F2 mul(F2 a, F2 b) { return kDF ? f2_mul(f2_norm(a.h, a.l), b) : F2{a.h * b.h, 0.f}; }
    static __device__ __forceinline__ F2 norm(F2 a) { return kDF ? f2_norm(a.h, a.l) : a; }
    static __device__ __forceinline__ F2 rsqrt(F2 a) { return kDF ? f2_rsqrt(a) : F2{f32_rsqrt(a.h), 0.f}; }
};

// Cholesky of the 32 x 32 Gram matrix in sG (upper triangle; hi, lo pairs) by
// the whole block, four columns a step: thread (w, j) holds entries (w, j)
// and (w + 16, j).  At step b warp 0 factors the 4 x 4 diagonal block
// D = R_BB^T R_BB, forms the block's four rows of R (lane x: R_B,x =
// R_BB^-T G_B,x) and writes them over sG's rows; after a block barrier every
// thread updates its entries below, and the holders of the next four rows
// publish them in sG — two block barriers a step.  Double-float (kDF) or
// FP32.  R in FP32 -> Rf (upper, zero below), its reciprocal diagonal ->
// rinv; a pivot not above thr times its column's original diagonal (or not
// finite) sets *fail.
template <bool kDF> __device__ __forceinline__ void cqr_cholesky(float2 (*sG)[kPanelMaxCols + 1], float (*Rf)[kCqrLd], float *rinv, float *sD0, float thr, int *fail) {
    using A = CqrArith<kDF>;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    F2 g0 = A::from(sG[w][lane]), g1 = A::from(sG[w + 16][lane]);
    if (threadIdx.x < kPanelMaxCols) sD0[threadIdx.x] = sG[threadIdx.x][threadIdx.x].x;
    __syncthreads();
    for (int k0 = 0; k0 < kPanelMaxCols; k0 += 4) {
        if (w == 0) {
            // the diagonal block's factor (upper, r[a][c] for a <= c) and the
            // reciprocals of its diagonal
            F2 r[4][4], ri[4];
            bool bad = false;
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = a; c < 4; ++c) r[a][c] = A::from(sG[k0 + a][k0 + c]);
#pragma unroll
            for (int a = 0; a < 4; ++a) {
#pragma unroll
                for (int m = 0; m < a; ++m)
#pragma unroll
                    for (int c = a; c < 4; ++c) r[a][c] = A::fms(r[a][c], r[m][a], r[m][c]);
                F2 piv = A::norm(r[a][a]);
                if (!(piv.h > thr * sD0[k0 + a]) || !(piv.h <= 3.0e38f)) {
                    bad = true;
                    piv = F2{1.f, 0.f};
                }
                ri[a] = A::rsqrt(piv);
                r[a][a] = A::mul(piv, ri[a]);
#pragma unroll
                for (int c = a + 1; c < 4; ++c) r[a][c] = A::mul(r[a][c], ri[a]);
            }
            // the block's rows of R in column `lane`
            F2 rj[4];
            if (lane > k0 + 3) {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    rj[a] = A::from(sG[k0 + a][lane]);
#pragma unroll
                    for (int m = 0; m < a; ++m) rj[a] = A::fms(rj[a], r[m][a], rj[m]);
                    rj[a] = A::mul(rj[a], ri[a]);
                }
            } else {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    rj[a] = F2{0.f, 0.f};
#pragma unroll
                    for (int c = a; c < 4; ++c)
                        if (lane == k0 + c) rj[a] = r[a][c];
                }
            }
            __syncwarp();
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                if (lane >= k0) sG[k0 + a][lane] = make_float2(rj[a].h, rj[a].l);
                Rf[k0 + a][lane] = (lane >= k0 + a) ? rj[a].h : 0.f;
            }
            if (lane == 0 && bad) *fail = 1;
        }
        __syncthreads();
        // this thread's entries (i, lane), i > k0 + 3, lane >= i
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const F2 rj = A::from(sG[k0 + a][lane]);
            if (w > k0 + 3 && lane >= w) g0 = A::fms(g0, A::from(sG[k0 + a][w]), rj);
            if (w + 16 > k0 + 3 && lane >= w + 16) g1 = A::fms(g1, A::from(sG[k0 + a][w + 16]), rj);
        }
        if (w >= k0 + 4 && w < k0 + 8) sG[w][lane] = make_float2(g0.h, g0.l);
        if (w + 16 >= k0 + 4 && w + 16 < k0 + 8) sG[w + 16][lane] = make_float2(g1.h, g1.l);
        __syncthreads();
    }
    if (threadIdx.x < kPanelMaxCols) rinv[threadIdx.x] = 1.0f / Rf[threadIdx.x][threadIdx.x];
    __syncthreads();
}

// LU without pivoting of Q1_top - S R2 = L M by the whole block, four rows a
// step (thread (w, c): rows w and w + 16, column c; the current rows are
// staged in sE), s_j = -sign of the j-th eliminated pivot of Q1_top (the sign
// of Q_top's, R2's diagonal being positive).  Warp 0 factors the 4 x 4
// diagonal block and writes the block's rows of M, their reciprocal pivots
// and the block's own multipliers; after a block barrier every thread forms
// the multipliers of its rows below and updates its entries.  M = U R2 -> Mt
// (upper), its reciprocal diagonal -> minv, L transposed -> Lt (Lt[c][i] =
// L(i, c) for c < i, zero elsewhere), the signs -> S.
__device__ __forceinline__ void cqr_top_lu(const float *qtop, const float (*R2)[kCqrLd], float (*Mt)[kCqrLd], float *minv, float (*Lt)[kCqrLd], float *S, float (*sE)[kCqrLd]) {
    constexpr unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float e0 = __ldcg(qtop + w * 32 + lane), e1 = __ldcg(qtop + (w + 16) * 32 + lane);
    if (w < 4) sE[w][lane] = e0;
    __syncthreads();
    for (int j0 = 0; j0 < kPanelMaxCols; j0 += 4) {
        if (w == 0) {
            // the diagonal block: m[a][c] (c >= a) rows of M, l[a][c] (c < a) multipliers
            float m[4][4], l[4][4], mi[4], sg[4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) m[a][c] = sE[j0 + a][j0 + c];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                sg[a] = (m[a][a] >= 0.f) ? -1.f : 1.f;
#pragma unroll
                for (int c = a; c < 4; ++c) m[a][c] = fmaf(-sg[a], R2[j0 + a][j0 + c], m[a][c]);
                mi[a] = 1.0f / m[a][a];
#pragma unroll
                for (int b = a + 1; b < 4; ++b) {
                    l[b][a] = m[b][a] * mi[a];
#pragma unroll
                    for (int c = a + 1; c < 4; ++c) m[b][c] = fmaf(-l[b][a], m[a][c], m[b][c]);
                }
            }
            // the block's rows of M in column `lane`
            float mc[4];
            if (lane > j0 + 3) {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    float v = fmaf(-sg[a], R2[j0 + a][lane], sE[j0 + a][lane]);
#pragma unroll
                    for (int b = 0; b < a; ++b) v = fmaf(-l[a][b], mc[b], v);
                    mc[a] = v;
                }
            } else {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    mc[a] = 0.f;
#pragma unroll
                    for (int c = a; c < 4; ++c)
                        if (lane == j0 + c) mc[a] = m[a][c];
                }
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) Mt[j0 + a][lane] = mc[a];
            if (lane < 4) {
#pragma unroll
                for (int a = 0; a < 4; ++a)
                    if (lane == a) {
                        S[j0 + a] = sg[a];
                        minv[j0 + a] = mi[a];
                    }
            }
            if (lane == 0) {
#pragma unroll
                for (int a = 1; a < 4; ++a)
#pragma unroll
                    for (int c = 0; c < a; ++c) Lt[j0 + c][j0 + a] = l[a][c];
            }
        }
        __syncthreads();
        // multipliers of this thread's rows i > j0 + 3 and their update
        auto eliminate = [&](float &e) {
            float li[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                float v = __shfl_sync(FULL, e, j0 + a);
#pragma unroll
                for (int b = 0; b < a; ++b) v = fmaf(-li[b], Mt[j0 + b][j0 + a], v);
                li[a] = v * minv[j0 + a];
            }
            if (lane > j0 + 3) {
#pragma unroll
                for (int a = 0; a < 4; ++a) e = fmaf(-li[a], Mt[j0 + a][lane], e);
            } else {
#pragma unroll
                for (int a = 0; a < 4; ++a)
                    if (lane == j0 + a) e = li[a];
            }
        };
        if (w > j0 + 3) eliminate(e0);
        if (w + 16 > j0 + 3) eliminate(e1);
        if (w >= j0 + 4 && w < j0 + 8) sE[w][lane] = e0;
        if (w + 16 >= j0 + 4 && w + 16 < j0 + 8) sE[w + 16][lane] = e1;
        __syncthreads();
    }
    // multipliers from earlier blocks (the block's own ones are in Lt already)
    if (lane < (w & ~3)) Lt[lane][w] = e0;
    else if (lane >= w) Lt[lane][w] = 0.f;
    if (lane < ((w + 16) & ~3)) Lt[lane][w + 16] = e1;
    else if (lane >= w + 16) Lt[lane][w + 16] = 0.f;
    __syncthreads();
}

template <int kTag> __global__ void __launch_bounds__(kCqrThreads, 1) k_panel_cqr(CqrArgs p) {
    constexpr int NB = kPanelMaxCols, LD = kCqrLd;
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // block 0 holds the top 32 rows (it also forms T and the top block at the
    // end); the other blocks share the rest, rows_per_cta each
    const int r0 = (b == 0) ? 0 : (G == 1 ? 0 : NB + (b - 1) * p.rows_per_cta);
    const int r1 = (G == 1) ? p.M : (b == 0 ? NB : min(p.M, r0 + p.rows_per_cta)), R = max(r1 - r0, 0);
    const int N = p.N;
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;

    extern __shared__ __align__(16) unsigned char s_dyn[];
    float *sQ = reinterpret_cast<float *>(s_dyn);  // the block's rows, row-major (LD)
    __shared__ __align__(16) float sR1[NB][LD];    // R1 in FP32 (upper)
    __shared__ __align__(16) float sR2[NB][LD];    // R2 (upper)
    __shared__ __align__(16) float sMt[NB][LD];    // M = U R2 (upper)
    __shared__ __align__(16) float sLt[NB][LD];    // L of the top block, transposed: sLt[k][j] = L(j, k), j > k
    __shared__ float2 sGram[NB][NB + 1];           // a summed Gram matrix (upper triangle), then R
    __shared__ __align__(16) float sE[NB][LD];     // rows of the top block's LU, staged
    __shared__ float sR1inv[NB], sR2inv[NB], sMinv[NB], sS[NB], sD0[NB];
    __shared__ int s_fail;
    __shared__ float s_dev;  // ||G2 - I||_F^2 of an FP32 first pass

    // FP32 Gram partial with 8 x 8 tiles (10 over the upper triangle, one per
    // warp): per row 4 shared loads for 64 FMAs (4 x 4 tiles: 2 for 16, and
    // 36 tiles over 16 warps take three rounds), then a reduce-scatter of
    // the 64 sums over the warp (lane L ends with entries 2L, 2L + 1 of the
    // tile, row L / 4) written into the 4 x 4 tile-major layout
    auto gram_partial_f32 = [&]() {
        if (warp < 10) {
            int TI = 0, t = warp;
            while (t >= 4 - TI) {
                t -= 4 - TI;
                ++TI;
            }
            const int TJ = TI + t;
            float2 acc[32];
#pragma unroll
            for (int e = 0; e < 32; ++e) acc[e] = make_float2(0.f, 0.f);
            for (int r = lane; r < R; r += 32) {
                const float *row = sQ + (size_t)r * LD;
                const float4 a0 = *reinterpret_cast<const float4 *>(row + 8 * TI), a1 = *reinterpret_cast<const float4 *>(row + 8 * TI + 4);
                const float4 c0 = *reinterpret_cast<const float4 *>(row + 8 * TJ), c1 = *reinterpret_cast<const float4 *>(row + 8 * TJ + 4);
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float2 cp[4] = {make_float2(c0.x, c0.y), make_float2(c0.z, c0.w), make_float2(c1.x, c1.y), make_float2(c1.z, c1.w)};
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[4 * a + q] = __ffma2_rn(cqr_dup(av[a]), cp[q], acc[4 * a + q]);
            }
            float v[64];
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                v[2 * e] = acc[e].x;
                v[2 * e + 1] = acc[e].y;
            }
#pragma unroll
            for (int lvl = 0; lvl < 5; ++lvl) {
                const int o = 16 >> lvl, n = 32 >> lvl;
                const bool up = (lane & o) != 0;
#pragma unroll
                for (int e = 0; e < n; ++e) {
                    const float send = up ? v[e] : v[e + n], keep = up ? v[e + n] : v[e];
                    v[e] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, o);
                }
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int x = 2 * lane + k, i = 8 * TI + (x >> 3), j = 8 * TJ + (x & 7);
                if (i <= j) {
                    const int ti = i >> 2, tj = j >> 2;
                    const int tt = ti * 8 - (ti * (ti - 1)) / 2 + (tj - ti);
                    p.gpart[(size_t)b * kCqrEntries + tt * 16 + 4 * (i & 3) + (j & 3)] = make_float2(v[k], 0.f);
                }
            }
        }
    };
    // the block's Gram partial of sQ into gpart[b]: double-float or FP32 sums,
    // entries of a tile row in packed pairs
    auto gram_partial = [&](bool df) {
        if (!df) {
            gram_partial_f32();
            return;
        }
        for (int t = warp; t < kCqrTiles; t += kCqrThreads / 32) {
            int ti, tj;
            cqr_tile(t, ti, tj);
            float2 h2[8], l2[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) h2[e] = l2[e] = make_float2(0.f, 0.f);
            if (df) {
                for (int r = lane; r < R; r += 32) {
                    const float4 a = *reinterpret_cast<const float4 *>(sQ + (size_t)r * LD + 4 * ti);
                    const float4 c = *reinterpret_cast<const float4 *>(sQ + (size_t)r * LD + 4 * tj);
                    const float av[4] = {a.x, a.y, a.z, a.w};
                    const float2 c01 = make_float2(c.x, c.y), c23 = make_float2(c.z, c.w);
#pragma unroll
                    for (int x = 0; x < 4; ++x) {
                        df_add_prod2(h2[2 * x], l2[2 * x], cqr_dup(av[x]), c01);
                        df_add_prod2(h2[2 * x + 1], l2[2 * x + 1], cqr_dup(av[x]), c23);
                    }
                }
            } else {
                for (int r = lane; r < R; r += 32) {
                    const float4 a = *reinterpret_cast<const float4 *>(sQ + (size_t)r * LD + 4 * ti);
                    const float4 c = *reinterpret_cast<const float4 *>(sQ + (size_t)r * LD + 4 * tj);
                    const float av[4] = {a.x, a.y, a.z, a.w};
                    const float2 c01 = make_float2(c.x, c.y), c23 = make_float2(c.z, c.w);
#pragma unroll
                    for (int x = 0; x < 4; ++x) {
                        h2[2 * x] = __ffma2_rn(cqr_dup(av[x]), c01, h2[2 * x]);
                        h2[2 * x + 1] = __ffma2_rn(cqr_dup(av[x]), c23, h2[2 * x + 1]);
                    }
                }
            }
            float h[16], l[16];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                h[2 * e] = h2[e].x;
                h[2 * e + 1] = h2[e].y;
                l[2 * e] = l2[e].x;
                l[2 * e + 1] = l2[e].y;
            }
            const int e = cqr_warp_reduce16(h, l, lane);
            if ((lane & 1) == 0) p.gpart[(size_t)b * kCqrEntries + t * 16 + e] = make_float2(h[0], l[0]);
        }
    };
    // the partials summed across blocks, one warp per entry, into gfin
    auto gram_sum = [&]() {
        for (int e = b + G * warp; e < kCqrEntries; e += G * (kCqrThreads / 32)) {
            // all of the lane's partials in flight at once (G <= 256), then
            // summed in the same order
            float2 v[kPanelMaxBlocksCqr / 32];
#pragma unroll
            for (int u = 0; u < kPanelMaxBlocksCqr / 32; ++u) {
                const int q = lane + 32 * u;
                v[u] = (q < G) ? __ldcg(&p.gpart[(size_t)q * kCqrEntries + e]) : make_float2(0.f, 0.f);
            }
            F2 s{0.f, 0.f};
#pragma unroll
            for (int u = 0; u < kPanelMaxBlocksCqr / 32; ++u)
                if (lane + 32 * u < G) s = f2_add(s, F2{v[u].x, v[u].y});
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = f2_add(s, F2{__shfl_xor_sync(0xFFFFFFFFu, s.h, o), __shfl_xor_sync(0xFFFFFFFFu, s.l, o)});
            if (lane == 0) __stcg(&p.gfin[e], make_float2(s.h, s.l));
        }
    };
    // every block: the summed Gram matrix into sGram (upper triangle), unit
    // diagonal on the padding columns
    auto gram_load = [&]() {
        for (int idx = tid; idx < kCqrEntries; idx += kCqrThreads) {
            int ti, tj;
            cqr_tile(idx >> 4, ti, tj);
            const int i = 4 * ti + ((idx >> 2) & 3), j = 4 * tj + (idx & 3);
            if (i <= j) sGram[i][j] = (i == j && i >= N) ? make_float2(1.f, 0.f) : __ldcg(&p.gfin[idx]);
        }
        __syncthreads();
    };
    auto failed = [&]() {
        if (s_fail && b == 0 && tid == 0) atomicExch(p.fail, 1);
        return s_fail != 0;
    };

    // ---- two passes: the first in FP32, accepted when Q1 comes out close to
    // orthonormal (||G2 - I||_F <= 0.1: the FP32 second pass then restores
    // orthogonality to working precision), else both again with the first in
    // double-float.  Every block decides from the same summed G2, so all take
    // the same barriers. ----
    if (tid == 0) s_fail = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        const bool df = attempt == 1;
        // the block's rows, row-major, zero padding columns (again on the
        // second attempt: the first left Q1 in sQ; A is written only at the end)
        for (int r = tid; r < R; r += kCqrThreads) {
            const float *src = p.A + (size_t)(r0 + r);
            float v[NB];
#pragma unroll
            for (int c = 0; c < NB; ++c) v[c] = (c < N) ? src[(size_t)c * p.lda] : 0.f;
#pragma unroll
            for (int q = 0; q < 8; ++q) *reinterpret_cast<float4 *>(sQ + (size_t)r * LD + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        __syncthreads();

        // first pass: G1 = A^T A, R1 = chol(G1), Q1 = A R1^-1
        gram_partial(df);
        if (!bar.sync()) return;
        gram_sum();
        if (!bar.sync()) return;
        gram_load();
        if (df) cqr_cholesky<true>(sGram, sR1, sR1inv, sD0, 0x1p-38f, &s_fail);
        else cqr_cholesky<false>(sGram, sR1, sR1inv, sD0, 0x1p-20f, &s_fail);
        if (s_fail != 0) {
            if (df) {
                failed();
                return;
            }
            __syncthreads();  // every thread has read the flag
            if (tid == 0) s_fail = 0;
            __syncthreads();
            continue;
        }
        for (int r = tid; r < R; r += kCqrThreads) {
            float2 x[NB / 2];
            cqr_row_load(x, sQ + (size_t)r * LD);
            // z = 0 (r < 2^30), but the compiler cannot tell: the factor's loads
            // stay in the loop instead of being hoisted out of it (they would
            // not fit in registers)
            const int z = r & 0x40000000;
            cqr_row_solve(x, sR1 + z, sR1inv + z);
            cqr_row_store(sQ + (size_t)r * LD, x);
        }
        __syncthreads();
        // the top 32 rows of Q1 for every block's reconstruction
        if (b == 0)
            for (int idx = tid; idx < NB * NB; idx += kCqrThreads) __stcg(&p.qtop[idx], sQ[(size_t)(idx >> 5) * LD + (idx & 31)]);

        // second pass: G2 = Q1^T Q1, R2 = chol(G2) (FP32)
        gram_partial(false);
        if (!bar.sync()) return;
        gram_sum();
        if (!bar.sync()) return;
        gram_load();
        if (!df) {
            if (warp == 0) {
                float d2 = 0.f;
                for (int i = 0; i <= lane; ++i) {
                    const float2 v = sGram[i][lane];
                    const float d = (v.x + v.y) - (i == lane ? 1.f : 0.f);
                    d2 = fmaf(i == lane ? d : 2.f * d, d, d2);
                }
                d2 = warp_sum(d2);
                if (lane == 0) s_dev = d2;
            }
            __syncthreads();
            if (!(s_dev <= 0.01f)) continue;
        }
        cqr_cholesky<false>(sGram, sR2, sR2inv, sD0, 0x1p-14f, &s_fail);
        if (failed()) return;
        break;
    }

    // ---- Householder reconstruction: Q1_top - S R2 = L M (M = U R2) ----
    cqr_top_lu(p.qtop, sR2, sMt, sMinv, sLt, sS, sE);
    // V below the top block: x M = q1 for every row
    for (int r = tid; r < R; r += kCqrThreads) {
        const int gr = r0 + r;
        if (gr < N) continue;
        float2 x[NB / 2];
        cqr_row_load(x, sQ + (size_t)r * LD);
        const int z = r & 0x40000000;  // zero, opaque: as in the first row solve
        cqr_row_solve(x, sMt + z, sMinv + z);
#pragma unroll
        for (int c = 0; c < NB; ++c)
            if (c < N) p.A[(size_t)gr + (size_t)c * p.lda] = (c & 1) ? x[c >> 1].y : x[c >> 1].x;
    }
    if (b != 0) return;

    // block 0: T = -U S L1^-T = -M P with P = R2^-1 S L1^-T (U = M R2^-1),
    // from the two triangular inverses (warp 0: R2^-1, warp 1: L1^-1, lane =
    // column); the top N x N block: L below the diagonal, R = S R2 R1 on and
    // above it
    float (*sInvR)[LD] = sE;                                     // R2^-1 (the LU's staging is free)
    float (*sInvL)[LD] = reinterpret_cast<float (*)[LD]>(&sGram[0][0]);  // L1^-1 (sGram is free)
    if (warp == 0) {
        float x[NB];
#pragma unroll
        for (int i = 0; i < NB; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
        for (int i = NB - 1; i >= 0; --i) {
            x[i] *= sR2inv[i];
#pragma unroll
            for (int k = 0; k < i; ++k) x[k] = fmaf(-sR2[k][i], x[i], x[k]);
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) sInvR[i][lane] = x[i];
    } else if (warp == 1) {
        float x[NB];
#pragma unroll
        for (int i = 0; i < NB; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
#pragma unroll
            for (int j = k + 1; j < NB; ++j) x[j] = fmaf(-sLt[k][j], x[k], x[j]);
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) sInvL[i][lane] = x[i];
    } else {
        for (int idx = tid - 64; idx < NB * NB; idx += kCqrThreads - 64) {
            const int i = idx & 31, j = idx >> 5;
            if (i >= N || j >= N) continue;
            float v;
            if (i > j) {
                v = sLt[j][i];
            } else {
                float s = 0.f;
                for (int k = i; k <= j; ++k) s = fmaf(sR2[i][k], sR1[k][j], s);
                v = sS[i] * s;
            }
            p.A[(size_t)i + (size_t)j * p.lda] = v;
        }
    }
    __syncthreads();
    // P(i, j) = sum_{i <= k <= j} R2^-1(i, k) s_k L1^-1(j, k) into sR1 (R1 is done with)
    for (int idx = tid; idx < NB * NB; idx += kCqrThreads) {
        const int i = idx >> 5, j = idx & 31;
        float s = 0.f;
        for (int k = i; k <= j; ++k) s = fmaf(sInvR[i][k] * sS[k], sInvL[j][k], s);
        sR1[i][j] = (i <= j) ? s : 0.f;
    }
    __syncthreads();
    // T(i, j) = -sum_{i <= k <= j} M(i, k) P(k, j); tau = diag(T)
    for (int idx = tid; idx < NB * NB; idx += kCqrThreads) {
        const int i = idx & 31, j = idx >> 5;
        if (i >= N || j >= N || i > j) continue;
        float s = 0.f;
        for (int k = i; k <= j; ++k) s = fmaf(sMt[i][k], sR1[k][j], s);
        if (p.Tm) p.Tm[i + (size_t)j * p.ldt] = -s;
        if (i == j) p.tau[i] = -s;
    }
}

} // namespace rnpgpu
