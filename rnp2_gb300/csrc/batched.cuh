// batched.cuh — thousands of small, uneven QR factorizations in one
// persistent launch.
//
// Each matrix of the batch is factored exactly as RNP::LA::QR::Factor would
// (same reflector convention, RNP/LA/QR.hpp:78-197), by one thread block:
// a blocked right-looking Householder QR whose NB-column panel is factored in
// shared memory (Generate / Apply per column, RNP/LA/Reflector.hpp:117-236,
// with the compact-WY T grown from the Gram column as in GenerateBlockTr,
// Reflector.hpp:580-626), followed by the trailing update
// C -= V (T^H (V^H C))... applied in column tiles staged in shared memory.
// Blocks take matrices from a work queue (one atomic counter) in the order of
// the descriptor array, which the host sorts by decreasing cost so the tail
// of the launch is made of small matrices.
#pragma once
#include "qr_kernels.cuh"

namespace rnpgpu {

struct BatchDesc {
    long long a_off;    // element offset of the matrix in the packed buffer
    long long tau_off;  // element offset of its tau
    long long b_off;    // least squares: element offsets of b (m) and x (n)
    long long x_off;
    int m, n, lda, index;
};

constexpr int kBatchMaxRows = 512;  // rows of the largest matrix a block stages

// MR: rows a block stages (the class's largest m); TILE: trailing-update
// column tile
template <class T, int NB, int MR, int TILE> struct BatchSmem {
    static constexpr size_t kP = (size_t)MR * NB;    // panel
    static constexpr size_t kC = (size_t)MR * TILE;  // trailing tile
    static constexpr size_t kW = (size_t)TILE * NB;
    static constexpr size_t kBytes = (kP + kC + kW + NB * NB + 2 * NB + MR) * sizeof(T);
};

template <class T, int NT, int NB, int MR, int TILE>
__global__ void __launch_bounds__(NT) k_geqrf_batched(const BatchDesc *__restrict__ desc, int count, T *A, T *tau, unsigned *queue) {
    typedef typename Tr<T>::R R;
    extern __shared__ __align__(16) unsigned char s_raw[];
    typedef BatchSmem<T, NB, MR, TILE> L;
    T *sP = reinterpret_cast<T *>(s_raw);  // panel, column-major, ld MR
    T *sC = sP + L::kP;                    // trailing tile, column-major, ld MR
    T *sW = sC + L::kC;                    // W (TILE x NB), ld TILE
    T *sT = sW + L::kW;                    // T (NB x NB), ld NB
    T *sG = sT + NB * NB;                  // w / Gram column (NB)
    T *sCv = sG + 2 * NB;                  // -conj(tau) v of the current reflector (MR)
    __shared__ NormAcc s_nacc[NT / 32];
    __shared__ T s_wp[NT / 32][NB];        // per-warp partials of w / Gram
    __shared__ ReflScalars<T> s_refl;
    __shared__ int s_idx;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;

    for (;;) {
        if (tid == 0) s_idx = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const BatchDesc d = desc[idx];
        T *a = A + d.a_off;
        T *tp = tau + d.tau_off;
        const int m = d.m, n = d.n, lda = d.lda;
        const int k = min(m, n);
        for (int j0 = 0; j0 < k; j0 += NB) {
            const int jb = min(NB, k - j0), mp = m - j0;
            // ---- panel into shared memory
            for (int e = tid; e < mp * jb; e += NT) {
                const int r = e % mp, c = e / mp;
                sP[c * MR + r] = a[(j0 + r) + (size_t)(j0 + c) * lda];
            }
            __syncthreads();
            // ---- factor the panel column by column
            for (int jj = 0; jj < jb; ++jj) {
                T *col = sP + jj * MR;
                NormAcc acc;
                acc.zero();
                for (int r = jj + 1 + tid; r < mp; r += NT) acc.add(col[r]);
                acc.warp_reduce();
                if (lane == 0) s_nacc[warp] = acc;
                __syncthreads();
                if (tid == 0) {
                    NormAcc t = s_nacc[0];
                    for (int w = 1; w < NW; ++w) t.merge(s_nacc[w]);
                    s_refl = reflector_scalars<T>(col[jj], t);
                }
                __syncthreads();
                const ReflScalars<T> rs = s_refl;
                if (!rs.identity)
                    for (int r = jj + 1 + tid; r < mp; r += NT) col[r] = scale_x(col[r], rs);
                __syncthreads();
                // the update's row factors -conj(tau) v_r, once per row
                if (!rs.identity && jj + 1 < jb) {
                    const T mct = -Tr<T>::conj(rs.tau);
                    for (int r = jj + tid; r < mp; r += NT) sCv[r] = (r == jj) ? mct : mct * col[r];
                }
                // w_c = v^H P[:,c] (c > jj) and Gram g_c = V[:,c]^H v (c < jj),
                // rows >= jj.  FP64 instructions cost the same for one lane as
                // for 32 on this GPU: lane = (column lane % NB, row group
                // lane / NB), the warps and row groups split the rows, the row
                // groups meet by log2(32 / NB) shuffles and the warps in
                // shared memory (no 32-lane reduction per column)
                {
                    constexpr int SUB = 32 / NB;
                    const int c = lane % NB, sg = lane / NB;
                    T s = T(0);
                    if (c < jb && c != jj) {
                        const T *pc = sP + c * MR;
                        for (int r = jj + sg + SUB * warp; r < mp; r += SUB * NW) {
                            const T v = (r == jj) ? T(1) : col[r];
                            s = (c > jj) ? fmac(Tr<T>::conj(v), pc[r], s) : fmac(Tr<T>::conj(pc[r]), v, s);
                        }
                    }
#pragma unroll
                    for (int o = NB; o < 32; o <<= 1) s = s + shfl_xor_t(s, o);
                    if (sg == 0) s_wp[warp][c] = s;
                }
                __syncthreads();
                if (tid < jb && tid != jj) {
                    T s = s_wp[0][tid];
#pragma unroll
                    for (int w = 1; w < NW; ++w) s = s + s_wp[w][tid];
                    sG[tid] = s;
                }
                __syncthreads();
                if (!rs.identity && jj + 1 < jb) {
                    // (row, column) pairs stepped with a carry (no division per pair)
                    const int nr = mp - jj;
                    const int dq = NT / nr, dr = NT % nr;
                    int r = jj + tid % nr, c = jj + 1 + tid / nr;
                    while (c < jb) {
                        sP[c * MR + r] = fmac(sCv[r], sG[c], sP[c * MR + r]);
                        r += dr;
                        c += dq;
                        if (r >= mp) {
                            r -= nr;
                            ++c;
                        }
                    }
                }
                // T(0:jj, jj) = -tau T(0:jj, 0:jj) g(0:jj), T(jj, jj) = tau
                if (tid < jj) {
                    T s = T(0);
                    for (int l = tid; l < jj; ++l) s = fmac(sT[tid + l * NB], sG[l], s);
                    sT[tid + jj * NB] = rs.identity ? T(0) : (-rs.tau) * s;
                }
                if (tid == 0) {
                    sT[jj + jj * NB] = rs.tau;
                    tp[j0 + jj] = rs.tau;
                    if (!rs.identity) col[jj] = Tr<T>::make((R)rs.beta, 0);
                }
                __syncthreads();
            }
            // ---- panel back to global memory
            for (int e = tid; e < mp * jb; e += NT) {
                const int r = e % mp, c = e / mp;
                a[(j0 + r) + (size_t)(j0 + c) * lda] = sP[c * MR + r];
            }
            // ---- trailing update, one column tile at a time:  C -= V (T^H ... ) : W = C^H V T, C -= V W^H
            for (int c0 = j0 + jb; c0 < n; c0 += TILE) {
                const int ct = min(TILE, n - c0);
                for (int e = tid; e < mp * ct; e += NT) {
                    const int r = e % mp, c = e / mp;
                    sC[c * MR + r] = a[(j0 + r) + (size_t)(c0 + c) * lda];
                }
                __syncthreads();
                // W(c, l) = sum_r conj(C(r, c)) V(r, l), V unit lower trapezoidal
                for (int e = tid; e < ct * jb; e += NT) {
                    const int c = e % ct, l = e / ct;
                    const T *vc = sP + l * MR;
                    const T *cc = sC + c * MR;
                    T s = Tr<T>::conj(cc[l]);
                    for (int r = l + 1; r < mp; ++r) s = fmac(Tr<T>::conj(cc[r]), vc[r], s);
                    sW[c + l * TILE] = s;
                }
                __syncthreads();
                // W := W T (upper triangular, in place by columns from the right)
                for (int c = tid; c < ct; c += NT) {
                    T w[NB];
#pragma unroll
                    for (int l = 0; l < NB; ++l) w[l] = (l < jb) ? sW[c + l * TILE] : T(0);
                    for (int l = jb - 1; l >= 0; --l) {
                        T s = T(0);
                        for (int q = 0; q <= l; ++q) s = fmac(w[q], sT[q + l * NB], s);
                        sW[c + l * TILE] = s;
                    }
                    // columns past a narrow last panel are read (times a zero
                    // coefficient) by the update below: they must hold zeros,
                    // not whatever the shared memory held before
                    for (int l = jb; l < NB; ++l) sW[c + l * TILE] = T(0);
                }
                __syncthreads();
                // C(r, c) -= sum_l V(r, l) conj(W(c, l))
                for (int r = tid; r < mp; r += NT) {
                    T v[NB];
#pragma unroll
                    for (int l = 0; l < NB; ++l) v[l] = (l < jb && r >= l) ? (r == l ? T(1) : sP[l * MR + r]) : T(0);
                    for (int c = 0; c < ct; ++c) {
                        T s = sC[c * MR + r];
#pragma unroll
                        for (int l = 0; l < NB; ++l) s = fmac(-v[l], Tr<T>::conj(sW[c + l * TILE]), s);
                        sC[c * MR + r] = s;
                    }
                }
                __syncthreads();
                for (int e = tid; e < mp * ct; e += NT) {
                    const int r = e % mp, c = e / mp;
                    a[(j0 + r) + (size_t)(c0 + c) * lda] = sC[c * MR + r];
                }
                __syncthreads();
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Warp per matrix, for the smallest size class (m <= 32, n <= 32): each warp
// of the block takes matrices from the work queue, keeps one in its slice of
// shared memory (column-major, leading dimension 33) and factors it column by
// column (Factor_unblocked, RNP/LA/QR.hpp:78-102): lanes over rows for the
// norm and the scaling of x, lanes over columns for w = v^H A and the update.
// No block-wide barrier is involved; lanes beyond m or n idle.
// ---------------------------------------------------------------------------
constexpr int kWarpRows = 32;
constexpr int kWarpLd = 33;

template <class T, int WPB> __global__ void __launch_bounds__(WPB * 32) k_geqrf_warp(const BatchDesc *__restrict__ desc, int count, T *A, T *tau, unsigned *queue) {
    typedef typename Tr<T>::R R;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    T *sM = reinterpret_cast<T *>(s_raw) + (size_t)wib * kWarpRows * kWarpLd;
    __shared__ ReflScalars<T> s_refl[WPB];
    for (;;) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(queue, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= (unsigned)count) break;
        const BatchDesc d = desc[idx];
        T *a = A + d.a_off;
        T *tp = tau + d.tau_off;
        const int m = d.m, n = d.n, lda = d.lda, k = min(m, n);
        for (int c = 0; c < n; ++c)
            if (lane < m) sM[c * kWarpLd + lane] = a[lane + (size_t)c * lda];
        __syncwarp();
        for (int j = 0; j < k; ++j) {
            T *col = sM + j * kWarpLd;
            NormAcc acc;
            acc.zero();
            if (lane > j && lane < m) acc.add(col[lane]);
            acc.warp_reduce();
            if (lane == 0) s_refl[wib] = reflector_scalars<T>(col[j], acc);
            __syncwarp();
            const ReflScalars<T> rs = s_refl[wib];
            if (!rs.identity && lane > j && lane < m) col[lane] = scale_x(col[lane], rs);
            __syncwarp();
            // H^H on the columns right of j: lane c forms w_c = v^H a_c and updates a_c
            const int c = lane;
            if (!rs.identity && c > j && c < n) {
                T *ac = sM + c * kWarpLd;
                T w = ac[j];
                for (int r = j + 1; r < m; ++r) w = fmac(Tr<T>::conj(col[r]), ac[r], w);
                const T cw = Tr<T>::conj(rs.tau) * w;
                ac[j] = ac[j] - cw;
                for (int r = j + 1; r < m; ++r) ac[r] = fmac(-col[r], cw, ac[r]);
            }
            if (lane == 0) {
                tp[j] = rs.tau;
                if (!rs.identity) col[j] = Tr<T>::make((R)rs.beta, 0);
            }
            __syncwarp();
        }
        for (int c = 0; c < n; ++c)
            if (lane < m) a[lane + (size_t)c * lda] = sM[c * kWarpLd + lane];
        __syncwarp();
    }
}

} // namespace rnpgpu
