// multq_thin.cuh — MultQ("L", trans) on a thin C (at most kThinMaxCols
// columns) in one cooperative launch, and the T factors of all reflector
// blocks of a MultQ call in two launches.
//
// RNP::LA::QR::MultQ (RNP/LA/QR.hpp:337-429) applies the reflector blocks one
// after another, each by ApplyBlock (RNP/LA/Reflector.hpp:725-815):
//   Q^H C:  C -= V_b (T_b^H (V_b^H C)),  b = 0, 1, ...
//   Q   C:  C -= V_b (T_b   (V_b^H C)),  b = ..., 1, 0
// For a thin C every block is a long reduction (V_b^H C over all rows)
// followed by a rank-32 update, far too little work for a launch of its own.
// Here thread block g owns rows [g R, (g+1) R) of C for the whole launch (in
// shared memory when they fit) and, per reflector block,
//   1. accumulates its part of V_b^H C over its rows (lanes along rows, a
//      4 x 4 tile of (reflector, column) per warp, reduced by shuffles),
//   2. writes it to its slot of the partial buffer;  grid barrier;
//   3. sums a slice of the (reflector, column) entries over all blocks in a
//      fixed order into the reduced buffer;  grid barrier;
//   4. reads V_b^H C back and forms Y = op(T_b) (V_b^H C) in shared memory,
//   5. updates its rows: C -= V_b Y.
// The summation order depends only on the grid size: results are
// deterministic.  Every barrier wait is bounded (GridBarrier).
#pragma once
#include "qr_kernels.cuh"

namespace rnpgpu {

constexpr int kThinMaxCols = 64;
constexpr int kThinThreads = 512;
constexpr int kThinWarps = kThinThreads / 32;

template <class T> struct ThinArgs {
    const T *A;
    size_t lda;
    const T *Tf;  // T of block b at Tf + b * kPanelMaxCols^2, leading dimension kPanelMaxCols
    T *C;
    size_t ldc;
    int m, n, k, nblk;
    int forward;  // 1: Q^H C (blocks ascending, op(T) = T^H); 0: Q C (descending, op(T) = T)
    T *part;      // [gridDim.x][kPanelMaxCols * n]
    T *wred;      // [kPanelMaxCols * n]
    unsigned *counter;
    int *err;
    int *status;  // library-wide status word
    int rows_per_cta;
};

// shared memory of the thin kernel: W, Y, T, VBUF staging buffers for the
// block's rows of V_b (column-major, leading dimension rows) and, when CSMEM,
// the block's rows of C (column-major, leading dimension rows + 4)
template <class T> inline size_t thin_smem_bytes(int rows, int n, bool csmem, int vbuf) {
    size_t e = (size_t)2 * kPanelMaxCols * n + (size_t)kPanelMaxCols * (kPanelMaxCols + 1);
    e += (size_t)vbuf * kPanelMaxCols * rows;
    if (csmem) e += (size_t)(rows + 4) * n;
    return e * sizeof(T);
}

// V_b element (row r, column l) in stored form: zero above the diagonal of
// the block, one on it
template <class T> __device__ __forceinline__ T vload(const T *A, size_t lda, int i, int r, int l) {
    const int d = r - (i + l);
    if (d < 0) return T(0);
    if (d == 0) return T(1);
    return A[r + (size_t)(i + l) * lda];
}

// one element global -> shared by cp.async, per real component (complex
// elements need only the alignment of their real type)
template <class T> __device__ __forceinline__ void stage_elem(T *dst, const T *src) {
    typedef typename Tr<T>::R R;
    constexpr int nc = sizeof(T) / sizeof(R);
#pragma unroll
    for (int q = 0; q < nc; ++q) cp_async<sizeof(R)>(reinterpret_cast<R *>(dst) + q, reinterpret_cast<const R *>(src) + q);
}

// VBUF: 0 = V read from global memory, 1 = V_b staged in shared memory before
// its use, 2 = V_{b+1} staged during block b's barriers (double buffer)
template <class T, bool CSMEM, int VBUF> __global__ void __launch_bounds__(kThinThreads) k_multq_thin(ThinArgs<T> p) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int n = p.n, R = p.rows_per_cta, ldcs = R + 4;
    T *sW = reinterpret_cast<T *>(s_dyn);                   // 32 x n (ld 32): V^H C
    T *sY = sW + kPanelMaxCols * n;                         // 32 x n (ld 32): op(T) V^H C
    T *sT = sY + kPanelMaxCols * n;                         // 32 x 33
    T *sV0 = sT + kPanelMaxCols * (kPanelMaxCols + 1);      // 32 x R (ld R)
    T *sV1 = sV0 + (VBUF >= 1 ? (size_t)kPanelMaxCols * R : 0);
    T *sC = sV0 + (size_t)VBUF * kPanelMaxCols * R;         // R x n, column-major (ldcs)
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * R;
    const int r1 = min(p.m, r0 + R);
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;
    auto cref = [&](int r, int c) -> T & {
        if (CSMEM) return sC[(size_t)c * ldcs + (r - r0)];
        return p.C[r + (size_t)c * p.ldc];
    };
    auto block_of = [&](int s) { return p.forward ? s : p.nblk - 1 - s; };
    // rows [max(r0, i_b), r1) of V_b into buf; entries above the diagonal of
    // the block and columns beyond its width as zeros, the diagonal as ones
    auto stage_v = [&](int bb, T *buf) {
        const int i = bb * kPanelMaxCols, ib = min(kPanelMaxCols, p.k - i), rs = max(r0, i);
        if constexpr (std::is_same<T, float>::value) {
            // FP32: 16-byte copies of row quads strictly below the diagonal
            // (block rows start at multiples of 4: rows_per_cta is one), the
            // quads that meet the diagonal or the end element by element
            if (((uintptr_t)p.A % 16 == 0) && (p.lda % 4 == 0) && (R % 4 == 0) && (r0 % 4 == 0)) {
                const int q0 = (rs - r0) / 4, nq = (r1 - r0 + 3) / 4;
                for (int idx = tid; idx < kPanelMaxCols * (nq - q0); idx += kThinThreads) {
                    const int l = idx / (nq - q0), r = r0 + 4 * (q0 + idx % (nq - q0));
                    const T *src = p.A + (size_t)(i + l) * p.lda;
                    T *dst = buf + (size_t)l * R + (r - r0);
                    if (l < ib && r > i + l && r + 4 <= r1) {
                        cp_async_cg16(dst, src + r);
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int rr = r + e;
                            if (rr >= r1 || rr < rs || l >= ib || rr < i + l) dst[e] = T(0);
                            else if (rr == i + l) dst[e] = T(1);
                            else dst[e] = src[rr];
                        }
                    }
                }
                cp_async_commit();
                return;
            }
        }
        // columns outer, rows inner: no index division per element
        for (int l = 0; l < kPanelMaxCols; ++l) {
            const T *src = p.A + (size_t)(i + l) * p.lda;
            T *dcol = buf + (size_t)l * R;
            for (int r = rs + tid; r < r1; r += kThinThreads) {
                T *dst = dcol + (r - r0);
                if (l >= ib || r < i + l) *dst = T(0);
                else if (r == i + l) *dst = T(1);
                else stage_elem(dst, src + r);
            }
        }
        cp_async_commit();
    };
    auto vget = [&](const T *buf, int i, int r, int l) -> T {
        if (VBUF > 0) return buf[(size_t)l * R + (r - r0)];
        return vload(p.A, p.lda, i, r, l);
    };
    if (CSMEM) {
        for (int c = 0; c < n; ++c)
            for (int r = r0 + tid; r < r0 + R; r += kThinThreads) sC[(size_t)c * ldcs + (r - r0)] = (r < r1) ? p.C[r + (size_t)c * p.ldc] : T(0);
    }
    if (VBUF > 0 && p.nblk > 0) stage_v(block_of(0), sV0);

    // FP32 with C and V in shared memory: 4-row quads as float4, 4 x 4
    // register tiles.  Rows past the block's end must read zeros in both: C's
    // are loaded as zeros, V's are written as zeros only by the 16-byte
    // staging (A 16-byte aligned, lda a multiple of 4), so the quads need it.
    constexpr bool kQuads = std::is_same<T, float>::value && CSMEM && VBUF > 0;
    const bool quads = kQuads && (n % 4 == 0) && (R % 4 == 0) && (r0 % 4 == 0) && ((uintptr_t)p.A % 16 == 0) && (p.lda % 4 == 0);
    const int nw = kPanelMaxCols * n;          // entries of V^H C
    const int ctiles = (n + 3) / 4;
    const int ntiles = (kPanelMaxCols / 4) * ctiles;
    const int slice = (nw + G - 1) / G;        // entries this block reduces
    for (int s = 0; s < p.nblk; ++s) {
        const int b = block_of(s);
        const int i = b * kPanelMaxCols;
        const int ib = min(kPanelMaxCols, p.k - i);
        const int rs = max(r0, i);
        const T *sV = (VBUF == 2 && (s & 1)) ? sV1 : sV0;
        if (VBUF > 0) cp_async_wait_all();
        __syncthreads();
        // 1. partial V^H C over own rows; tile t = (reflectors 4*(t % 8) .., columns 4*(t / 8) ..)
        T *mine = p.part + (size_t)g * nw;
        if constexpr (kQuads) {
            if (quads) {
                // tile t per half warp, its 16 lanes over interleaved row quads
                for (int t = 2 * warp + (lane >> 4); t < ntiles; t += 2 * kThinWarps) {
                    const int l0 = 4 * (t % (kPanelMaxCols / 4)), c0 = 4 * (t / (kPanelMaxCols / 4));
                    float acc[16];
#pragma unroll
                    for (int e = 0; e < 16; ++e) acc[e] = 0.f;
                    if (l0 < ib) {
                        for (int r4 = rs + 4 * (lane & 15); r4 < r1; r4 += 64) {
                            float4 v[4], c[4];
#pragma unroll
                            for (int a = 0; a < 4; ++a) v[a] = *reinterpret_cast<const float4 *>(sV + (size_t)(l0 + a) * R + (r4 - r0));
#pragma unroll
                            for (int q = 0; q < 4; ++q) c[q] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + q) * ldcs + (r4 - r0));
#pragma unroll
                            for (int a = 0; a < 4; ++a)
#pragma unroll
                                for (int q = 0; q < 4; ++q) {
                                    float x = acc[4 * a + q];
                                    x = fmaf(v[a].x, c[q].x, x);
                                    x = fmaf(v[a].y, c[q].y, x);
                                    x = fmaf(v[a].z, c[q].z, x);
                                    acc[4 * a + q] = fmaf(v[a].w, c[q].w, x);
                                }
                        }
                    }
                    // sum over the half warp's 16 lanes: lane (& 15) ends with entry (lane & 15)
#pragma unroll
                    for (int lvl = 0; lvl < 4; ++lvl) {
                        const int o = 8 >> lvl, m = 8 >> lvl;
                        const bool up = (lane & o) != 0;
#pragma unroll
                        for (int e = 0; e < m; ++e) {
                            const float send = up ? acc[e] : acc[e + m], keep = up ? acc[e + m] : acc[e];
                            acc[e] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                        }
                    }
                    const int e = lane & 15;
                    if (c0 + (e & 3) < n) mine[(l0 + (e >> 2)) + (size_t)(c0 + (e & 3)) * kPanelMaxCols] = acc[0];
                }
            }
        }
        for (int t = warp; t < ntiles && !quads; t += kThinWarps) {
            const int l0 = 4 * (t % (kPanelMaxCols / 4)), c0 = 4 * (t / (kPanelMaxCols / 4));
            T acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[a][q] = T(0);
            if (l0 < ib) {
                for (int r = rs + lane; r < r1; r += 32) {
                    T v[4], c[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) v[a] = (VBUF > 0 || l0 + a < ib) ? Tr<T>::conj(vget(sV, i, r, l0 + a)) : T(0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = (c0 + q < n) ? cref(r, c0 + q) : T(0);
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[a][q] = fmac(v[a], c[q], acc[a][q]);
                }
            }
            // entry e = 4 a + q of the tile, summed over the warp's lanes
            T v[16];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int q = 0; q < 4; ++q) v[4 * a + q] = acc[a][q];
            const int e = warp_reduce16(v, lane);
            if ((lane & 1) == 0) {
                const int a = e >> 2, q = e & 3;
                if (c0 + q < n) mine[(l0 + a) + (size_t)(c0 + q) * kPanelMaxCols] = v[0];
            }
        }
        // the next block's V streams in while this one waits at the barriers
        if (VBUF == 2 && s + 1 < p.nblk) stage_v(block_of(s + 1), (s & 1) ? sV0 : sV1);
        if (!bar.sync()) return;
        // T_b (the previous step's Y is done with sT): its loads overlap the
        // reduction and the second barrier
        const T *Tb = p.Tf + (size_t)b * kPanelMaxCols * kPanelMaxCols;
        for (int e = tid; e < kPanelMaxCols * kPanelMaxCols; e += kThinThreads) {
            const int r = e % kPanelMaxCols, c = e / kPanelMaxCols;
            sT[r * (kPanelMaxCols + 1) + c] = (r <= c && c < ib) ? Tb[r + (size_t)c * kPanelMaxCols] : T(0);
        }
        // 3. this block's slice of the reduction, fixed order over blocks
        for (int e = g * slice + warp; e < min(nw, (g + 1) * slice); e += kThinWarps) {
            T a = T(0);
            for (int q = lane; q < G; q += 32) a = a + ldcg(&p.part[(size_t)q * nw + e]);
            a = warp_sum(a);
            if (lane == 0) p.wred[e] = a;
        }
        if (!bar.sync()) return;
        // 4. Y = op(T) (V^H C)
        for (int e = tid; e < nw; e += kThinThreads) sW[e] = ldcg(&p.wred[e]);
        __syncthreads();
        for (int e = tid; e < nw; e += kThinThreads) {
            const int l = e % kPanelMaxCols, c = e / kPanelMaxCols;
            T acc = T(0);
            if (l < ib) {
                if (p.forward) {
                    // (T^H W)(l, c) = sum_{j <= l} conj(T(j, l)) W(j, c)
                    for (int j = 0; j <= l; ++j) acc = fmac(Tr<T>::conj(sT[j * (kPanelMaxCols + 1) + l]), sW[j + c * kPanelMaxCols], acc);
                } else {
                    // (T W)(l, c) = sum_{j >= l} T(l, j) W(j, c)
                    for (int j = l; j < ib; ++j) acc = fmac(sT[l * (kPanelMaxCols + 1) + j], sW[j + c * kPanelMaxCols], acc);
                }
            }
            if (quads) sY[l * n + c] = acc;  // row-major for the quad update
            else sY[e] = acc;
        }
        __syncthreads();
        // 5. C(r, c) -= sum_l V(r, l) Y(l, c) on own rows
        if constexpr (kQuads) {
            if (quads) {
                const int nq = (r1 - rs + 3) / 4;
                for (int w = tid; w < nq * ctiles; w += kThinThreads) {
                    const int r4 = rs + 4 * (w % nq), c0 = 4 * (w / nq);
                    float4 acc[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[q] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + q) * ldcs + (r4 - r0));
                    const int lmax = min(ib, r4 + 4 - i);  // V(r, l) = 0 for l > r - i
                    for (int l = 0; l < lmax; ++l) {
                        const float4 v = *reinterpret_cast<const float4 *>(sV + (size_t)l * R + (r4 - r0));
                        const float4 y = *reinterpret_cast<const float4 *>(sY + (size_t)l * n + c0);
                        const float yq[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            acc[q].x = fmaf(-v.x, yq[q], acc[q].x);
                            acc[q].y = fmaf(-v.y, yq[q], acc[q].y);
                            acc[q].z = fmaf(-v.z, yq[q], acc[q].z);
                            acc[q].w = fmaf(-v.w, yq[q], acc[q].w);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) *reinterpret_cast<float4 *>(sC + (size_t)(c0 + q) * ldcs + (r4 - r0)) = acc[q];
                }
            }
        }
        const int nrc = (r1 > rs && !quads) ? (r1 - rs + 31) / 32 : 0;
        for (int w = warp; w < nrc * ctiles; w += kThinWarps) {
            const int rc = w % nrc, c0 = 4 * (w / nrc);
            const int r = rs + rc * 32 + lane;
            if (r < r1) {
                T acc[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[q] = (c0 + q < n) ? cref(r, c0 + q) : T(0);
                const int lmax = min(ib, r - i + 1);  // V(r, l) = 0 for l > r - i
                for (int l0 = 0; l0 < lmax; l0 += 8) {
                    T v[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) v[u] = (l0 + u < lmax) ? -vget(sV, i, r, l0 + u) : T(0);
#pragma unroll
                    for (int u = 0; u < 8; ++u)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] = fmac(v[u], sY[l0 + u + min(c0 + q, n - 1) * kPanelMaxCols], acc[q]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (c0 + q < n) cref(r, c0 + q) = acc[q];
            }
        }
        if (VBUF == 1 && s + 1 < p.nblk) {
            __syncthreads();
            stage_v(block_of(s + 1), sV0);
        }
    }
    __syncthreads();
    if (CSMEM) {
        for (int c = 0; c < n; ++c)
            for (int r = r0 + tid; r < r1; r += kThinThreads) p.C[r + (size_t)c * p.ldc] = sC[(size_t)c * ldcs + (r - r0)];
    }
}

// ---------------------------------------------------------------------------
// The same product when the reflectors cover most of C's rows (k close to m):
// a fixed row range per block would leave the blocks above the current
// reflector block idle, so here every reflector block's active rows
// [i_b, m) are split evenly over all blocks (C stays in global memory, read
// through L2 after the barrier that makes the previous block's updates
// visible).  The block stages its rows of V_b and C in shared memory and
// forms V_b^H C and the update with one output per thread and no warp
// reductions (the shuffle reductions of the tiled form cost more FP64 work
// than the products when a block holds few rows).  Shared memory holds the
// largest such row range (rows_per_cta = ceil(m / gridDim.x)) of V and C.
// ---------------------------------------------------------------------------
template <class T> inline size_t thin_dyn_smem_bytes(int rmax, int n) {
    return ((size_t)2 * kPanelMaxCols * n + (size_t)kPanelMaxCols * (kPanelMaxCols + 1) + (size_t)rmax * (kPanelMaxCols + 1) + (size_t)rmax * n) * sizeof(T);
}

template <class T> __global__ void __launch_bounds__(kThinThreads) k_multq_thin_dyn(ThinArgs<T> p) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int n = p.n, RMAX = p.rows_per_cta;
    T *sW = reinterpret_cast<T *>(s_dyn);                   // 32 x n (ld 32)
    T *sY = sW + kPanelMaxCols * n;                         // 32 x n (ld 32)
    T *sT = sY + kPanelMaxCols * n;                         // 32 x 33
    T *sV = sT + kPanelMaxCols * (kPanelMaxCols + 1);       // 32 x RMAX+1 ... stored [l][r], ld RMAX + 1
    T *sC = sV + (size_t)kPanelMaxCols * (RMAX + 1);        // n x RMAX, stored [c][r], ld RMAX
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ldv = RMAX + 1;
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;
    const int nw = kPanelMaxCols * n;
    const int slice = (nw + G - 1) / G;
    for (int s = 0; s < p.nblk; ++s) {
        const int b = p.forward ? s : p.nblk - 1 - s;
        const int i = b * kPanelMaxCols;
        const int ib = min(kPanelMaxCols, p.k - i);
        const int rb = (p.m - i + G - 1) / G;                  // rows per block for this reflector block
        const int r0 = min(p.m, i + g * rb), r1 = min(p.m, r0 + rb), nr = r1 - r0;
        // the previous reflector block's updates (by other blocks) are visible
        if (s > 0 && !bar.sync()) return;
        // stage V_b (stored form) and C for rows [r0, r1)
        for (int e = tid; e < nr * kPanelMaxCols; e += kThinThreads) {
            const int rr = e % nr, l = e / nr, r = r0 + rr;
            sV[l * ldv + rr] = (l < ib) ? vload(p.A, p.lda, i, r, l) : T(0);
        }
        for (int e = tid; e < nr * n; e += kThinThreads) {
            const int rr = e % nr, c = e / nr;
            sC[(size_t)c * RMAX + rr] = ldcg(&p.C[(r0 + rr) + (size_t)c * p.ldc]);
        }
        __syncthreads();
        // 1. partial V^H C: one (reflector, column) entry per thread and step
        T *mine = p.part + (size_t)g * nw;
        for (int e = tid; e < nw; e += kThinThreads) {
            const int l = e % kPanelMaxCols, c = e / kPanelMaxCols;
            T acc = T(0);
            if (l < ib)
                for (int rr = 0; rr < nr; ++rr) acc = fmac(Tr<T>::conj(sV[l * ldv + rr]), sC[(size_t)c * RMAX + rr], acc);
            mine[e] = acc;
        }
        if (!bar.sync()) return;
        // 2. this block's slice of the reduction, fixed order over blocks
        for (int e = g * slice + warp; e < min(nw, (g + 1) * slice); e += kThinWarps) {
            T a = T(0);
            for (int q = lane; q < G; q += 32) a = a + ldcg(&p.part[(size_t)q * nw + e]);
            a = warp_sum(a);
            if (lane == 0) p.wred[e] = a;
        }
        if (!bar.sync()) return;
        // 3. Y = op(T) (V^H C)
        for (int e = tid; e < nw; e += kThinThreads) sW[e] = ldcg(&p.wred[e]);
        const T *Tb = p.Tf + (size_t)b * kPanelMaxCols * kPanelMaxCols;
        for (int e = tid; e < kPanelMaxCols * kPanelMaxCols; e += kThinThreads) {
            const int r = e % kPanelMaxCols, c = e / kPanelMaxCols;
            sT[r * (kPanelMaxCols + 1) + c] = (r <= c && c < ib) ? Tb[r + (size_t)c * kPanelMaxCols] : T(0);
        }
        __syncthreads();
        for (int e = tid; e < nw; e += kThinThreads) {
            const int l = e % kPanelMaxCols, c = e / kPanelMaxCols;
            T acc = T(0);
            if (l < ib) {
                if (p.forward) {
                    for (int j = 0; j <= l; ++j) acc = fmac(Tr<T>::conj(sT[j * (kPanelMaxCols + 1) + l]), sW[j + c * kPanelMaxCols], acc);
                } else {
                    for (int j = l; j < ib; ++j) acc = fmac(sT[l * (kPanelMaxCols + 1) + j], sW[j + c * kPanelMaxCols], acc);
                }
            }
            sY[e] = acc;
        }
        __syncthreads();
        // 4. C(r, c) -= sum_l V(r, l) Y(l, c): one entry per thread and step
        for (int e = tid; e < nr * n; e += kThinThreads) {
            const int rr = e % nr, c = e / nr;
            T acc = sC[(size_t)c * RMAX + rr];
            for (int l = 0; l < ib; ++l) acc = fmac(-sV[l * ldv + rr], sY[l + c * kPanelMaxCols], acc);
            p.C[(r0 + rr) + (size_t)c * p.ldc] = acc;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Gram matrices V_b^H V_b of all reflector blocks, split over row chunks:
// block (s, b) sums rows [i_b + s*chunk, i_b + (s+1)*chunk) of block b and
// writes the 32 x 32 partial at P + (b * S + s) * 32 * 32 (leading dimension
// 32).  k_build_t then runs the GenerateBlockTr recurrence on every block.
// ---------------------------------------------------------------------------
template <class T> __global__ void __launch_bounds__(256) k_gram_blocks(const T *A, size_t lda, int m, int k, int chunk, T *P) {
    __shared__ T sV[64][kPanelMaxCols + 1];
    const int s = blockIdx.x, b = blockIdx.y, S = gridDim.x, tid = threadIdx.x;
    const int i = b * kPanelMaxCols;
    const int ib = min(kPanelMaxCols, k - i);
    const int rb = i + s * chunk, re = min(m, rb + chunk);
    // thread: row l1 = tid % 32 of the Gram matrix, columns l2 = tid / 32 + 8 q
    const int l1 = tid % kPanelMaxCols, lq = tid / kPanelMaxCols;
    T acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = T(0);
    for (int c0 = rb; c0 < re; c0 += 64) {
        const int rows = min(64, re - c0);
        __syncthreads();
        for (int e = tid; e < 64 * kPanelMaxCols; e += 256) {
            const int r = e % 64, l = e / 64;
            sV[r][l] = (r < rows && l < ib) ? vload(A, lda, i, c0 + r, l) : T(0);
        }
        __syncthreads();
        for (int r = 0; r < rows; ++r) {
            const T a = Tr<T>::conj(sV[r][l1]);
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fmac(a, sV[r][lq + 8 * q], acc[q]);
        }
    }
    T *out = P + ((size_t)b * S + s) * kPanelMaxCols * kPanelMaxCols;
#pragma unroll
    for (int q = 0; q < 4; ++q) out[l1 + (size_t)(lq + 8 * q) * kPanelMaxCols] = acc[q];
}


// ---------------------------------------------------------------------------
// Q^T C for a thin FP32 C (at most kQtcMaxCols columns) with wide reflector
// blocks: the same one-launch structure as k_multq_thin, but a reflector
// block may be 128 columns wide when its 128 x 128 T is at hand (the mixed
// factor's tensor-core path forms one per 128-column block), so that a
// 512-column Q takes 3 + 4 steps of two grid barriers instead of 16.  Each
// step (columns [i, i + w), T_s) is
//   1. W = V_s^T C over the block's rows, 32 reflectors (one staged chunk of
//      V) at a time,
//   2./3. the cross-block sum (two grid barriers, fixed order),
//   4. Y = T_s^T W (T_s staged in shared memory during the barriers),
//   5. C -= V_s Y, chunk by chunk.
// V's 32-column chunks (the block's rows of 32 columns, one bulk copy per
// column, completing on the buffer's mbarrier) stream through two buffers in
// the order they are used (a 32-column step keeps its chunk for both
// phases), so that each copy overlaps the previous chunk's work or the
// barriers; the triangle of the chunk (zeros above the diagonal, ones on it)
// is written over the copied rows by the block that holds them.  C's rows
// stay in shared memory for the whole launch (columns padded to a multiple
// of 4 with zeros).  Requires A 16-byte aligned, lda and m multiples of 4.
// Every wait is bounded.
// ---------------------------------------------------------------------------
constexpr int kQtcMaxW = 128;
constexpr int kQtcMaxCols = 16;
constexpr size_t kQtcSmemMax = 226 * 1024;
struct QtcArgs {
    const float *A;
    size_t lda;
    const float *Tf;    // 32-column panel T's: panel p at Tf + p * 32 * 32 (column-major, ld 32)
    const float *T128;  // 128-column block T's: block b at T128 + b * 128 * 128 (row-major, ld 128)
    float *C;
    size_t ldc;
    int m, n, k, nwide;
    float *part;        // [gridDim.x][kQtcMaxW * nq]
    float *wred;        // [kQtcMaxW * nq]
    unsigned *counter;
    int *err;
    int *status;
    int rows_per_cta;
};
inline size_t qtc_smem_bytes(int rows, int nq) {
    return ((size_t)2 * kQtcMaxW * nq + (size_t)kQtcMaxW * kQtcMaxW + (size_t)2 * kPanelMaxCols * rows + (size_t)(rows + 4) * nq) * sizeof(float);
}

namespace qtc {
__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t *b) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(b)) : "memory"); }
__device__ __forceinline__ void bar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// the generic proxy's accesses to a buffer before the async proxy writes it
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void arrive_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void copy(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)), "l"(src), "r"(bytes), "r"(saddr(b)) : "memory");
}
// bounded wait for the phase of the given parity
__device__ __forceinline__ bool wait(uint64_t *b, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n" : "=r"(done) : "r"(saddr(b)), "r"(parity) : "memory");
        if (done) return true;
        if (clock64() - t0 > 2000000000LL) return false;
    }
}
} // namespace qtc

template <int kTag> __global__ void __launch_bounds__(kThinThreads) k_qtc_blocks(QtcArgs p) {
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ __align__(8) uint64_t s_bar[3];  // V buffers 0 and 1, T
    const int n = p.n, nq = (n + 3) & ~3, R = p.rows_per_cta, ldcs = R + 4;
    float *sT = reinterpret_cast<float *>(s_dyn);           // T_s as stored (row- or column-major)
    float *sW = sT + kQtcMaxW * kQtcMaxW;                   // W(l, c) at l * nq + c
    float *sY = sW + kQtcMaxW * nq;                         // Y(l, c) at l * nq + c
    float *sV0 = sY + kQtcMaxW * nq;                        // two chunks, 32 x R each (ld R)
    float *sC = sV0 + (size_t)2 * kPanelMaxCols * R;        // R x nq, column-major (ldcs)
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * R;
    const int r1 = min(p.m, r0 + R);
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;
    const int wide_cols = kQtcMaxW * p.nwide;
    const int nsteps = p.nwide + (p.k - wide_cols + kPanelMaxCols - 1) / kPanelMaxCols;
    auto step_i = [&](int s) { return s < p.nwide ? kQtcMaxW * s : wide_cols + kPanelMaxCols * (s - p.nwide); };
    auto step_w = [&](int s) { return s < p.nwide ? kQtcMaxW : min(kPanelMaxCols, p.k - step_i(s)); };
    auto vbuf = [&](int b) { return sV0 + (size_t)b * kPanelMaxCols * R; };
    uint32_t par0 = 0, par1 = 0, part = 0;
    auto fail = [&]() {
        atomicExch(p.err, (int)kStatusBarrierTimeout);
        if (p.status) atomicExch(p.status, (int)kStatusBarrierTimeout);
    };
    // warp 0: rows [max(r0, ic), r1) of reflector columns [ic, ic + wc) into
    // buffer b, one bulk copy per column from lane l (the block's earlier
    // accesses to the buffer are ordered before by a block barrier)
    auto stage = [&](int ic, int wc, int b) {
        if (warp != 0) return;
        qtc::proxy_fence();
        const int rs = max(r0, ic);
        const uint32_t bytes = rs < r1 ? (uint32_t)(r1 - rs) * 4u : 0u;
        if (lane == 0) qtc::arrive_tx(&s_bar[b], bytes * (uint32_t)wc);
        __syncwarp();
        if (bytes && lane < wc) qtc::copy(vbuf(b) + (size_t)lane * R + (rs - r0), p.A + (size_t)(ic + lane) * p.lda + rs, bytes, &s_bar[b]);
    };
    // the chunk after (s, ph, q) in the order of use: phase 0 (W) chunks, then
    // phase 1 (update) chunks when the step has more than one
    auto stage_next = [&](int s, int ph, int q, int b) {
        const int nchk = (step_w(s) + kPanelMaxCols - 1) / kPanelMaxCols;
        if (q + 1 < nchk) {
            ++q;
        } else if (ph == 0 && nchk > 1) {
            ph = 1;
            q = 0;
        } else {
            ++s;
            q = 0;
            if (s >= nsteps) return;
        }
        const int ic = step_i(s) + kPanelMaxCols * q;
        stage(ic, min(kPanelMaxCols, step_i(s) + step_w(s) - ic), b);
    };
    // wait for chunk (ic, wc) in buffer b, then write its triangle: zeros
    // above the diagonal, ones on it (rows [ic, ic + wc) that this block holds)
    auto land = [&](int ic, int wc, int b) -> bool {
        uint32_t &par = b ? par1 : par0;
        if (!qtc::wait(&s_bar[b], par)) return false;
        par ^= 1u;
        const int t0 = max(r0, ic), t1 = min(r1, ic + wc);
        if (t0 < t1) {
            float *buf = vbuf(b);
            for (int e = tid; e < wc * (t1 - t0); e += kThinThreads) {
                const int l = e / (t1 - t0), rr = t0 + e % (t1 - t0);
                if (rr <= ic + l) buf[(size_t)l * R + (rr - r0)] = (rr == ic + l) ? 1.f : 0.f;
            }
        }
        return true;
    };
    if (tid == 0) {
        qtc::bar_init(&s_bar[0]);
        qtc::bar_init(&s_bar[1]);
        qtc::bar_init(&s_bar[2]);
        qtc::bar_init_fence();
    }
    for (int c = 0; c < nq; ++c)
        for (int r = r0 + tid; r < r0 + R; r += kThinThreads) sC[(size_t)c * ldcs + (r - r0)] = (r < r1 && c < n) ? p.C[r + (size_t)c * p.ldc] : 0.f;
    __syncthreads();
    int ck = 0;  // chunks consumed so far: chunk ck sits in buffer ck & 1
    if (nsteps > 0) stage(step_i(0), min(kPanelMaxCols, step_w(0)), 0);
    const int ctiles = nq / 4;
    bool ok = true;
    for (int s = 0; s < nsteps && ok; ++s) {
        const int i = step_i(s), w = step_w(s);
        const int nchk = (w + kPanelMaxCols - 1) / kPanelMaxCols;
        const int nw = w * nq;
        float *mine = p.part + (size_t)g * kQtcMaxW * nq;
        // 1. partial W = V^T C over own rows, one chunk of 32 reflectors at a time
        for (int q = 0; q < nchk; ++q, ++ck) {
            const int ic = i + kPanelMaxCols * q, wc = min(kPanelMaxCols, i + w - ic);
            if (!land(ic, wc, ck & 1)) { ok = false; break; }
            __syncthreads();
            stage_next(s, 0, q, (ck + 1) & 1);
            const float *sV = vbuf(ck & 1);
            const int rs = max(r0, ic);
            // tile t per half warp: reflectors 4 (t % 8) .., columns 4 (t / 8) ..
            for (int t = 2 * warp + (lane >> 4); t < 8 * ctiles; t += 2 * kThinWarps) {
                const int l0 = 4 * (t % 8), c0 = 4 * (t / 8);
                float acc[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) acc[e] = 0.f;
                // (every lane takes part in the shuffles below, whatever l0)
                for (int r4 = rs + 4 * (lane & 15); l0 < wc && r4 < r1; r4 += 64) {
                    float4 v[4], c[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) v[a] = *reinterpret_cast<const float4 *>(sV + (size_t)(l0 + a) * R + (r4 - r0));
#pragma unroll
                    for (int qq = 0; qq < 4; ++qq) c[qq] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0));
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int qq = 0; qq < 4; ++qq) {
                            float x = acc[4 * a + qq];
                            x = fmaf(v[a].x, c[qq].x, x);
                            x = fmaf(v[a].y, c[qq].y, x);
                            x = fmaf(v[a].z, c[qq].z, x);
                            acc[4 * a + qq] = fmaf(v[a].w, c[qq].w, x);
                        }
                }
                // butterfly over the half warp: lane (& 15) ends with entry (lane & 15)
#pragma unroll
                for (int lvl = 0; lvl < 4; ++lvl) {
                    const int o = 8 >> lvl, mm = 8 >> lvl;
                    const bool up = (lane & o) != 0;
#pragma unroll
                    for (int e = 0; e < mm; ++e) {
                        const float send = up ? acc[e] : acc[e + mm], keep = up ? acc[e + mm] : acc[e];
                        acc[e] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                    }
                }
                const int e = lane & 15, l = l0 + (e >> 2);
                if (l < wc) mine[(ic - i + l) + (size_t)(c0 + (e & 3)) * kQtcMaxW] = acc[0];
            }
        }
        if (!ok) break;
        if (nchk == 1) --ck;  // the step keeps its one chunk for the update
        if (!bar.sync()) return;
        // T_s into shared memory while the blocks sum and wait (the previous
        // step's Y is done with sT: block barriers since)
        const bool wide = s < p.nwide;
        if (tid == 0) {
            qtc::proxy_fence();
            const float *src = wide ? p.T128 + (size_t)s * kQtcMaxW * kQtcMaxW : p.Tf + (size_t)(i / kPanelMaxCols) * kPanelMaxCols * kPanelMaxCols;
            const uint32_t bytes = (uint32_t)(wide ? kQtcMaxW * kQtcMaxW : kPanelMaxCols * kPanelMaxCols) * 4u;
            qtc::arrive_tx(&s_bar[2], bytes);
            qtc::copy(sT, src, bytes, &s_bar[2]);
        }
        // 3. this block's slice of the cross-block sum, fixed order over blocks
        const int slice = (nw + G - 1) / G;
        for (int e = g * slice + warp; e < min(nw, (g + 1) * slice); e += kThinWarps) {
            const int idx = (e % w) + (e / w) * kQtcMaxW;
            // the lane's partials in flight together (G <= 256), summed in order
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = (lane + 32 * u < G) ? ldcg(&p.part[(size_t)(lane + 32 * u) * kQtcMaxW * nq + idx]) : 0.f;
            float a = 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (lane + 32 * u < G) a += v[u];
            a = warp_sum(a);
            if (lane == 0) p.wred[idx] = a;
        }
        if (!bar.sync()) return;
        // 4. Y = T^T W: Y(l, c) = sum_{j <= l} T(j, l) W(j, c)
        for (int e = tid; e < nw; e += kThinThreads) {
            const int l = e % w, c = e / w;
            sW[l * nq + c] = ldcg(&p.wred[l + c * kQtcMaxW]);
        }
        if (!qtc::wait(&s_bar[2], part)) { ok = false; break; }
        part ^= 1u;
        __syncthreads();
        {
            const int tr = wide ? kQtcMaxW : 1, tc = wide ? 1 : kPanelMaxCols;  // T(j, l) at sT[j tr + l tc]
            for (int e = tid; e < nw; e += kThinThreads) {
                const int l = e / nq, c = e % nq;
                const float *tl = sT + l * tc;
                const float *wcol = sW + c;  // W(j, c) at wcol[j nq]
                float a0 = 0.f, a1 = 0.f;
                int j = 0;
                for (; j + 1 <= l; j += 2) {
                    a0 = fmaf(tl[j * tr], wcol[j * nq], a0);
                    a1 = fmaf(tl[(j + 1) * tr], wcol[(j + 1) * nq], a1);
                }
                if (j <= l) a0 = fmaf(tl[j * tr], wcol[j * nq], a0);
                sY[l * nq + c] = a0 + a1;
            }
        }
        // 5. C -= V Y on own rows, chunk by chunk
        for (int q = 0; q < nchk; ++q, ++ck) {
            const int ic = i + kPanelMaxCols * q, wc = min(kPanelMaxCols, i + w - ic);
            if (nchk > 1) {
                if (!land(ic, wc, ck & 1)) { ok = false; break; }
                __syncthreads();
                stage_next(s, 1, q, (ck + 1) & 1);
            } else {
                __syncthreads();  // sY complete; the next step's first chunk is already on its way
            }
            const float *sV = vbuf(ck & 1);
            const int rs = max(r0, ic);
            const int nqr = (r1 - rs + 3) / 4;
            for (int u = tid; u < nqr * ctiles; u += kThinThreads) {
                const int r4 = rs + 4 * (u % nqr), c0 = 4 * (u / nqr);
                float4 acc[4];
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) acc[qq] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0));
                const int lmax = min(wc, r4 + 4 - ic);  // V(r, l) = 0 for l > r - ic
                for (int l = 0; l < lmax; ++l) {
                    const float4 v = *reinterpret_cast<const float4 *>(sV + (size_t)l * R + (r4 - r0));
                    const float4 y = *reinterpret_cast<const float4 *>(sY + (size_t)(ic - i + l) * nq + c0);
                    const float yq[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                    for (int qq = 0; qq < 4; ++qq) {
                        acc[qq].x = fmaf(-v.x, yq[qq], acc[qq].x);
                        acc[qq].y = fmaf(-v.y, yq[qq], acc[qq].y);
                        acc[qq].z = fmaf(-v.z, yq[qq], acc[qq].z);
                        acc[qq].w = fmaf(-v.w, yq[qq], acc[qq].w);
                    }
                }
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) *reinterpret_cast<float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0)) = acc[qq];
            }
        }
    }
    if (!ok) {
        // a copy did not land in time: stop every block, let the copies in
        // flight finish (bounded), leave C as it was
        fail();
        qtc::wait(&s_bar[0], par0);
        qtc::wait(&s_bar[1], par1);
        return;
    }
    __syncthreads();
    for (int c = 0; c < n; ++c)
        for (int r = r0 + tid; r < r1; r += kThinThreads) p.C[r + (size_t)c * p.ldc] = sC[(size_t)c * ldcs + (r - r0)];
}

// ---------------------------------------------------------------------------
// One block reflector (K <= 32 columns, compact WY with T) applied from the
// left to an FP32 C of at most kA32MaxCols columns in one cooperative launch:
// C -= V (T^T (V^T C)), the mixed factor's updates inside a 128-column block.
// Every block copies its rows of V and C into shared memory once (bulk
// copies on one mbarrier), forms its part of V^T C (4 x 4 tiles per half
// warp, as k_qtc_blocks), the blocks sum the partials (two grid barriers,
// fixed order), then each block forms Y = T^T W and updates and stores its
// rows of C.  One launch instead of three (W partials, their sum times T, the
// update), C read and written once.  Requires V and C 16-byte aligned,
// ldv, ldc and M multiples of 4.
// ---------------------------------------------------------------------------
constexpr int kA32MaxCols = 64;
struct A32Args {
    const float *V;
    size_t ldv;
    const float *T;  // K x K upper (column-major, leading dimension 32)
    float *C;
    size_t ldc;
    int M, N, K;
    float *part;     // [gridDim.x][32 * N]
    float *wred;     // [32 * N]
    unsigned *counter;
    int *err;
    int *status;
    int rows_per_cta;
};
inline size_t a32_smem_bytes(int rows, int n) { return ((size_t)2 * kPanelMaxCols * n + (size_t)kPanelMaxCols * rows + (size_t)(rows + 4) * n) * sizeof(float); }

template <int kTag> __global__ void __launch_bounds__(kThinThreads) k_apply32(A32Args p) {
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ __align__(8) uint64_t s_bar;
    const int N = p.N, K = p.K, R = p.rows_per_cta, ldcs = R + 4;
    float *sW = reinterpret_cast<float *>(s_dyn);           // W(l, c) at l * N + c
    float *sY = sW + kPanelMaxCols * N;                     // Y(l, c) at l * N + c
    float *sV = sY + kPanelMaxCols * N;                     // 32 x R (ld R)
    float *sC = sV + (size_t)kPanelMaxCols * R;             // R x N, column-major (ldcs)
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * R;
    const int r1 = min(p.M, r0 + R);
    GridBarrier bar{p.counter, p.err, (unsigned)G, 0u};
    bar.status = p.status;
    if (tid == 0) {
        qtc::bar_init(&s_bar);
        qtc::bar_init_fence();
    }
    __syncthreads();
    // warp 0: the block's rows of the K columns of V and the N columns of C
    if (warp == 0) {
        const uint32_t bytes = r0 < r1 ? (uint32_t)(r1 - r0) * 4u : 0u;
        if (lane == 0) qtc::arrive_tx(&s_bar, bytes * (uint32_t)(K + N));
        __syncwarp();
        if (bytes) {
            for (int c = lane; c < K + N; c += 32) {
                if (c < K) qtc::copy(sV + (size_t)c * R, p.V + (size_t)c * p.ldv + r0, bytes, &s_bar);
                else qtc::copy(sC + (size_t)(c - K) * ldcs, p.C + (size_t)(c - K) * p.ldc + r0, bytes, &s_bar);
            }
        }
    }
    // rows past r1 (the last block) read as zeros; V's columns past K too
    for (int e = tid; e < N * (r0 + R - max(r1, r0)); e += kThinThreads) {
        const int nr = r0 + R - max(r1, r0);
        sC[(size_t)(e / nr) * ldcs + (max(r1, r0) - r0) + e % nr] = 0.f;
    }
    for (int e = tid; e < kPanelMaxCols * R; e += kThinThreads) {
        const int l = e / R, rr = r0 + e % R;
        if (l >= K || rr >= r1) sV[e] = 0.f;
    }
    if (!qtc::wait(&s_bar, 0)) {
        // the copies did not land in time: stop every block, let them finish (bounded)
        atomicExch(p.err, (int)kStatusBarrierTimeout);
        if (p.status) atomicExch(p.status, (int)kStatusBarrierTimeout);
        qtc::wait(&s_bar, 0);
        return;
    }
    // the triangle of V: zeros above the diagonal, ones on it
    for (int e = tid; e < K * (min(r1, K) - r0); e += kThinThreads) {
        const int nr = min(r1, K) - r0, l = e / nr, rr = r0 + e % nr;
        if (rr <= l) sV[(size_t)l * R + (rr - r0)] = (rr == l) ? 1.f : 0.f;
    }
    __syncthreads();
    const int ctiles = N / 4, nw = K * N;
    float *mine = p.part + (size_t)g * kPanelMaxCols * N;
    // 1. partial W = V^T C over own rows: tile t per half warp, reflectors
    // 4 (t % 8) .., columns 4 (t / 8) ..
    for (int t = 2 * warp + (lane >> 4); t < 8 * ctiles; t += 2 * kThinWarps) {
        const int l0 = 4 * (t % 8), c0 = 4 * (t / 8);
        float acc[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[e] = 0.f;
        for (int r4 = r0 + 4 * (lane & 15); l0 < K && r4 < r1; r4 += 64) {
            float4 v[4], c[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) v[a] = *reinterpret_cast<const float4 *>(sV + (size_t)(l0 + a) * R + (r4 - r0));
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) c[qq] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0));
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    float x = acc[4 * a + qq];
                    x = fmaf(v[a].x, c[qq].x, x);
                    x = fmaf(v[a].y, c[qq].y, x);
                    x = fmaf(v[a].z, c[qq].z, x);
                    acc[4 * a + qq] = fmaf(v[a].w, c[qq].w, x);
                }
        }
#pragma unroll
        for (int lvl = 0; lvl < 4; ++lvl) {
            const int o = 8 >> lvl, mm = 8 >> lvl;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int e = 0; e < mm; ++e) {
                const float send = up ? acc[e] : acc[e + mm], keep = up ? acc[e + mm] : acc[e];
                acc[e] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
        }
        const int e = lane & 15, l = l0 + (e >> 2);
        if (l < K) mine[l + (size_t)(c0 + (e & 3)) * kPanelMaxCols] = acc[0];
    }
    if (!bar.sync()) return;
    // 2. this block's slice of the cross-block sum, fixed order over blocks
    const int slice = (nw + G - 1) / G;
    for (int e = g * slice + warp; e < min(nw, (g + 1) * slice); e += kThinWarps) {
        const int idx = (e % K) + (e / K) * kPanelMaxCols;
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (lane + 32 * u < G) ? ldcg(&p.part[(size_t)(lane + 32 * u) * kPanelMaxCols * N + idx]) : 0.f;
        float a = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (lane + 32 * u < G) a += v[u];
        a = warp_sum(a);
        if (lane == 0) p.wred[idx] = a;
    }
    if (!bar.sync()) return;
    // 3. Y = T^T W: Y(l, c) = sum_{j <= l} T(j, l) W(j, c)
    for (int e = tid; e < nw; e += kThinThreads) {
        const int l = e % K, c = e / K;
        sW[l * N + c] = ldcg(&p.wred[l + c * kPanelMaxCols]);
    }
    __syncthreads();
    for (int e = tid; e < kPanelMaxCols * N; e += kThinThreads) {
        const int l = e / N, c = e % N;
        float a0 = 0.f, a1 = 0.f;
        if (l < K) {
            const float *tl = p.T + (size_t)l * kPanelMaxCols;
            int j = 0;
            for (; j + 1 <= l; j += 2) {
                a0 = fmaf(__ldg(tl + j), sW[j * N + c], a0);
                a1 = fmaf(__ldg(tl + j + 1), sW[(j + 1) * N + c], a1);
            }
            if (j <= l) a0 = fmaf(__ldg(tl + j), sW[j * N + c], a0);
        }
        sY[l * N + c] = a0 + a1;
    }
    __syncthreads();
    // 4. C -= V Y on own rows, then the rows back to global memory
    const int nqr = (r1 - r0 + 3) / 4;
    for (int u = tid; u < nqr * ctiles; u += kThinThreads) {
        const int r4 = r0 + 4 * (u % nqr), c0 = 4 * (u / nqr);
        float4 acc[4];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) acc[qq] = *reinterpret_cast<const float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0));
        const int lmax = min(K, r4 + 4);  // V(r, l) = 0 for l > r
        for (int l = 0; l < lmax; ++l) {
            const float4 v = *reinterpret_cast<const float4 *>(sV + (size_t)l * R + (r4 - r0));
            const float4 y = *reinterpret_cast<const float4 *>(sY + (size_t)l * N + c0);
            const float yq[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
                acc[qq].x = fmaf(-v.x, yq[qq], acc[qq].x);
                acc[qq].y = fmaf(-v.y, yq[qq], acc[qq].y);
                acc[qq].z = fmaf(-v.z, yq[qq], acc[qq].z);
                acc[qq].w = fmaf(-v.w, yq[qq], acc[qq].w);
            }
        }
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) *reinterpret_cast<float4 *>(sC + (size_t)(c0 + qq) * ldcs + (r4 - r0)) = acc[qq];
    }
    __syncthreads();
    for (int c = 0; c < N; ++c)
        for (int r = r0 + tid; r < r1; r += kThinThreads) p.C[r + (size_t)c * p.ldc] = sC[(size_t)c * ldcs + (r - r0)];
}

} // namespace rnpgpu
