// update_f32.cuh — the FP32 trailing update of the blocked factorization
// (RNP/LA/Reflector.hpp:725-815, ApplyBlock with a 32-column block) in its
// two passes over the trailing matrix C:
//   W partials  P_g = C^T V over split g's rows (W = C^H V), summed afterwards
//   update      C -= V Y^T with Y = W T formed in between
// V unit-lower trapezoidal in stored form, K <= 32.  Both are bandwidth-bound
// rank-32 products (the update moves 8 bytes per 32 FMAs of every element of
// C, the W pass reads 4): the operands stream through shared memory in two
// cp.async stages while the previous tile is computed, register tiles of 16
// or 32 outputs per thread, packed FP32x2 FMAs, plain FP32 rounding.
// (Measured against tcgen05 forms with three-way BF16 operand splitting and
// TMEM accumulators at one block per SM, for the 15 updates of a 65536 x 512
// factor: update 0.72 against 1.01 ms, W 0.58-0.61 against 1.04 ms.)
#pragma once
#include "rnp_common.cuh"

namespace rnpgpu {

struct UpdArgs {
    const float *V;  // M x K (ldv), unit-lower in stored form
    size_t ldv;
    const float *W;  // N x K (ldw): the product W T of the blocked update
    size_t ldw;
    float *C;        // M x N (ldc)
    size_t ldc;
    int M, N, K;
};

constexpr int kUpdMaxN = 512;   // widest trailing matrix taken by these kernels
constexpr int kUfRows = 64;     // rows of C per update tile
constexpr int kUfCols = 128;    // columns of C per update tile
constexpr int kUfThreads = 256;

// C(M x N) -= V(M x K) W(N x K)^T.  Block (bx, by) takes the column tile by
// and row tiles bx, bx + gridDim.x, ...: W's tile rows are staged once; the
// next row tile's C and V rows are copied into shared memory asynchronously
// (cp.async, two stages) while the current tile is computed.  Thread (tx =
// tid % 16, ty = tid / 16) owns rows 4 tx .. 4 tx + 3 and columns 8 ty .. 8
// ty + 7 of the tile (as pairs of adjacent columns for the packed FMAs): it
// copies and reads back only its own C elements, so only V needs a block
// barrier.  Dynamic shared memory: kUfSmem.
constexpr size_t kUfSmem = (size_t)(32 * kUfCols + 2 * 32 * kUfRows + 2 * kUfCols * kUfRows) * sizeof(float);
template <bool VEC> __global__ void __launch_bounds__(kUfThreads, 2) k_update_f32(UpdArgs g) {
    static_assert(kUfRows == 4 * 16 && kUfCols == 8 * (kUfThreads / 16), "thread tile");
    extern __shared__ __align__(16) float s_uf[];
    float (*sW)[kUfCols] = reinterpret_cast<float (*)[kUfCols]>(s_uf);                             // [k][col], negated
    float (*sV)[32][kUfRows] = reinterpret_cast<float (*)[32][kUfRows]>(s_uf + 32 * kUfCols);      // [stage][k][row]
    float (*sC)[kUfCols][kUfRows] = reinterpret_cast<float (*)[kUfCols][kUfRows]>(s_uf + 32 * kUfCols + 2 * 32 * kUfRows);  // [stage][col][row]
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int n0 = blockIdx.y * kUfCols, K = g.K;
    const bool vecv = VEC && ((uintptr_t)g.V % 16 == 0) && (g.ldv % 4 == 0);
    for (int idx = tid; idx < 32 * kUfCols; idx += kUfThreads) {
        const int c = idx % kUfCols, k = idx / kUfCols, gn = n0 + c;
        sW[k][c] = (k < K && gn < g.N) ? -g.W[gn + (size_t)k * g.ldw] : 0.f;  // negated: C += V (-W)^T
    }
    const int ntiles = (g.M + kUfRows - 1) / kUfRows;
    const int gc = n0 + 8 * ty;
    // row tile t into stage st: V's rows (unit-lower in stored form) and this
    // thread's C elements
    auto issue = [&](int t, int st) {
        const int m0 = t * kUfRows;
        for (int idx = tid; idx < 32 * (kUfRows / 4); idx += kUfThreads) {
            const int k = idx / (kUfRows / 4), r4 = 4 * (idx % (kUfRows / 4)), gm = m0 + r4;
            float *dst = &sV[st][k][r4];
            if (vecv && k < K && gm > k && gm + 4 <= g.M) {
                cp_async_cg16(dst, g.V + gm + (size_t)k * g.ldv);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int r = gm + e;
                    dst[e] = (k < K && r < g.M) ? (r > k ? g.V[r + (size_t)k * g.ldv] : (r == k ? 1.f : 0.f)) : 0.f;
                }
            }
        }
        const int gr = m0 + 4 * tx;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (gc + j >= g.N) continue;
            const float *src = g.C + gr + (size_t)(gc + j) * g.ldc;
            float *dst = &sC[st][8 * ty + j][4 * tx];
            if (VEC && gr + 4 <= g.M) {
                cp_async_cg16(dst, src);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) dst[e] = (gr + e < g.M) ? src[e] : 0.f;
            }
        }
        cp_async_commit();
    };
    int st = 0;
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, st ^= 1) {
        const int tn = t + gridDim.x;
        if (tn < ntiles) {
            issue(tn, st ^ 1);
            cp_async_wait_group<1>();
        } else {
            cp_async_wait_group<0>();
        }
        __syncthreads();  // V of tile t (and W) visible to the whole block
        const int gr = t * kUfRows + 4 * tx;
        float2 acc[4][4];  // acc[r][p] = (C(row r, col 2p), C(row r, col 2p + 1))
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float4 a = *reinterpret_cast<const float4 *>(&sC[st][8 * ty + 2 * p][4 * tx]);
            const float4 b = *reinterpret_cast<const float4 *>(&sC[st][8 * ty + 2 * p + 1][4 * tx]);
            acc[0][p] = make_float2(a.x, b.x);
            acc[1][p] = make_float2(a.y, b.y);
            acc[2][p] = make_float2(a.z, b.z);
            acc[3][p] = make_float2(a.w, b.w);
        }
#pragma unroll 8
        for (int k = 0; k < K; ++k) {
            const float4 v = *reinterpret_cast<const float4 *>(&sV[st][k][4 * tx]);
            const float4 wa = *reinterpret_cast<const float4 *>(&sW[k][8 * ty]);
            const float4 wb = *reinterpret_cast<const float4 *>(&sW[k][8 * ty + 4]);
            const float2 w[4] = {make_float2(wa.x, wa.y), make_float2(wa.z, wa.w), make_float2(wb.x, wb.y), make_float2(wb.z, wb.w)};
            const float vr[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int p = 0; p < 4; ++p) acc[r][p] = __ffma2_rn(make_float2(vr[r], vr[r]), w[p], acc[r][p]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (gc + j < g.N) {
                float *dst = g.C + gr + (size_t)(gc + j) * g.ldc;
                float x[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) x[r] = (j & 1) ? acc[r][j >> 1].y : acc[r][j >> 1].x;
                if (VEC && gr + 4 <= g.M) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(x[0], x[1], x[2], x[3]);
                } else {
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        if (gr + r < g.M) dst[r] = x[r];
                }
            }
        }
        __syncthreads();  // the stage is free for the tile after next
    }
}

// W partials for the first half of the same update: P[g][n + k N] = sum over
// split g's rows r of C(r, n) V(r, k) (V unit-lower in stored form), FP32
// sums; the partials are added afterwards in a fixed order.  Block (bx, by):
// split bx, columns 64 by .. 64 by + 63 of C.  The split's rows go through
// shared memory 64 at a time (cp.async, two stages, column-major with a
// padded stride); thread (tn = tid % 16, tk = (tid / 16) % 8, h = tid / 128)
// accumulates columns tn + 16 a against k = tk + 8 b (a, b < 4) over rows
// 32 h .. 32 h + 31 of every chunk, four rows per shared-memory load, even and
// odd rows in the two lanes of the packed FMAs; the lanes and the two halves
// are added at the end.
constexpr int kWfCols = 64, kWfRows = 64, kWfLd = kWfRows + 4;
constexpr size_t kWfSmem = (size_t)2 * (kWfCols + 32) * kWfLd * sizeof(float);
template <bool VEC> __global__ void __launch_bounds__(kUfThreads) k_w_f32(UpdArgs g, float *P, int rows_per_split) {
    extern __shared__ __align__(16) float s_wf[];
    float (*sC)[kWfCols][kWfLd] = reinterpret_cast<float (*)[kWfCols][kWfLd]>(s_wf);                      // [stage][col][row]
    float (*sV)[32][kWfLd] = reinterpret_cast<float (*)[32][kWfLd]>(s_wf + 2 * kWfCols * kWfLd);          // [stage][k][row]
    const int tid = threadIdx.x, tn = tid & 15, tk = (tid >> 4) & 7, h = tid >> 7;
    const int n0 = blockIdx.y * kWfCols, K = g.K;
    const int ra = blockIdx.x * rows_per_split, rb = min(g.M, ra + rows_per_split);
    const bool vecv = VEC && ((uintptr_t)g.V % 16 == 0) && (g.ldv % 4 == 0);
    auto issue = [&](int m0, int st) {
        for (int idx = tid; idx < kWfCols * (kWfRows / 4); idx += kUfThreads) {
            const int c = idx / (kWfRows / 4), r4 = 4 * (idx % (kWfRows / 4)), gm = m0 + r4, gn = n0 + c;
            float *dst = &sC[st][c][r4];
            const float *src = g.C + gm + (size_t)gn * g.ldc;
            if (VEC && gn < g.N && gm + 4 <= rb) {
                cp_async_cg16(dst, src);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) dst[e] = (gn < g.N && gm + e < rb) ? src[e] : 0.f;
            }
        }
        for (int idx = tid; idx < 32 * (kWfRows / 4); idx += kUfThreads) {
            const int k = idx / (kWfRows / 4), r4 = 4 * (idx % (kWfRows / 4)), gm = m0 + r4;
            float *dst = &sV[st][k][r4];
            if (vecv && k < K && gm > k && gm + 4 <= rb) {
                cp_async_cg16(dst, g.V + gm + (size_t)k * g.ldv);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int r = gm + e;
                    dst[e] = (k < K && r < rb) ? (r > k ? g.V[r + (size_t)k * g.ldv] : (r == k ? 1.f : 0.f)) : 0.f;
                }
            }
        }
        cp_async_commit();
    };
    // acc[a][b] = column tn + 16 a against k = tk + 8 b, as (even rows, odd
    // rows) partial sums: both FMA operands are adjacent rows of a 4-row load
    float2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
    int st = 0;
    if (ra < rb) issue(ra, 0);
    for (int m0 = ra; m0 < rb; m0 += kWfRows, st ^= 1) {
        if (m0 + kWfRows < rb) {
            issue(m0 + kWfRows, st ^ 1);
            cp_async_wait_group<1>();
        } else {
            cp_async_wait_group<0>();
        }
        __syncthreads();
#pragma unroll 2
        for (int r = 32 * h; r < 32 * h + 32; r += 4) {
            float4 c4[4], v4[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) c4[a] = *reinterpret_cast<const float4 *>(&sC[st][tn + 16 * a][r]);
#pragma unroll
            for (int b = 0; b < 4; ++b) v4[b] = *reinterpret_cast<const float4 *>(&sV[st][tk + 8 * b][r]);
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    acc[a][b] = __ffma2_rn(make_float2(c4[a].x, c4[a].y), make_float2(v4[b].x, v4[b].y), acc[a][b]);
                    acc[a][b] = __ffma2_rn(make_float2(c4[a].z, c4[a].w), make_float2(v4[b].z, v4[b].w), acc[a][b]);
                }
        }
        __syncthreads();  // the stage is free for the chunk after next
    }
    // add the two row halves (h = 1 into h = 0) and write the partial
    float *red = s_wf;  // 128 threads x 16 values, stride 17 (no bank conflicts)
    if (h == 1) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) red[(tid - 128) * 17 + 4 * a + b] = acc[a][b].x + acc[a][b].y;
    }
    __syncthreads();
    if (h == 0) {
        float *Pg = P + (size_t)blockIdx.x * g.N * K;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int n = n0 + tn + 16 * a;
            float sum[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) sum[b] = (acc[a][b].x + acc[a][b].y) + red[tid * 17 + 4 * a + b];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int k = tk + 8 * b;
                if (n < g.N && k < K) Pg[n + (size_t)k * g.N] = sum[b];
            }
        }
    }
}

} // namespace rnpgpu
