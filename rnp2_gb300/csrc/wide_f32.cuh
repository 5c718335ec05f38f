// wide_f32.cuh — the trailing update of the mixed solver's FP32 factor with
// 128-column reflector blocks on the 5th-generation tensor cores.
//
// The mixed least-squares solver factors an FP32 copy of A only to
// precondition the FP64 refinement, so its internal blocking is free: four
// 32-column panels (CholeskyQR2 with Householder reconstruction, updated
// among themselves by the rank-32 kernels of update_f32.cuh) form a
// 128-column block V, whose compact-WY factor T (128 x 128) is assembled from
// the four 32 x 32 panel factors and the Gram matrix V^T V
// (RNP/LA/Reflector.hpp:580-626 builds T column by column; the blocked form
// [[T_a, -T_a V_a^T V_b T_b], [0, T_b]] gives the same matrix).  The
// remaining columns C then take one ApplyBlock (RNP/LA/Reflector.hpp:725-815,
// side L, trans T) per 128 columns instead of four:
//     W = C^T V  (with V^T V in the same pass),  Y = W T,  C -= V Y^T.
//
// Both products run on tcgen05 with every FP32 operand split into three BF16
// slices x = x0 + 2^-8 x1 + 2^-16 x2 (each remainder scaled up by 2^8 before
// rounding; Henry, Tang & Heinecke 2019) and six BF16 products per K step
// accumulated in three FP32 TMEM accumulators by magnitude class (x0 y0 |
// x0 y1 + x1 y0 | x0 y2 + x1 y1 + x2 y0), summed small classes first in the
// epilogue: FP32-level products at tensor-core rates.
//
//   k_wide_vsplit   V (unit lower in stored form) -> two BF16-slice images in
//                   the UMMA canonical K-major layout: VA (K = V's columns,
//                   the A operand of the update) and VB (K = rows, the B
//                   operand of W and both operands of V^T V).  Rows past the
//                   block are zero.
//   k_wide_w        per (row split, 128-column tile): partial C^T V (tile 0:
//                   V^T V) in TMEM.  A warp issues the copies: C's FP32 tile
//                   by TMA (cp.async.bulk.tensor, 32 rows x 128 columns), the
//                   VB chunk by a bulk copy; four converter warps split C into
//                   slices in shared memory; one thread issues the MMAs;
//                   three stages on mbarriers.
//   k_wide_reduce   sum of the per-split partials (fixed order).
//   k_wide_t        T (128 x 128) from the panel factors and V^T V, one CTA.
//   k_wide_y        Y = W T, split into the BF16 slice image of the update's
//                   B operand (64-column tiles).
//   k_wide_update   C -= V Y^T per (128-row, 64-column) tile: Y's tile stays in
//                   shared memory, V's halves (64 K each) stream in by bulk
//                   copies, C's tile comes in and goes back by TMA; MMAs into
//                   one of two TMEM accumulator sets while the epilogue warps
//                   drain the other (C -= big + 2^-8 mid + 2^-16 small).
//
// Every wait is bounded: on timeout a CTA records kStatusBarrierTimeout in
// the library's device status word, stops issuing work, waits (bounded) for
// its own copies and MMAs in flight, frees its tensor memory and returns.
#pragma once
#include "tc_gemm.cuh"
#include "rnp_common.cuh"
#include <cuda.h>

namespace rnpgpu {
namespace wide {

constexpr int kNb = 128;           // columns of a wide reflector block
constexpr int kSlice = 3;          // BF16 slices per FP32 value
// VA image: per 128-row tile, two K halves of 64; per half three slices of
// 128 rows x 64 K (16 KB), core matrix (row/8, k/8) at ((row/8)*8 + k/8)*128
constexpr int kVaSlice = 128 * 64 * 2;
constexpr int kVaHalf = kSlice * kVaSlice;       // 48 KB
constexpr int kVaTile = 2 * kVaHalf;             // 96 KB
// VB image: per 32-row chunk three slices of 128 V-columns x 32 rows (8 KB),
// core matrix (vcol/8, row/8) at ((vcol/8)*4 + row/8)*128
constexpr int kVbSlice = 128 * 32 * 2;
constexpr int kVbChunk = kSlice * kVbSlice;      // 24 KB
// Y image: per 64-column tile of C, two K halves, three slices of 64 columns
// x 64 K (8 KB), core matrix (col/8, k/8) at ((col/8)*8 + k/8)*128
constexpr int kYSlice = 64 * 64 * 2;
constexpr int kYHalf = kSlice * kYSlice;         // 24 KB
constexpr int kYTile = 2 * kYHalf;               // 48 KB
constexpr int kUpdCols = 64;                     // columns of C per update tile

__host__ __device__ constexpr size_t va_bytes(int rows) { return (size_t)((rows + 127) / 128) * kVaTile; }
__host__ __device__ constexpr size_t vb_bytes(int rows) { return (size_t)((rows + 127) / 128) * 4 * kVbChunk; }
__host__ __device__ constexpr size_t y_bytes(int cols) { return (size_t)((cols + kUpdCols - 1) / kUpdCols) * kYTile; }

__device__ __forceinline__ uint32_t core_off(int mn, int k, int kcores) {
    return (uint32_t)(((mn >> 3) * kcores + (k >> 3)) * 128 + (mn & 7) * 16 + (k & 7) * 2);
}

// eight values of one 16-byte core-matrix row, split, one 16-byte store per slice
__device__ __forceinline__ void put8(unsigned char *slice0, int slice_bytes, uint32_t off, const float (&x)[8]) {
    tc::put8_slices(slice0, (size_t)slice_bytes, off, x);
}

// ---------------------------------------------------------------------------
// mbarrier / bulk-copy / TMA helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void arrive(uint64_t *bar) { asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory"); }
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(bytes),
                 "r"(tc::smem_u32(bar))
                 : "memory");
}
// 2-D tile of a column-major FP32 matrix: x = first row (a multiple of 4),
// y = first column; rows / columns outside the matrix read as zero
__device__ __forceinline__ void tma_load(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(tc::smem_u32(dst)), "l"(map), "r"(x),
                 "r"(y), "r"(tc::smem_u32(bar))
                 : "memory");
}
// the same tile back; elements outside the matrix are not written
__device__ __forceinline__ void tma_store(const CUtensorMap *map, int x, int y, const void *src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map), "r"(x), "r"(y), "r"(tc::smem_u32(src)) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void named_sync(int id, int threads) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory"); }

// ---------------------------------------------------------------------------
// k_wide_vsplit: V (rows x 128, unit lower in stored form, at A) -> VA, VB.
// One 256-thread block per 128-row tile; the tile goes through shared memory.
// ---------------------------------------------------------------------------
template <int kTag = 0> __global__ void __launch_bounds__(256) k_wide_vsplit(const float *A, size_t lda, int rows, unsigned char *va, unsigned char *vb) {
    extern __shared__ __align__(16) float s_v[];  // [128 cols][129]
    constexpr int LD = 129;
    const int t = blockIdx.x, tid = threadIdx.x;
    const int r0 = t * 128;
    // 64 loads per thread, 16 in flight at a time
    for (int i0 = 0; i0 < 64; i0 += 16) {
        float v[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int idx = tid + 256 * (i0 + i);
            const int r = idx & 127, k = idx >> 7, gr = r0 + r;
            v[i] = (gr < rows && gr > k) ? __ldg(A + gr + (size_t)k * lda) : (gr == k ? 1.f : 0.f);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int idx = tid + 256 * (i0 + i);
            s_v[(idx >> 7) * LD + (idx & 127)] = v[i];
        }
    }
    __syncthreads();
    // VA: unit (row, 8 consecutive K) -> one 16-byte chunk per slice
    unsigned char *vat = va + (size_t)t * kVaTile;
    for (int u = tid; u < 128 * 16; u += 256) {
        const int r = u & 127, kg = u >> 7, k0 = kg * 8, h = k0 >> 6;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = s_v[(k0 + e) * LD + r];
        put8(vat + h * kVaHalf, kVaSlice, core_off(r, k0 & 63, 8), x);
    }
    // VB: unit (V column, 8 consecutive rows) -> one chunk per slice
    for (int u = tid; u < 128 * 16; u += 256) {
        const int k = u & 127, rg = u >> 7, rr = rg * 8, c = rr >> 5;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = s_v[k * LD + rr + e];
        put8(vb + ((size_t)t * 4 + c) * kVbChunk, kVbSlice, core_off(k, rr & 31, 4), x);
    }
}

// ---------------------------------------------------------------------------
// k_wide_w: partials of W = C^T V and of V^T V.
// grid (nsplit, ntile): tile 0 is V^T V (A operand = VB), tile j >= 1 takes
// C's columns c1 + 128 (j-1) ... .  P[(split * ntile + tile) * 128 * 128 +
// v * 128 + c] = sum over the split's rows of V(row, v) X(row, c).
//
// The large-magnitude class (x0 y0) is accumulated by the tensor cores over
// kWFlush chunks (128 rows) at a time only, in one of two TMEM buffers; four
// drain warps add each finished buffer into FP32 registers (round to nearest)
// while the MMAs fill the other.  The tensor cores' own accumulation then
// spans 8 MMAs per value instead of the whole split, which keeps the partial
// at FP32 accuracy for any split length.  The two small classes stay in TMEM
// for the whole split.
// ---------------------------------------------------------------------------
struct WArgs {
    int rows;          // rows of the block (V and C)
    int r0, c1;        // first row of the block, first column of C (matrix coordinates)
    int ntile, nsplit, rows_per_split;  // rows_per_split: a multiple of 32
    const unsigned char *vb;
    float *P;
    int *status;
};
constexpr int kWStages = 3;
constexpr int kWStageBytes = 2 * kVbChunk + 32 * 128 * 4;  // VB chunk, A slices, C FP32 tile
constexpr int kWSmem = kWStages * kWStageBytes + 256;
constexpr int kWFlush = 4;      // chunks (of 32 rows) per class-0 accumulation
constexpr int kWThreads = 320;  // warp 0 copies, 1-4 convert, 5 issues MMAs, 6-9 drain
// TMEM columns: class 0 buffers at 0 and 384, class 1 at 128, class 2 at 256
__host__ __device__ constexpr uint32_t w_col(int cls, int buf) { return cls == 0 ? (buf ? 384u : 0u) : (uint32_t)(cls * 128); }

template <int kTag = 0> __global__ void __launch_bounds__(kWThreads, 1) k_wide_w(const __grid_constant__ CUtensorMap cmap, WArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kWStages * kWStageBytes);
    uint64_t *ready = full + kWStages;
    uint64_t *freed = ready + kWStages;
    uint64_t *c0full = freed + kWStages;  // [2] class-0 buffer holds a finished group
    uint64_t *c0free = c0full + 2;        // [2] class-0 buffer drained
    uint64_t *done = c0free + 2;          // every MMA has completed
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    int *abort_flag = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int split = blockIdx.x, tile = blockIdx.y;
    const int rbeg = split * a.rows_per_split;
    const int rend = min(a.rows, rbeg + a.rows_per_split);
    const int nch = rend > rbeg ? (rend - rbeg + 31) / 32 : 0;
    const int ngrp = (nch + kWFlush - 1) / kWFlush;
    const bool gram = (tile == 0);

    if (tid == 0) {
        for (int s = 0; s < kWStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&ready[s], 4);
            tc::mbar_init(&freed[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&c0full[b], 1);
            tc::mbar_init(&c0free[b], 4);
        }
        tc::mbar_init(done, 1);
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 5) {
        tc::tmem_alloc(tslot, 512);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;
    auto fail = [&]() {
        *(volatile int *)abort_flag = 1;
        if (a.status) atomicExch(a.status, (int)kStatusBarrierTimeout);
    };
    auto aborted = [&]() { return *(volatile int *)abort_flag != 0; };

    if (warp == 0) {
        // copies: VB chunk (+ C tile) per stage
        if (lane == 0) {
            uint32_t fph[kWStages] = {0, 0, 0};
            int arms[kWStages] = {0, 0, 0};
            for (int ch = 0; ch < nch && !aborted(); ++ch) {
                const int s = ch % kWStages;
                if (ch >= kWStages) {
                    if (!tc::mbar_wait(&freed[s], fph[s])) { fail(); break; }
                    fph[s] ^= 1u;
                }
                unsigned char *st = smem + s * kWStageBytes;
                const int row = rbeg + ch * 32;
                expect_tx(&full[s], (uint32_t)(kVbChunk + (gram ? 0 : 32 * 128 * 4)));
                ++arms[s];
                bulk_load(st, a.vb + (size_t)(row / 32) * kVbChunk, kVbChunk, &full[s]);
                if (!gram) tma_load(st + 2 * kVbChunk, &cmap, a.r0 + row, a.c1 + (tile - 1) * 128, &full[s]);
            }
            if (aborted()) {
                // copies in flight land before the CTA leaves (bounded wait
                // for the last phase each stage was armed for)
                for (int s = 0; s < kWStages; ++s)
                    if (arms[s] > 0) tc::mbar_wait(&full[s], (uint32_t)((arms[s] - 1) & 1));
            }
        }
    } else if (warp == 5) {
        // MMAs: per stage two K steps of 16 rows, six products each
        constexpr uint32_t idesc = tc::idesc_bf16(128, 128);
        const int pa[6] = {0, 0, 1, 0, 1, 2};
        const int pb[6] = {0, 1, 0, 2, 1, 0};
        const int pc[6] = {0, 1, 1, 2, 2, 2};
        uint32_t rph[kWStages] = {0, 0, 0};
        uint32_t fph[2] = {0, 0};
        for (int ch = 0; ch < nch; ++ch) {
            const int s = ch % kWStages;
            const int grp = ch / kWFlush, buf = grp & 1;
            const bool grp_first = (ch % kWFlush) == 0;
            const bool grp_last = ((ch + 1) % kWFlush) == 0 || ch + 1 == nch;
            if (grp_first && grp >= 2) {
                // the class-0 buffer of group grp - 2 has been drained
                const bool got = tc::mbar_wait(&c0free[buf], fph[buf]);
                if (!__all_sync(0xFFFFFFFFu, got) || aborted()) { fail(); break; }
                fph[buf] ^= 1u;
                tc::tc_fence_after();
            }
            const bool got = tc::mbar_wait(&ready[s], rph[s]);
            if (!__all_sync(0xFFFFFFFFu, got) || aborted()) { fail(); break; }
            rph[s] ^= 1u;
            tc::tc_fence_after();
            const uint32_t base = tc::smem_u32(smem + s * kWStageBytes);
            const uint32_t bop = base, aop = gram ? base : base + kVbChunk;
            __syncwarp();
            if (tc::elect_one()) {
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const uint64_t ad = tc::smem_desc(aop + pa[q] * kVbSlice + kk * 256, 128, 4 * 128);
                        const uint64_t bd = tc::smem_desc(bop + pb[q] * kVbSlice + kk * 256, 128, 4 * 128);
                        const bool fresh = pc[q] == 0 ? (grp_first && kk == 0) : (ch == 0 && kk == 0 && (q == 1 || q == 3));
                        tc::umma_bf16(tmem + w_col(pc[q], buf), ad, bd, idesc, fresh ? 0u : 1u);
                    }
                }
                tc::umma_commit(&freed[s]);
                if (grp_last) tc::umma_commit(&c0full[buf]);
            }
            __syncwarp();
        }
        // one commit after the last MMA: the final drain waits for it, and an
        // aborted CTA waits for it before freeing tensor memory
        __syncwarp();
        if (tc::elect_one()) tc::umma_commit(done);
        __syncwarp();
    } else if (warp >= 1 && warp <= 4) {
        // converters: C's FP32 tile [col][32 rows] -> A slices.  The tile
        // arrives 128-byte swizzled: the 16-byte chunk q of column c (rows
        // 4q .. 4q+3) sits at chunk q ^ (c & 7) of its 128-byte row.  Eight
        // consecutive threads take eight consecutive columns and the same
        // row group, so both their loads (distinct swizzled chunks) and their
        // slice stores (eight rows of one core matrix) hit distinct banks.
        const int ct = tid - 32;  // 0..127
        uint32_t fph[kWStages] = {0, 0, 0};
        for (int ch = 0; ch < nch; ++ch) {
            const int s = ch % kWStages;
            if (!tc::mbar_wait(&full[s], fph[s]) || aborted()) { fail(); break; }
            fph[s] ^= 1u;
            unsigned char *st = smem + s * kWStageBytes;
            if (!gram) {
                const float *cf = reinterpret_cast<const float *>(st + 2 * kVbChunk);
                unsigned char *as = st + kVbChunk;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int u = ct + 128 * i;
                    const int c = (u & 7) + 8 * (u >> 5), g = (u >> 3) & 3;
                    const int sw = c & 7;
                    const float4 lo = *reinterpret_cast<const float4 *>(cf + c * 32 + (((2 * g) ^ sw) << 2));
                    const float4 hi = *reinterpret_cast<const float4 *>(cf + c * 32 + (((2 * g + 1) ^ sw) << 2));
                    const float x[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
                    put8(as, kVbSlice, core_off(c, g * 8, 4), x);
                }
                tc::fence_proxy_async();
            }
            __syncwarp();
            if (lane == 0) arrive(&ready[s]);
        }
    } else {
        // drain warps 6-9: thread = TMEM lane (tile column c); class-0 groups
        // summed in registers, then the small classes, then the partial
        const int q = warp & 3;
        const int c = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        float acc[128];
#pragma unroll
        for (int i = 0; i < 128; ++i) acc[i] = 0.f;
        bool ok = nch > 0;
        uint32_t gph[2] = {0, 0};
        for (int grp = 0; ok && grp < ngrp; ++grp) {
            const int buf = grp & 1;
            if (!tc::mbar_wait(&c0full[buf], gph[buf]) || aborted()) { fail(); ok = false; break; }
            gph[buf] ^= 1u;
            tc::tc_fence_after();
#pragma unroll
            for (int v0 = 0; v0 < 128; v0 += 16) {
                float t[16];
                tc::tmem_ld16(lane_base + w_col(0, buf) + (uint32_t)v0, t);
#pragma unroll
                for (int i = 0; i < 16; ++i) acc[v0 + i] += t[i];
            }
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) arrive(&c0free[buf]);
        }
        if (ok && !tc::mbar_wait(done, 0)) { fail(); ok = false; }
        tc::tc_fence_after();
        float *P = a.P + ((size_t)split * a.ntile + tile) * 128 * 128;
#pragma unroll
        for (int v0 = 0; v0 < 128; v0 += 16) {
            float mid[16], small[16];
            if (ok) {
                tc::tmem_ld16(lane_base + w_col(1, 0) + (uint32_t)v0, mid);
                tc::tmem_ld16(lane_base + w_col(2, 0) + (uint32_t)v0, small);
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float out = ok ? acc[v0 + i] + fmaf(small[i], 0x1p-16f, mid[i] * 0x1p-8f) : 0.f;
                P[(size_t)(v0 + i) * 128 + c] = out;
            }
        }
    }
    if (aborted() && warp == 5) tc::mbar_wait(done, 0);  // MMAs in flight finish before TMEM is freed
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 5) tc::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// k_wide_reduce: GW[tile][v][c] = sum_s P[s][tile][v][c], fixed order.
// ---------------------------------------------------------------------------
template <int kTag = 0> __global__ void __launch_bounds__(128) k_wide_reduce(const float *P, int nsplit, int ntile, float *GW) {
    const int row = blockIdx.x;  // tile * 128 + v
    const int c = threadIdx.x;
    const size_t stride = (size_t)ntile * 128 * 128;
    const float *p = P + (size_t)row * 128 + c;
    // eight partial sums in flight, combined in a fixed order
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int s = 0;
    for (; s + 8 <= nsplit; s += 8) {
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] += __ldg(p + (size_t)(s + i) * stride);
    }
    for (int i = 0; s + i < nsplit; ++i) acc[i] += __ldg(p + (size_t)(s + i) * stride);
    GW[(size_t)row * 128 + c] = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
}

// ---------------------------------------------------------------------------
// k_wide_t: T (128 x 128, row-major, upper) from the four 32 x 32 panel
// factors Tp (column-major, 32 x 32 each, kTstride apart) and G = V^T V
// (GW tile 0, G[v][c]).  T(0:32b, blk b) = -T(0:32b, 0:32b) G(0:32b, blk b) T_b.
// ---------------------------------------------------------------------------
constexpr int kTLd = 132, kTGld = 36;  // row strides (16-byte rows for float4 loads)
constexpr int kTSmem = (128 * kTLd + 96 * kTGld + 96 * 33) * 4;
constexpr int kTThreads = 1024;
template <int kTag = 0> __global__ void __launch_bounds__(kTThreads) k_wide_t(const float *GW, const float *Tp, size_t tstride, int nblk, float *Tout) {
    extern __shared__ __align__(16) float s_t[];
    float (*sT)[kTLd] = reinterpret_cast<float (*)[kTLd]>(s_t);
    float (*sG)[kTGld] = reinterpret_cast<float (*)[kTGld]>(s_t + 128 * kTLd);
    float (*sX)[33] = reinterpret_cast<float (*)[33]>(s_t + 128 * kTLd + 96 * kTGld);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int idx = tid; idx < 128 * kTLd; idx += kTThreads) (&sT[0][0])[idx] = 0.f;
    __syncthreads();
    // the panel factors: 4 x 1024 values, upper triangles only (the panels
    // leave whatever the workspace held below their diagonals)
    {
        float v[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int idx = tid + kTThreads * i, b = idx >> 10, e = idx & 1023;
            v[i] = (b < nblk && (e & 31) <= (e >> 5)) ? __ldg(Tp + (size_t)b * tstride + e) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int idx = tid + kTThreads * i, b = idx >> 10, e = idx & 1023;
            if (b < nblk) sT[32 * b + (e & 31)][32 * b + (e >> 5)] = v[i];
        }
    }
    // warp w forms rows w, w + 32, w + 64 of each product, lane = column:
    // the row operand comes as float4 broadcasts, the column operand one
    // value per lane (four FMAs per five shared loads instead of one per two)
    for (int b = 1; b < nblk; ++b) {
        const int nr = 32 * b;
        // G(0:nr, blk b)
        {
            float v[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int idx = tid + kTThreads * i;
                v[i] = idx < nr * 32 ? __ldg(GW + (size_t)(idx >> 5) * 128 + 32 * b + (idx & 31)) : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int idx = tid + kTThreads * i;
                if (idx < nr * 32) sG[idx >> 5][idx & 31] = v[i];
            }
        }
        __syncthreads();
        // X = G(0:nr, blk b) T_b  (T_b upper: zeros below its diagonal in sT)
        {
            float x[3] = {0.f, 0.f, 0.f};
            for (int l = 0; l < 32; l += 4) {
                const float t0 = sT[32 * b + l][32 * b + lane], t1 = sT[32 * b + l + 1][32 * b + lane];
                const float t2 = sT[32 * b + l + 2][32 * b + lane], t3 = sT[32 * b + l + 3][32 * b + lane];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int r = warp + 32 * i;
                    if (r < nr) {
                        const float4 gv = *reinterpret_cast<const float4 *>(&sG[r][l]);
                        x[i] = fmaf(gv.w, t3, fmaf(gv.z, t2, fmaf(gv.y, t1, fmaf(gv.x, t0, x[i]))));
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if (warp + 32 * i < nr) sX[warp + 32 * i][lane] = x[i];
        }
        __syncthreads();
        // T(0:nr, blk b) = -T(0:nr, 0:nr) X  (T upper: zeros left of its diagonal)
        {
            float acc[3] = {0.f, 0.f, 0.f};
            for (int l = (warp & ~3); l < nr; l += 4) {
                const float x0 = sX[l][lane], x1 = sX[l + 1][lane], x2 = sX[l + 2][lane], x3 = sX[l + 3][lane];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int r = warp + 32 * i;
                    if (r < nr && l + 3 >= r) {
                        const float4 tv = *reinterpret_cast<const float4 *>(&sT[r][l]);
                        acc[i] = fmaf(tv.w, x3, fmaf(tv.z, x2, fmaf(tv.y, x1, fmaf(tv.x, x0, acc[i]))));
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if (warp + 32 * i < nr) sT[warp + 32 * i][32 * b + lane] = -acc[i];
        }
        __syncthreads();
    }
    __syncthreads();
    for (int idx = tid; idx < 128 * 128; idx += kTThreads) Tout[idx] = sT[idx >> 7][idx & 127];
}

// ---------------------------------------------------------------------------
// k_wide_y: Y = W T (W[c][v] = GW[1 + c/128][v][c%128], c < nc), split into
// the update's B-operand image; 16 columns of C per block.
// ---------------------------------------------------------------------------
constexpr int kYSmem = (128 * 128 + 16 * 129) * 4;
template <int kTag = 0> __global__ void __launch_bounds__(256) k_wide_y(const float *GW, const float *Tm, int nc, unsigned char *yimg) {
    extern __shared__ __align__(16) float s_y[];
    float (*sT)[128] = reinterpret_cast<float (*)[128]>(s_y);
    float (*sW)[129] = reinterpret_cast<float (*)[129]>(s_y + 128 * 128);
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * 16;
    {
        // T: 4096 float4, 16 per thread in flight
        float4 v[16];
        const float4 *t4 = reinterpret_cast<const float4 *>(Tm);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = __ldg(t4 + tid + 256 * i);
#pragma unroll
        for (int i = 0; i < 16; ++i) reinterpret_cast<float4 *>(&sT[0][0])[tid + 256 * i] = v[i];
        float w[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = tid + 256 * i, cc = idx & 15, vv = idx >> 4, c = c0 + cc;
            w[i] = c < nc ? __ldg(GW + ((size_t)(1 + c / 128) * 128 + vv) * 128 + (c % 128)) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = tid + 256 * i;
            sW[idx & 15][idx >> 4] = w[i];
        }
    }
    __syncthreads();
    // thread: column cc = tid / 16, K values k = 8 (tid % 16) .. + 7
    const int cc = tid >> 4, k0 = (tid & 15) * 8;
    float y[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) y[e] = 0.f;
    for (int v = 0; v < k0 + 8; ++v) {
        const float w = sW[cc][v];
#pragma unroll
        for (int e = 0; e < 8; ++e) y[e] = fmaf(w, sT[v][k0 + e], y[e]);  // T upper: zero below the diagonal
    }
    const int c = c0 + cc, u = c / kUpdCols, n = c % kUpdCols, h = k0 >> 6;
    put8(yimg + (size_t)u * kYTile + h * kYHalf, kYSlice, core_off(n, k0 & 63, 8), y);
}

// ---------------------------------------------------------------------------
// k_wide_update: C -= V Y^T.
// CTA b takes column tile u = b % J and row tiles b / J, b / J + G / J, ...
// (G = gridDim.x, a multiple of J): the CTAs working on one row tile run at
// the same time, so V's tile is read from memory once and from L2 after.
// ---------------------------------------------------------------------------
struct UArgs {
    int rows, r0, c1, ntiles_r, J;
    const unsigned char *va;
    const unsigned char *yimg;
    int *status;
};
constexpr int kUThreads = 192;  // warp 0 copies, warp 1 MMAs, warps 2-5 epilogue
constexpr int kUCtile = 128 * kUpdCols * 4;  // 32 KB
constexpr int kUSmem = kYTile + 2 * kVaHalf + 2 * kUCtile + 256;
constexpr uint32_t kUAcc = 3 * kUpdCols;  // TMEM columns of one accumulator set

template <int kTag = 0> __global__ void __launch_bounds__(kUThreads, 1) k_wide_update(const __grid_constant__ CUtensorMap cmap, UArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sY = smem;
    unsigned char *sV = smem + kYTile;                    // [half] 48 KB each
    float *sC = reinterpret_cast<float *>(smem + kYTile + 2 * kVaHalf);  // [buf][64 cols][128 rows]
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kYTile + 2 * kVaHalf + 2 * kUCtile);
    uint64_t *ybar = bars;            // Y loaded
    uint64_t *vfull = bars + 1;       // [2] V half loaded
    uint64_t *vfree = bars + 3;       // [2] V half consumed by the MMAs
    uint64_t *cfull = bars + 5;       // [2] C tile loaded
    uint64_t *cfree = bars + 7;       // [2] C tile stored (smem readable again)
    uint64_t *tfull = bars + 9;       // [2] accumulator set ready
    uint64_t *tfree = bars + 11;      // [2] accumulator set drained
    uint64_t *mdone = bars + 13;      // every MMA issued has completed
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 14);
    int *abort_flag = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int u = blockIdx.x % a.J;
    const int rstep = gridDim.x / a.J;
    const int rfirst = blockIdx.x / a.J;
    const int nitems = rfirst < a.ntiles_r ? (a.ntiles_r - rfirst + rstep - 1) / rstep : 0;

    if (tid == 0) {
        tc::mbar_init(ybar, 1);
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&vfull[i], 1);
            tc::mbar_init(&vfree[i], 1);
            tc::mbar_init(&cfull[i], 1);
            tc::mbar_init(&cfree[i], 1);
            tc::mbar_init(&tfull[i], 1);
            tc::mbar_init(&tfree[i], 4);
        }
        tc::mbar_init(mdone, 1);
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(tslot, 512);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;
    auto fail = [&]() {
        *(volatile int *)abort_flag = 1;
        if (a.status) atomicExch(a.status, (int)kStatusBarrierTimeout);
    };
    auto aborted = [&]() { return *(volatile int *)abort_flag != 0; };

    if (warp == 0) {
        if (lane == 0 && nitems > 0) {
            expect_tx(ybar, kYTile);
            bulk_load(sY, a.yimg + (size_t)u * kYTile, kYTile, ybar);
            uint32_t vph[2] = {0, 0}, cph[2] = {0, 0};
            int varms[2] = {0, 0}, carms[2] = {0, 0};
            for (int i = 0; i < nitems && !aborted(); ++i) {
                const int r = rfirst + i * rstep;
                bool ok = true;
                for (int h = 0; h < 2; ++h) {
                    if (i > 0) {
                        if (!tc::mbar_wait(&vfree[h], vph[h])) { ok = false; break; }
                        vph[h] ^= 1u;
                    }
                    expect_tx(&vfull[h], kVaHalf);
                    ++varms[h];
                    bulk_load(sV + h * kVaHalf, a.va + (size_t)r * kVaTile + h * kVaHalf, kVaHalf, &vfull[h]);
                }
                if (!ok) { fail(); break; }
                const int b = i & 1;
                if (i >= 2) {
                    if (!tc::mbar_wait(&cfree[b], cph[b])) { fail(); break; }
                    cph[b] ^= 1u;
                }
                expect_tx(&cfull[b], kUCtile);
                ++carms[b];
                tma_load(sC + b * (128 * kUpdCols), &cmap, a.r0 + r * 128, a.c1 + u * kUpdCols, &cfull[b]);
            }
            if (aborted()) {
                // copies in flight land before the CTA leaves (bounded)
                tc::mbar_wait(ybar, 0);
                for (int h = 0; h < 2; ++h)
                    if (varms[h] > 0) tc::mbar_wait(&vfull[h], (uint32_t)((varms[h] - 1) & 1));
                for (int b = 0; b < 2; ++b)
                    if (carms[b] > 0) tc::mbar_wait(&cfull[b], (uint32_t)((carms[b] - 1) & 1));
            }
        }
    } else if (warp == 1) {
        constexpr uint32_t idesc = tc::idesc_bf16(128, kUpdCols);
        const int pa[6] = {0, 0, 1, 0, 1, 2};
        const int pb[6] = {0, 1, 0, 2, 1, 0};
        const int pc[6] = {0, 1, 1, 2, 2, 2};
        const bool first_in_class[6] = {true, true, false, true, false, false};
        bool ok = nitems == 0 || __all_sync(0xFFFFFFFFu, tc::mbar_wait(ybar, 0));
        if (!ok) fail();
        uint32_t vph[2] = {0, 0}, tph[2] = {0, 0};
        for (int i = 0; ok && i < nitems; ++i) {
            const int b = i & 1;
            if (i >= 2) {
                const bool got = tc::mbar_wait(&tfree[b], tph[b]);
                if (!__all_sync(0xFFFFFFFFu, got) || aborted()) { fail(); break; }
                tph[b] ^= 1u;
            }
            tc::tc_fence_after();
            for (int h = 0; h < 2; ++h) {
                const bool got = tc::mbar_wait(&vfull[h], vph[h]);
                if (!__all_sync(0xFFFFFFFFu, got) || aborted()) { fail(); ok = false; break; }
                vph[h] ^= 1u;
                tc::tc_fence_after();
                const uint32_t va0 = tc::smem_u32(sV + h * kVaHalf), y0 = tc::smem_u32(sY + h * kYHalf);
                __syncwarp();
                if (tc::elect_one()) {
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
                        for (int q = 0; q < 6; ++q) {
                            const uint64_t ad = tc::smem_desc(va0 + pa[q] * kVaSlice + kk * 256, 128, 8 * 128);
                            const uint64_t bd = tc::smem_desc(y0 + pb[q] * kYSlice + kk * 256, 128, 8 * 128);
                            const bool fresh = (h == 0 && kk == 0 && first_in_class[q]);
                            tc::umma_bf16(tmem + b * kUAcc + (uint32_t)(pc[q] * kUpdCols), ad, bd, idesc, fresh ? 0u : 1u);
                        }
                    }
                    tc::umma_commit(&vfree[h]);
                    if (h == 1) tc::umma_commit(&tfull[b]);
                }
                __syncwarp();
            }
        }
        __syncwarp();
        if (tc::elect_one()) tc::umma_commit(mdone);
        __syncwarp();
    } else {
        // epilogue warps 2-5: thread = row of the tile
        const int q = warp & 3, row = q * 32 + lane;
        const int et = tid - 64;  // 0..127
        uint32_t tph[2] = {0, 0}, cph[2] = {0, 0};
        for (int i = 0; i < nitems; ++i) {
            const int b = i & 1;
            const int r = rfirst + i * rstep;
            if (!tc::mbar_wait(&tfull[b], tph[b]) || !tc::mbar_wait(&cfull[b], cph[b]) || aborted()) { fail(); break; }
            tph[b] ^= 1u;
            cph[b] ^= 1u;
            tc::tc_fence_after();
            float *cb = sC + b * (128 * kUpdCols);
#pragma unroll
            for (int c0 = 0; c0 < kUpdCols; c0 += 16) {
                const uint32_t lb = tmem + ((uint32_t)(q * 32) << 16) + b * kUAcc + (uint32_t)c0;
                float big[16], mid[16], small[16];
                tc::tmem_ld16(lb, big);
                tc::tmem_ld16(lb + kUpdCols, mid);
                tc::tmem_ld16(lb + 2 * kUpdCols, small);
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    float *p = cb + (c0 + e) * 128 + row;
                    *p = *p - (big[e] + fmaf(small[e], 0x1p-16f, mid[e] * 0x1p-8f));
                }
            }
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) arrive(&tfree[b]);
            tc::fence_proxy_async();
            named_sync(1, 128);
            if (et == 0) {
                tma_store(&cmap, a.r0 + r * 128, a.c1 + u * kUpdCols, cb);
                bulk_commit();
                bulk_wait_read_all();
                arrive(&cfree[b]);
            }
        }
        if (et == 0) bulk_wait_all();
    }
    // teardown: MMAs and copies of an aborted CTA are waited for (bounded)
    if (aborted() && warp == 1) tc::mbar_wait(mdone, 0);
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, 512);
}

} // namespace wide
} // namespace rnpgpu

// ===========================================================================
// host side
// ===========================================================================
namespace rnpgpu {

// 2-D tensor map of a column-major FP32 matrix (rows x cols, leading
// dimension ld elements) with box_rows x box_cols tiles (api_context.cu)
int encode_map_f32(CUtensorMap *map, const float *base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols, bool swizzle128 = false);

namespace wide {

struct WideWs {
    unsigned char *va = nullptr, *vb = nullptr, *y = nullptr;
    float *P = nullptr, *GW = nullptr, *T = nullptr;
    size_t p_floats = 0;
};

inline size_t al256(size_t b) { return (b + 255) / 256 * 256; }
inline int max_tiles(size_t n) { return 1 + (int)((n + kNb - 1) / kNb); }
inline size_t p_floats_for(size_t n) { return (size_t)(std::max(device_facts().sm_count, 1) + max_tiles(n)) * 128 * 128; }
inline size_t ws_bytes(size_t m, size_t n) {
    return al256(va_bytes((int)m)) + al256(vb_bytes((int)m)) + al256(y_bytes((int)n)) + al256(p_floats_for(n) * 4) + al256((size_t)max_tiles(n) * 128 * 128 * 4) +
           al256(128 * 128 * 4) + 256;
}
template <class Carv> WideWs carve(Carv &cv, size_t m, size_t n) {
    WideWs w;
    w.va = cv.template take<unsigned char>(va_bytes((int)m));
    w.vb = cv.template take<unsigned char>(vb_bytes((int)m));
    w.y = cv.template take<unsigned char>(y_bytes((int)n));
    w.p_floats = p_floats_for(n);
    w.P = cv.template take<float>(w.p_floats);
    w.GW = cv.template take<float>((size_t)max_tiles(n) * 128 * 128);
    w.T = cv.template take<float>(128 * 128);
    return w;
}

// The wide update applies to a factorization of A (m x n, lda) whose TMA
// tiles start on 16-byte boundaries.
inline bool usable(size_t m, size_t n, const float *a, size_t lda) {
    return m >= n && n > (size_t)kNb && m >= 256 && lda % 4 == 0 && ((uintptr_t)a % 16) == 0 && m < (size_t)INT32_MAX / 2 && n < (size_t)INT32_MAX / 2;
}

// C = A(r0:m, c1:n) -= V Y^T for the 128-column block V = A(r0:m, r0:r0+128)
// (c1 = r0 + 128 unless given: any column right of the block, e.g. one
// 128-column range of a left-looking order) with the four 32 x 32 panel
// factors at Tp (tstride apart).  The block's 128 x 128 T (row-major) goes to
// Tsave when given (kept for later applications of Q), else to the workspace.
// vcache (optional): the block's own V slice images (va_bytes(rows) +
// vb_bytes(rows) bytes) instead of the workspace's; with reuse they already
// hold this block's slices and Tsave its T from an earlier call, so the
// slicing and the T build are skipped.
inline int apply(float *A, size_t lda, int m, int n, int r0, const float *Tp, size_t tstride, const WideWs &w, cudaStream_t st, float *Tsave = nullptr, int c1_at = -1,
                 unsigned char *vcache = nullptr, bool reuse = false) {
    const int rows = m - r0, c1 = c1_at >= 0 ? c1_at : r0 + kNb, nc = n - c1;
    if (c1 < r0 + kNb) return kErrDevice;
    if (reuse && (vcache == nullptr || Tsave == nullptr)) return kErrDevice;
    if (rows <= 0 || nc <= 0) return kOk;
    const int sms = std::max(1, device_facts().sm_count);
    int *status = device_status_ptr();
    int rc;
    unsigned char *va = vcache ? vcache : w.va;
    unsigned char *vb = vcache ? vcache + al256(va_bytes(rows)) : w.vb;
    if (!reuse) {
        KScope ks("wide_vsplit", st);
        const int smem = 128 * 129 * 4;
        if ((rc = kernel_attr((const void *)k_wide_vsplit<0>, smem))) return rc;
        k_wide_vsplit<0><<<(rows + 127) / 128, 256, smem, st>>>(A + r0 + (size_t)r0 * lda, lda, rows, va, vb);
        RNPGPU_CHECK_LAUNCH();
    }
    const int ntile = 1 + (nc + kNb - 1) / kNb;
    int nsplit = std::max(1, sms / ntile);
    int rps = ((rows + nsplit - 1) / nsplit + 31) / 32 * 32;
    nsplit = (rows + rps - 1) / rps;
    if ((size_t)nsplit * ntile * 128 * 128 > w.p_floats) return kErrDevice;
    {
        KScope ks("wide_w", st);
        CUtensorMap map;
        if ((rc = encode_map_f32(&map, A, (uint64_t)m, (uint64_t)n, lda, 32, 128, true))) return rc;
        if ((rc = kernel_attr((const void *)k_wide_w<0>, kWSmem))) return rc;
        WArgs wa;
        wa.rows = rows; wa.r0 = r0; wa.c1 = c1; wa.ntile = ntile; wa.nsplit = nsplit; wa.rows_per_split = rps;
        wa.vb = vb; wa.P = w.P; wa.status = status;
        k_wide_w<0><<<dim3(nsplit, ntile), kWThreads, kWSmem, st>>>(map, wa);
        RNPGPU_CHECK_LAUNCH();
    }
    {
        KScope ks("wide_t", st);
        k_wide_reduce<0><<<ntile * 128, 128, 0, st>>>(w.P, nsplit, ntile, w.GW);
        RNPGPU_CHECK_LAUNCH();
        float *Tb = Tsave ? Tsave : w.T;
        if (!reuse) {
            if ((rc = kernel_attr((const void *)k_wide_t<0>, kTSmem))) return rc;
            k_wide_t<0><<<1, kTThreads, kTSmem, st>>>(w.GW, Tp, tstride, 4, Tb);
            RNPGPU_CHECK_LAUNCH();
        }
        const int J = (nc + kUpdCols - 1) / kUpdCols;
        if ((rc = kernel_attr((const void *)k_wide_y<0>, kYSmem))) return rc;
        k_wide_y<0><<<J * kUpdCols / 16, 256, kYSmem, st>>>(w.GW, Tb, nc, w.y);
        RNPGPU_CHECK_LAUNCH();
    }
    {
        KScope ks("wide_update", st);
        CUtensorMap map;
        if ((rc = encode_map_f32(&map, A, (uint64_t)m, (uint64_t)n, lda, 128, kUpdCols))) return rc;
        if ((rc = kernel_attr((const void *)k_wide_update<0>, kUSmem))) return rc;
        const int J = (nc + kUpdCols - 1) / kUpdCols;
        const int ntr = (rows + 127) / 128;
        const int per = std::max(1, std::min(sms / J, ntr));
        UArgs ua;
        ua.rows = rows; ua.r0 = r0; ua.c1 = c1; ua.ntiles_r = ntr; ua.J = J;
        ua.va = va; ua.yimg = w.y; ua.status = status;
        k_wide_update<0><<<J * per, kUThreads, kUSmem, st>>>(map, ua);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

} // namespace wide
} // namespace rnpgpu
