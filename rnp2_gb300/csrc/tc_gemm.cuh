// tc_gemm.cuh — FP32 contractions on the 5th-generation tensor cores
// (tcgen05, sm_103a) by three-term BF16 splitting.
//
// Every FP32 operand element x is split as x = x0 + x1 + x2 with
// x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1) (Henry, Tang and
// Heinecke, "Leveraging the bfloat16 artificial intelligence datatype for
// higher-precision computations", 2019); x1 and x2 are stored scaled by 2^8
// and 2^16 so that they do not underflow for small x.  The product a*b is formed from the
// six terms of order <= 2^-16 relative, each a BF16 x BF16 MMA.  The three
// magnitude classes accumulate in separate FP32 accumulators in tensor
// memory (a0b0 | a0b1 + a1b0 | a0b2 + a1b1 + a2b0), so the low-order bits
// the tensor-core accumulation drops stay proportional to each class's own
// size; the epilogue adds them with round-to-nearest FP32 arithmetic, small
// classes first.  The K range one accumulator sees is capped by the caller
// (split-K), which keeps the accumulated rounding at FP32 level.
//
// One CTA computes a 128 x BN tile of D = alpha*op(A)*op(B) (+D | +I) over a
// K chunk.  All 256 threads stage FP32 tiles from global memory (any op, the
// Householder-V unit-lower convention of k_gemm), split them and store the
// bf16 slices into shared memory in the canonical K-major, no-swizzle layout
// (8 x 16-byte core matrices).  One thread issues the tcgen05.mma
// instructions for a stage and commits them to the stage's mbarrier; the
// stage is refilled only after that mbarrier completes (two stages, so the
// global loads of the next K step overlap the MMAs of the current one).  The
// accumulator (128 lanes x BN FP32 columns) lives in TMEM and is read back
// with tcgen05.ld for the epilogue.  Every wait is bounded: on timeout the
// CTA records an error and skips its epilogue.
#pragma once
#include "qr_kernels.cuh"
#include <cuda_bf16.h>

namespace rnpgpu {
namespace tc {

constexpr int kBM = 128;      // rows of a tile (UMMA M)
constexpr int kBK = 32;       // K per stage (two UMMA K=16 steps)
constexpr int kThreads = 256;
constexpr long long kWaitLimit = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kWaitLimit) return false;
    }
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// true in exactly one lane of the (converged) warp
__device__ __forceinline__ bool elect_one() {
    uint32_t pred = 0;
    asm volatile("{\n.reg .b32 rx;\n.reg .pred px;\nelect.sync rx|px, 0xFFFFFFFF;\n@px mov.u32 %0, 1;\n}\n" : "+r"(pred));
    return pred != 0;
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// 32 lanes x 16 consecutive 32-bit TMEM columns into 16 registers per thread
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, K-major without swizzle: start address,
// leading byte offset (between core matrices along K), stride byte offset
// (between 8-row groups), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// Instruction descriptor: BF16 x BF16 -> FP32, both operands K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row, k) in a K-major no-swizzle bf16 tile with kBK
// columns: core matrix (row/8, k/8) is 128 contiguous bytes
__device__ __forceinline__ uint32_t tile_off(int row, int k) {
    return (uint32_t)(((row >> 3) * (kBK / 8) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// x = h0 + 2^-8 h1 + 2^-16 h2: each remainder is scaled up by 2^8 (exactly)
// before it is rounded, so the low slices stay as far from the bottom of the
// exponent range as x itself; the accumulator of class c carries 2^(8c)
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h0, __nv_bfloat16 &h1, __nv_bfloat16 &h2) {
    h0 = __float2bfloat16_rn(x);
    float r = (x - __bfloat162float(h0)) * 256.0f;
    h1 = __float2bfloat16_rn(r);
    r = (r - __bfloat162float(h1)) * 256.0f;
    h2 = __float2bfloat16_rn(r);
}

// eight consecutive-K values of one row, split, as one 16-byte store per
// slice at byte offset o of slice 0 (slices slice_bytes apart)
__device__ __forceinline__ void put8_slices(unsigned char *slice0, size_t slice_bytes, uint32_t o, const float (&x)[8]) {
    __align__(16) __nv_bfloat16 h[3][8];
#pragma unroll
    for (int e = 0; e < 8; ++e) split3(x[e], h[0][e], h[1][e], h[2][e]);
#pragma unroll
    for (int q = 0; q < 3; ++q) *reinterpret_cast<uint4 *>(slice0 + q * slice_bytes + o) = *reinterpret_cast<const uint4 *>(h[q]);
}

template <int BN> struct SmemLayout {
    static constexpr int kSliceA = kBM * kBK * 2;          // bytes of one bf16 slice of the A tile
    static constexpr int kSliceB = BN * kBK * 2;
    static constexpr int kStage = 3 * kSliceA + 3 * kSliceB;
    static constexpr int kBytes = 2 * kStage + 64;          // two stages + mbarriers/TMEM slot
};

template <int BN> __global__ void __launch_bounds__(kThreads) k_gemm_tc(GemmArgs<float> g, int *err) {
    typedef SmemLayout<BN> L;
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * L::kStage);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 2 * L::kStage + 32);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * g.kchunk;
    const int kend = min(g.K, kbeg + g.kchunk);
    // three accumulators of BN columns each, rounded up to a power of two
    constexpr uint32_t kCols = (3 * BN <= 32) ? 32 : (3 * BN <= 64) ? 64 : (3 * BN <= 128) ? 128 : (3 * BN <= 256) ? 256 : 512;

    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_d = *tmem_slot;

    // registers for one K step of both operands (FP32), fetched ahead
    constexpr int LA = kBM * kBK / kThreads, LB = (BN * kBK + kThreads - 1) / kThreads;
    float ra[LA], rb[LB];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int idx = tid + u * kThreads;
            int mi, ki;
            if (g.opA == kOpN) { mi = idx % kBM; ki = idx / kBM; }
            else { ki = idx % kBK; mi = idx / kBK; }
            const int gm = m0 + mi, gk = k0 + ki;
            ra[u] = (gm < g.M && gk < kend) ? load_op(g.A, g.lda, g.opA, g.vunitA, gm, gk) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int idx = tid + u * kThreads;
            int ni, ki;
            if (g.opB == kOpN) { ki = idx % kBK; ni = idx / kBK; }
            else { ni = idx % BN; ki = idx / BN; }
            const int gn = n0 + ni, gk = k0 + ki;
            rb[u] = (idx < BN * kBK && gn < g.N && gk < kend) ? load_op(g.B, g.ldb, g.opB, g.vunitB, gk, gn) : 0.f;
        }
    };
    // split and store into stage s
    auto stash = [&](int s) {
        unsigned char *st = smem + s * L::kStage;
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int idx = tid + u * kThreads;
            int mi, ki;
            if (g.opA == kOpN) { mi = idx % kBM; ki = idx / kBM; }
            else { ki = idx % kBK; mi = idx / kBK; }
            __nv_bfloat16 h0, h1, h2;
            split3(ra[u], h0, h1, h2);
            const uint32_t o = tile_off(mi, ki);
            *reinterpret_cast<__nv_bfloat16 *>(st + o) = h0;
            *reinterpret_cast<__nv_bfloat16 *>(st + L::kSliceA + o) = h1;
            *reinterpret_cast<__nv_bfloat16 *>(st + 2 * L::kSliceA + o) = h2;
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int idx = tid + u * kThreads;
            if (idx < BN * kBK) {
                int ni, ki;
                if (g.opB == kOpN) { ki = idx % kBK; ni = idx / kBK; }
                else { ni = idx % BN; ki = idx / BN; }
                __nv_bfloat16 h0, h1, h2;
                split3(rb[u], h0, h1, h2);
                const uint32_t o = tile_off(ni, ki);
                unsigned char *sb = st + 3 * L::kSliceA;
                *reinterpret_cast<__nv_bfloat16 *>(sb + o) = h0;
                *reinterpret_cast<__nv_bfloat16 *>(sb + L::kSliceB + o) = h1;
                *reinterpret_cast<__nv_bfloat16 *>(sb + 2 * L::kSliceB + o) = h2;
            }
        }
    };

    constexpr uint32_t idesc = idesc_bf16(kBM, BN);
    const int nsteps = (kend - kbeg + kBK - 1) / kBK;
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    if (nsteps > 0) fetch(kbeg);
    for (int t = 0; t < nsteps; ++t) {
        const int s = t & 1;
        if (t >= 2) {
            // stage s was last read by the MMAs of step t-2
            if (!mbar_wait(&bars[s], phase[s])) ok = false;
            phase[s] ^= 1u;
        }
        if (!__syncthreads_and(ok ? 1 : 0)) {
            ok = false;
            break;
        }
        stash(s);
        fence_proxy_async();
        __syncthreads();
        if (t + 1 < nsteps) fetch(kbeg + (t + 1) * kBK);
        if (warp == 0) {  // warp-uniform descriptors, one elected issuing lane
            tc_fence_after();
            const uint32_t base = smem_u32(smem + s * L::kStage);
            const uint32_t a0 = base, b0 = base + 3 * L::kSliceA;
            // (a-slice, b-slice, accumulator): class 0 = a0b0, class 1 =
            // a0b1 + a1b0, class 2 = a0b2 + a1b1 + a2b0
            const int pa[6] = {0, 0, 1, 0, 1, 2};
            const int pb[6] = {0, 1, 0, 2, 1, 0};
            const int pc[6] = {0, 1, 1, 2, 2, 2};
            const bool first_in_class[6] = {true, true, false, true, false, false};
            if (elect_one()) {
#pragma unroll
                for (int kk = 0; kk < kBK / 16; ++kk) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const uint64_t ad = smem_desc(a0 + pa[q] * L::kSliceA + kk * 256, 128, (kBK / 8) * 128);
                        const uint64_t bd = smem_desc(b0 + pb[q] * L::kSliceB + kk * 256, 128, (kBK / 8) * 128);
                        const bool fresh = (t == 0 && kk == 0 && first_in_class[q]);
                        umma_bf16(tmem_d + (uint32_t)(pc[q] * BN), ad, bd, idesc, fresh ? 0u : 1u);
                    }
                }
                umma_commit(&bars[s]);
            }
            __syncwarp();
        }
    }
    // wait for the last MMAs (both stages' outstanding commits)
    if (ok && nsteps > 0) {
        const int last = (nsteps - 1) & 1;
        if (!mbar_wait(&bars[last], phase[last])) ok = false;
        if (nsteps >= 2) {
            const int other = last ^ 1;
            if (!mbar_wait(&bars[other], phase[other])) ok = false;
        }
    }
    tc_fence_after();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok && tid == 0) atomicExch(err, (int)kStatusBarrierTimeout);

    // epilogue: warp w reads TMEM lanes 32*(w%4).. (tile rows), column half w/4
    if (ok) {
        float *D = g.D + (size_t)blockIdx.z * g.dstride;
        const int q = warp & 3, half = warp >> 2;
        const int row = m0 + q * 32 + lane;
        constexpr int kHalf = BN / 2;
        for (int c0 = half * kHalf; c0 < (half + 1) * kHalf; c0 += 16) {
            float v[16];
            if (nsteps > 0) {
                const uint32_t lane_base = tmem_d + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
                float big[16], mid[16], small[16];
                tmem_ld16(lane_base, big);
                tmem_ld16(lane_base + BN, mid);
                tmem_ld16(lane_base + 2 * BN, small);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = big[i] + fmaf(small[i], 0x1p-16f, mid[i] * 0x1p-8f);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (row < g.M) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int col = n0 + c0 + i;
                    if (col < g.N) {
                        float x = g.alpha * v[i];
                        float *dp = &D[row + (size_t)col * g.ldd];
                        if (g.beta_mode == kBetaOne) x = x + *dp;
                        else if (g.beta_mode == kBetaIdentity && row == col) x = x + 1.0f;
                        *dp = x;
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem_d, kCols);
}


// ---------------------------------------------------------------------------
// Persistent rank-K update (K <= 32), the FP32 trailing update of the
// blocked factorization:  C(M x N) -= V(M x K) W(N x K)^T, V unit-lower
// trapezoidal in stored form (vunit), N <= kUpdMaxN.
// W's three BF16 slices are split once per CTA and stay in shared memory;
// the CTA then walks 128-row tiles (t = blockIdx.x, += gridDim.x): it splits
// the tile's V into its slices, and streams the tile's C in 64-column chunks
// through two TMEM accumulator sets (the MMAs of chunk c+1 run while the
// epilogue of chunk c reads C, subtracts and writes it back).
// ---------------------------------------------------------------------------
constexpr int kUpdChunk = 64;
constexpr int kUpdMaxN = 512;

struct UpdArgs {
    const float *V;  // M x K (ldv), unit-lower in stored form
    size_t ldv;
    const float *W;  // N x K (ldw)
    size_t ldw;
    float *C;        // M x N (ldc)
    size_t ldc;
    int M, N, K;
};

__host__ __device__ constexpr int upd_npad(int N) { return (N + kUpdChunk - 1) / kUpdChunk * kUpdChunk; }
__host__ __device__ constexpr size_t upd_smem_bytes(int N) {
    return (size_t)3 * kBM * kBK * 2 + (size_t)3 * upd_npad(N) * kBK * 2 + 64;
}

template <int CH> __global__ void __launch_bounds__(kThreads) k_update_tc(UpdArgs g, int *err) {
    static_assert(CH == kUpdChunk, "chunk width");
    extern __shared__ __align__(1024) unsigned char smem[];
    const int npad = upd_npad(g.N);
    constexpr int kSliceA = kBM * kBK * 2;
    const int sliceB = npad * kBK * 2;
    unsigned char *sA = smem;                    // 3 slices of the V tile
    unsigned char *sB = smem + 3 * kSliceA;      // 3 slices of W (all N rows)
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + 3 * sliceB);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr uint32_t kCols = 512;              // 2 sets x 3 classes x 64 columns
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kCols);
        tmem_relinquish();
    }
    // W -> B slices: element (n, k) of the N x K operand is W(n, k); a thread
    // takes 8 consecutive k of one row (consecutive threads, consecutive
    // rows: the 16-byte stores of a warp fall into distinct banks)
    for (int idx = tid; idx < npad * (kBK / 8); idx += kThreads) {
        const int n = idx % npad, k0 = (idx / npad) * 8;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = (n < g.N && k0 + e < g.K) ? g.W[n + (size_t)(k0 + e) * g.ldw] : 0.f;
        put8_slices(sB, sliceB, tile_off(n, k0), x);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    constexpr uint32_t idesc = idesc_bf16(kBM, kUpdChunk);
    const int nchunks = npad / kUpdChunk;
    const int ntiles = (g.M + kBM - 1) / kBM;
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    // MMAs of chunk c into accumulator set s: called by all of warp 0 (the
    // descriptors are warp-uniform values), issued by one elected lane
    auto issue = [&](int c, int s) {
        tc_fence_after();
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB) + (uint32_t)(c * kUpdChunk / 8) * (kBK / 8) * 128;
        const uint32_t d0 = tmem_base + (uint32_t)(s * 3 * kUpdChunk);
        const int pa[6] = {0, 0, 1, 0, 1, 2};
        const int pb[6] = {0, 1, 0, 2, 1, 0};
        const int pc[6] = {0, 1, 1, 2, 2, 2};
        const bool first_in_class[6] = {true, true, false, true, false, false};
        if (elect_one()) {
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const uint64_t ad = smem_desc(a0 + pa[q] * kSliceA + kk * 256, 128, (kBK / 8) * 128);
                    const uint64_t bd = smem_desc(b0 + pb[q] * sliceB + kk * 256, 128, (kBK / 8) * 128);
                    umma_bf16(d0 + (uint32_t)(pc[q] * kUpdChunk), ad, bd, idesc, (kk == 0 && first_in_class[q]) ? 0u : 1u);
                }
            }
            umma_commit(&bars[s]);
        }
        __syncwarp();
    };
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int m0 = t * kBM;
        // V tile -> A slices (rows m0.., unit-lower in stored form), 8
        // consecutive k of one row per thread as for W
        for (int idx = tid; idx < kBM * (kBK / 8); idx += kThreads) {
            const int mi = idx % kBM, k0 = (idx / kBM) * 8, gm = m0 + mi;
            float x[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = k0 + e;
                float v = 0.f;
                if (gm < g.M && k < g.K) v = (gm > k) ? g.V[gm + (size_t)k * g.ldv] : (gm == k ? 1.f : 0.f);
                x[e] = v;
            }
            put8_slices(sA, kSliceA, tile_off(mi, k0), x);
        }
        fence_proxy_async();
        __syncthreads();
        if (warp == 0) issue(0, 0);
        // epilogue mapping: warp w reads TMEM lanes 32*(w%4).. (tile rows) and
        // the column half w/4 of each chunk; its C values for the next chunk
        // are loaded while the current chunk is finished
        const int q = warp & 3, half = warp >> 2;
        const int row = m0 + q * 32 + lane;
        constexpr int kHalf = kUpdChunk / 2;
        auto load_c = [&](int c, float (&buf)[kHalf]) {
            const int col0 = c * kUpdChunk + half * kHalf;
            const float *cp = g.C + row + (size_t)col0 * g.ldc;
#pragma unroll
            for (int i = 0; i < kHalf; ++i) buf[i] = (row < g.M && col0 + i < g.N) ? cp[(size_t)i * g.ldc] : 0.f;
        };
        float cur[kHalf], nxt[kHalf];
        load_c(0, cur);
        for (int c = 0; c < nchunks; ++c) {
            const int s = c & 1;
            if (warp == 0 && c + 1 < nchunks) issue(c + 1, s ^ 1);
            if (c + 1 < nchunks) load_c(c + 1, nxt);
            if (!mbar_wait(&bars[s], phase[s])) ok = false;
            phase[s] ^= 1u;
            tc_fence_after();
            if (!__syncthreads_and(ok ? 1 : 0)) {
                ok = false;
                break;
            }
            const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(s * 3 * kUpdChunk);
            const int col0 = c * kUpdChunk + half * kHalf;
            float *cp = g.C + row + (size_t)col0 * g.ldc;
#pragma unroll
            for (int c0 = 0; c0 < kHalf; c0 += 16) {
                float big[16], mid[16], small[16];
                tmem_ld16(lane_base + (uint32_t)(half * kHalf + c0), big);
                tmem_ld16(lane_base + (uint32_t)(kUpdChunk + half * kHalf + c0), mid);
                tmem_ld16(lane_base + (uint32_t)(2 * kUpdChunk + half * kHalf + c0), small);
                if (row < g.M) {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (col0 + c0 + i < g.N) cp[(size_t)(c0 + i) * g.ldc] = cur[c0 + i] - (big[i] + fmaf(small[i], 0x1p-16f, mid[i] * 0x1p-8f));
                }
            }
#pragma unroll
            for (int i = 0; i < kHalf; ++i) cur[i] = nxt[i];
            tc_fence_before();
            __syncthreads();
        }
    }
    if (!ok && tid == 0) atomicExch(err, (int)kStatusBarrierTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem_base, kCols);
}


// ---------------------------------------------------------------------------
// Persistent reduction W_g = C^T V over row blocks (the first half of the
// trailing update, W = C^H V for FP32 data), N <= kUpdMaxN, K <= 32.
// The MMA's M dimension runs over C's columns (128 per chunk), N over V's
// columns, K over rows: both operands are K-major straight from column-major
// storage.  Block g takes 128-row blocks kb = g, g + gridDim.x, ...; for each
// it splits V's rows once, then streams the block's C in 128-column chunks
// through two shared-memory stages (the next chunk's loads are in flight
// while the current chunk's MMAs run) into per-chunk TMEM accumulators that
// persist across the block's row blocks.  The epilogue writes block g's
// partial W (N x K, leading dimension N) at P + g * N * K; the partials are
// summed afterwards in a fixed order.
// ---------------------------------------------------------------------------
constexpr int kWRows = 128;   // K per row block
constexpr int kWCols = 128;   // C columns per chunk (MMA M)
constexpr int kWThreads = 256;

template <int KB> __device__ __forceinline__ uint32_t tile_off_k(int row, int k) {
    return (uint32_t)(((row >> 3) * (KB / 8) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

struct WArgs {
    const float *C;  // M x N (ldc)
    size_t ldc;
    const float *V;  // M x K (ldv), unit-lower in stored form
    size_t ldv;
    float *P;        // [gridDim.x][N x K], leading dimension N
    int M, N, K;
};

constexpr int kWSliceA = kWCols * kWRows * 2;  // 32 KB: one BF16 slice of a C chunk
constexpr int kWSliceB = 32 * kWRows * 2;      // 8 KB: one BF16 slice of V's rows
constexpr size_t kWSmem = (size_t)2 * 3 * kWSliceA + 3 * kWSliceB + 64;

// VEC: C's base is 16-byte aligned and ldc a multiple of 4, so a thread's
// 8 rows come in two 16-byte loads (8 scalar loads of one column would each
// touch another cache line of the chunk, and the L1 left beside this shared
// memory cannot hold them between the loads)
template <int CH, bool VEC> __global__ void __launch_bounds__(kWThreads) k_w_tc(WArgs g, int *err) {
    static_assert(CH == kWCols, "chunk width");
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;                         // 2 stages x 3 slices
    unsigned char *sB = smem + 2 * 3 * kWSliceA;      // 3 slices of V's rows
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + 3 * kWSliceB);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr uint32_t kCols = 512;                   // up to 4 chunks x 3 classes x 32
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const int nkb = (g.M + kWRows - 1) / kWRows;
    const int nch = (g.N + kWCols - 1) / kWCols;
    const int my_kb = ((int)blockIdx.x < nkb) ? (nkb - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nsteps = my_kb * nch;
    constexpr uint32_t idesc = idesc_bf16(kWCols, 32);
    // a thread moves 8 consecutive rows of one column at a time: consecutive
    // threads take consecutive columns, so the 16-byte slice stores of a
    // warp fall into distinct banks (core-matrix rows are 16 bytes apart)
    constexpr int LU = kWCols * (kWRows / 8) / kWThreads;  // 8-row pieces per thread per step
    float cr[LU][8];
    auto fetch = [&](int t) {
        const int kb = blockIdx.x + (t / nch) * gridDim.x, cc = t % nch;
#pragma unroll
        for (int u = 0; u < LU; ++u) {
            const int idx = tid + u * kWThreads;
            const int c = idx % kWCols, r0 = (idx / kWCols) * 8;
            const int gr = kb * kWRows + r0, gc = cc * kWCols + c;
            const float *src = g.C + gr + (size_t)gc * g.ldc;
            if (VEC && gc < g.N && gr + 8 <= g.M) {
                const float4 lo = *reinterpret_cast<const float4 *>(src), hi = *reinterpret_cast<const float4 *>(src + 4);
                cr[u][0] = lo.x; cr[u][1] = lo.y; cr[u][2] = lo.z; cr[u][3] = lo.w;
                cr[u][4] = hi.x; cr[u][5] = hi.y; cr[u][6] = hi.z; cr[u][7] = hi.w;
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) cr[u][e] = (gc < g.N && gr + e < g.M) ? src[e] : 0.f;
            }
        }
    };
    auto put8 = [&](unsigned char *slice0, size_t slice_bytes, uint32_t o, const float (&x)[8]) {
        __align__(16) __nv_bfloat16 h[3][8];
#pragma unroll
        for (int e = 0; e < 8; ++e) split3(x[e], h[0][e], h[1][e], h[2][e]);
#pragma unroll
        for (int q = 0; q < 3; ++q) *reinterpret_cast<uint4 *>(slice0 + q * slice_bytes + o) = *reinterpret_cast<const uint4 *>(h[q]);
    };
    auto stash = [&](int st) {
        unsigned char *a = sA + st * 3 * kWSliceA;
#pragma unroll
        for (int u = 0; u < LU; ++u) {
            const int idx = tid + u * kWThreads;
            const int c = idx % kWCols, r0 = (idx / kWCols) * 8;
            put8(a, kWSliceA, tile_off_k<kWRows>(c, r0), cr[u]);
        }
    };
    auto split_v = [&](int kb) {
        for (int idx = tid; idx < 32 * (kWRows / 8); idx += kWThreads) {
            const int n = idx % 32, r0 = (idx / 32) * 8;
            float x[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int gr = kb * kWRows + r0 + e;
                float v = 0.f;
                if (gr < g.M && n < g.K) v = (gr > n) ? g.V[gr + (size_t)n * g.ldv] : (gr == n ? 1.f : 0.f);
                x[e] = v;
            }
            put8(sB, kWSliceB, tile_off_k<kWRows>(n, r0), x);
        }
    };
    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    bool ok = true;
    auto wait_stage = [&](int st) {
        if (pending[st]) {
            if (!mbar_wait(&bars[st], phase[st])) ok = false;
            phase[st] ^= 1u;
            pending[st] = false;
        }
    };
    if (nsteps > 0) fetch(0);
    for (int t = 0; t < nsteps; ++t) {
        const int st = t & 1, cc = t % nch, kbl = t / nch;
        if (cc == 0) {
            // V's rows of the next row block: every MMA still reading them is done
            wait_stage(0);
            wait_stage(1);
            split_v(blockIdx.x + kbl * gridDim.x);
        }
        wait_stage(st);
        if (!__syncthreads_and(ok ? 1 : 0)) {
            ok = false;
            break;
        }
        stash(st);
        fence_proxy_async();
        __syncthreads();
        if (t + 1 < nsteps) fetch(t + 1);
        if (warp == 0) {  // warp-uniform descriptors, one elected issuing lane
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + st * 3 * kWSliceA), b0 = smem_u32(sB);
            const uint32_t d0 = tmem_base + (uint32_t)(cc * 96);
            const int pa[6] = {0, 0, 1, 0, 1, 2};
            const int pb[6] = {0, 1, 0, 2, 1, 0};
            const int pc[6] = {0, 1, 1, 2, 2, 2};
            const bool first_in_class[6] = {true, true, false, true, false, false};
            if (elect_one()) {
#pragma unroll
                for (int kk = 0; kk < kWRows / 16; ++kk) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const uint64_t ad = smem_desc(a0 + pa[q] * kWSliceA + kk * 256, 128, (kWRows / 8) * 128);
                        const uint64_t bd = smem_desc(b0 + pb[q] * kWSliceB + kk * 256, 128, (kWRows / 8) * 128);
                        const bool fresh = (kbl == 0 && kk == 0 && first_in_class[q]);
                        umma_bf16(d0 + (uint32_t)(pc[q] * 32), ad, bd, idesc, fresh ? 0u : 1u);
                    }
                }
                umma_commit(&bars[st]);
            }
            __syncwarp();
        }
        pending[st] = true;
    }
    wait_stage(0);
    wait_stage(1);
    tc_fence_after();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok && tid == 0) atomicExch(err, (int)kStatusBarrierTimeout);
    // epilogue: warp w reads TMEM lanes 32*(w%4).. (C columns), V columns 16*(w/4)..
    if (ok) {
        float *P = g.P + (size_t)blockIdx.x * g.N * g.K;
        const int q = warp & 3, half = warp >> 2;
        for (int cc = 0; cc < nch; ++cc) {
            const int n = cc * kWCols + q * 32 + lane;
            float v[16];
            if (nsteps > 0) {
                const uint32_t base = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(cc * 96 + half * 16);
                float big[16], mid[16], small[16];
                tmem_ld16(base, big);
                tmem_ld16(base + 32, mid);
                tmem_ld16(base + 64, small);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = big[i] + fmaf(small[i], 0x1p-16f, mid[i] * 0x1p-8f);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (n < g.N) {
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (half * 16 + i < g.K) P[n + (size_t)(half * 16 + i) * g.N] = v[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem_base, kCols);
}

} // namespace tc
} // namespace rnpgpu
