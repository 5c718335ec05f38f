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


} // namespace tc
} // namespace rnpgpu
