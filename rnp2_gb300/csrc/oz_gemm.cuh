// oz_gemm.cuh — the FP64 products of the mixed least-squares refinement,
// r = b - A x and g = A^T r, on the FP16 tensor cores by exact integer
// slicing.
//
// On this GPU the FP64 pipe runs at about 1.2 TFLOP/s: as FP64 FMAs each of
// these products takes ~1 ms at 65536 x 512 x 16 right-hand sides, while
// reading A once takes ~40 us.  Here they are formed from exact fixed-point
// slices instead (the error-free splitting of Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59, 2012;
// on low-precision tensor cores as in Mukunoki, Ozaki, Ogita and Imamura,
// "DGEMM using Tensor Cores, and Its Accurate and Reproducible Versions",
// ISC 2020):
//
// * every column k of A has a power-of-two scale 2^e_k with |a_ik| < 2^(e_k-1)
//   (computed once per solve); every right-hand side j of the other operand a
//   scale 2^f_j chosen the same way for the scaled values;
// * a scaled value v in (-1/2, 1/2) is rounded to the integer N = round(v 2^56)
//   and written as eight balanced base-128 digits, v ~ sum_p d_p 2^(-7(p+1)),
//   d_p an integer in [-64, 64] (exact in FP16);
// * a digit product d_p D_q is an integer of magnitude <= 2^12; the products
//   of one level L = p + q go into one FP32 tensor-memory accumulator.  Over
//   512 K values a level L <= 4 stays below 5 * 2^12 * 2^9 < 2^24, so those
//   sums are exact integers; levels 5..7 weigh less than 2^-35 relative, where
//   FP32 rounding of their sums no longer matters; levels >= 8 are dropped;
// * every 512 K values the exact levels are combined exactly in 64-bit
//   integers, sum_{L<=4} S_L 2^(7(4-L)) (< 2^53), the others in FP32, and at
//   the end result = 2^scale * 2^-14 * sum_L 2^(-7L) S_L in FP64.
//
// The error is that of representing both operands to 2^-56 of their scales
// plus the dropped levels: about 2^-50 of sum_k 2^e_k |x_kj| 2^(f_j - e_k) —
// the accuracy of an FP64 dot product, independent of the condition of A.
//
// Tensor-core layout.  One accumulation D (128 TMEM lanes x 128 FP32 columns)
// per 128 rows of A (residual) or 128 columns of A (A^T r): lane = that row or
// column, column c = 16 b + j holds level 7 - b of right-hand side j.  The
// A tile's digits are eight planes in tensor memory (the UMMA A operand,
// M = 128: row i in lane i, K packed two FP16 per column), written by the
// converter warps with tcgen05.st so that shared memory only carries the
// packed bytes and the stacks; the
// other operand's digits are one stack of eight 16-row blocks, block b = digit
// 7 - b (the UMMA B operand).  Digit plane p multiplies the window of blocks
// p..7 (N = 16 (8 - p)) into columns 0 .. 16 (8 - p): column block b' then
// receives digit 7 - p - b' of the other operand, i.e. level 7 - b', so all
// eight MMAs of a K step add into the same accumulator and every level lands
// in its own column block.
//
// Operand preparation.  A does not change during a solve, so its digits are
// extracted once (k_adigits, fused with the FP32 copy the factorization
// needs) into a packed form of the same size as the FP64 matrix: eight bytes
// per element, byte p = (d_p + 64) xor 64 (zero bytes are zero digits),
// stored in 16 x 16 element blocks (2 KB: row-major, the 16-byte chunks of
// row r rotated by xor with r mod 8) so that one 16-K step of either product
// is eight whole blocks: contiguous for the residual (block column), eight
// 2 KB pieces for A^T r (block row).  A is padded with zero blocks to whole
// 128 x 128 tiles.  The other operand (x, or r for A^T r) is small;
// k_xstack / k_rstack compute its scales f_j and write its digits directly as
// the FP16 digit-stack image of every 16-K step (the UMMA B operand, read by
// the tensor core straight from the staging buffer).
//
// CTA of k_oz (warp-specialised, all hand-offs on mbarriers):
//   warp 16       one thread issues the bulk copies (cp.async.bulk) of each
//                 step's A blocks into a ring of kNA buffers (freed by the
//                 converters); warp 22 the same for the stack images (ring of
//                 kNT, freed by the MMAs), so that neither waits on the other
//                 and the A copies run up to kNA steps ahead;
//   warps 0..15   two groups of eight warps, for even and odd steps (so that
//                 one group's waits overlap the other's work), expand the
//                 packed bytes of a step into the eight FP16 digit planes of
//                 one of kNS tensor-memory stages (tcgen05.st);
//   warp 17       issues the eight tcgen05.mma of a step from one elected
//                 lane and commits them to the stage's and the stack buffer's
//                 mbarriers (and to the accumulator's at a chunk end);
//   warps 18..21  drain a finished accumulator (tcgen05.ld), combine the
//                 levels exactly in integer arithmetic (running sums in shared
//                 memory), write the outputs.
// Two accumulator sets let the drain of one chunk overlap the MMAs of the
// next.  Every wait is bounded.
#pragma once
#include "ls_kernels.cuh"
#include "qr_driver.cuh"
#include <cuda_fp16.h>

namespace rnpgpu {
namespace oz {

constexpr int kDig = 8;                          // digits per operand
constexpr int kKst = 16;                         // K values per step (one UMMA K)
constexpr int kChunkSteps = 32;                  // steps per exact accumulation chunk (512 K)
constexpr int kRhs = 16;                         // right-hand sides per launch
constexpr int kConvWarps = 16;                   // converter warps 0..15
constexpr int kLoadWarp = 16, kMmaWarp = 17;      // then the drain warps 18..21
constexpr int kStackWarp = 22;
constexpr int kThreads = 23 * 32;
constexpr int kNA = 8;                           // staging ring of A blocks (bulk copies up to kNA steps ahead)
constexpr int kNT = 8;                           // staging ring of stack images
constexpr int kNS = 4;                           // digit-plane stages in TMEM
constexpr int kBlock = 16 * 16 * 8;              // one 16 x 16 block of packed A (2 KB)
constexpr int kRawA = 8 * kBlock;                // a step's A blocks (16 KB)
constexpr int kStack = kDig * kRhs * kKst * 2;   // a step's stack image of the other operand (4 KB)
constexpr int kPlaneCols = kKst / 2;            // one digit plane of the A tile in TMEM: 128 lanes x 8 columns
constexpr int kStageCols = kDig * kPlaneCols;    // 64 columns per stage
constexpr int kAccCols = 128;                    // one accumulator set
constexpr int kTmemCols = 512;                   // 2 accumulator sets + kNS stages
static_assert(2 * kAccCols + kNS * kStageCols <= kTmemCols, "tensor memory");
constexpr int kSmemA = 0;
constexpr int kSmemT = kSmemA + kNA * kRawA;
constexpr int kSmemAcc = kSmemT + kNT * kStack;  // the drain's running sums: 128 rows x 16 x (8 + 4) bytes
constexpr int kSmemCtl = kSmemAcc + 128 * kRhs * 12;
constexpr int kCtlBytes = (2 * kNA + 2 * kNT + 2 * kNS + 4) * 8 + 8 + 3 * kRhs * 4;  // mbarriers, TMEM slot, flags
constexpr int kSmem = kSmemCtl + (kCtlBytes + 255) / 256 * 256;
// one CTA per SM: each allocates all of tensor memory
static_assert(kSmem > 114 * 1024, "the shared-memory request must keep a second CTA off the SM");
constexpr int kZeroExp = -(1 << 20);             // scale of an all-zero column / vector
constexpr int kNonFinite = 1 << 20;              // an Inf or NaN was seen
constexpr unsigned long long kBias = 0x81020408102040ull;  // 64 * sum_q 128^q, q = 0..7

enum Mode : int { kResidual = 0, kNormal = 1 };

struct Args {
    int mode;
    int m, n, nrhs;             // nrhs <= 16
    const unsigned char *Ad;    // packed digits of A in 16 x 16 blocks, nbr block rows per block column
    int nbr;
    const uint4 *XS;            // stack images of the other operand, one per 16-K step (256 x 16 bytes)
    const int *fexp;            // f_j of the other operand (16)
    const double *B;            // residual: b (m x nrhs)
    size_t ldb;
    double *out;                // residual: r (m x nrhs); A^T r: partial q of g at out + q * pstride
    size_t ldo, pstride;
    const int *colexp;          // e_k for the n columns of A
    int *rexp_out;              // residual: per CTA, per right-hand side, max exponent of r
    int range_rows, nranges;    // A^T r: rows of A per partial, number of partials
    int *err;
};

// floor(log2 |v|) for finite nonzero v (subnormals report -1023, an upper
// bound), kZeroExp for zero, kNonFinite for Inf/NaN
__device__ __forceinline__ int oz_exp(double v) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int eb = (int)((bits >> 52) & 0x7FF);
    if (eb == 0x7FF) return kNonFinite;
    if ((bits << 1) == 0) return kZeroExp;
    return (eb == 0 ? 1 : eb) - 1023;
}


// The eight balanced base-128 digit fields of v 2^se (which must lie in
// (-1/2, 1/2)), top digit first: u_p = d_p + 64 in [0, 128].
__device__ __forceinline__ void oz_fields(double v, int se, uint32_t (&u)[kDig]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    int eb = (int)((bits >> 52) & 0x7FF);
    unsigned long long M = bits & 0xFFFFFFFFFFFFFull;
    if (eb != 0) {
        M |= 1ull << 52;
    } else if (M != 0) {  // subnormal: normalise the significand
        const int lz = __clzll((long long)M) - 11;
        M <<= lz;
        eb = 1 - lz;
    }
    // v = M 2^(eb - 1075) and N = round(M 2^(eb - 1075 + se + 56)) = round((M << 3) 2^-t)
    const int t = min(max(1022 - eb - se, 1), 63);
    const unsigned long long Nm = ((M << 3) + (1ull << (t - 1))) >> t;
    const unsigned long long U = ((bits >> 63) ? (0ull - Nm) : Nm) + kBias;
    // U = sum_q (d_q + 64) 128^q with d_q in [-64, 63] for q < 7; the top digit is unmasked
    const uint32_t lo = (uint32_t)U, hi = (uint32_t)(U >> 32);
    u[0] = hi >> 17;
    u[1] = (hi >> 10) & 127u;
    u[2] = (hi >> 3) & 127u;
    u[3] = __funnelshift_r(lo, hi, 28) & 127u;
    u[4] = (lo >> 21) & 127u;
    u[5] = (lo >> 14) & 127u;
    u[6] = (lo >> 7) & 127u;
    u[7] = lo & 127u;
}

// a digit field as an exact FP32 integer d = u - 64 (2^23 + u is exact in
// FP32; subtracting 2^23 + 64 leaves u - 64)
__device__ __forceinline__ float oz_digit_value(uint32_t u) { return __uint_as_float(0x4B000000u | u) - 8388672.0f; }

// FP16 bits of a digit (an integer of magnitude <= 64: exact)
__device__ __forceinline__ uint16_t oz_digit_f16(uint32_t u) { return __half_as_ushort(__float2half_rn(oz_digit_value(u))); }

// packed form of one element: byte p = u_p xor 64 (zero bytes = zero digits)
__device__ __forceinline__ uint2 oz_pack(const uint32_t (&u)[kDig]) {
    uint2 w;
    w.x = (u[0] | (u[1] << 8) | (u[2] << 16) | (u[3] << 24)) ^ 0x40404040u;
    w.y = (u[4] | (u[5] << 8) | (u[6] << 16) | (u[7] << 24)) ^ 0x40404040u;
    return w;
}

// byte offset of (row, k) in a K-major, no-swizzle 16-bit tile with kKst = 16
// columns: core matrix (row/8, k/8) is 128 contiguous bytes
__device__ __forceinline__ uint32_t toff(int row, int k) { return (uint32_t)(((row >> 3) * 2 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes) : "memory");
}
// bulk global -> shared copy completing on an mbarrier (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) { asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory"); }
// 32 lanes x 4 consecutive 32-bit TMEM columns from registers
__device__ __forceinline__ void tmem_st4(uint32_t taddr, uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "r"(r0), "r"(r1), "r"(r2), "r"(r3) : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// instruction descriptor: FP16 x FP16 -> FP32, both operands K-major, M x N
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) { return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24); }
// D (TMEM) += A (TMEM) * B (shared memory descriptor), kind::f16 -> FP32
__device__ __forceinline__ void umma_f16_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc),
                 "r"(accumulate)
                 : "memory");
}
// 32 lanes x 8 consecutive 32-bit TMEM columns
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// Operand preparation
// ---------------------------------------------------------------------------
// e_k = max_i floor(log2 |a_ik|) + 2 (kZeroExp for a zero column, kNonFinite
// when the column holds an Inf or NaN), from the exponent bits alone (no
// floating-point work: the FP64 pipe of this GPU is slow); one block per column
template <int kTag> __global__ void __launch_bounds__(256) k_col_exp(int m, int n, const double *A, size_t lda, int *colexp) {
    __shared__ int sx[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        int ex = kZeroExp;
        const double *col = A + (size_t)c * lda;
        int r = tid;
        for (; r + 3 * 256 < m; r += 4 * 256) {
            const int e0 = oz_exp(col[r]), e1 = oz_exp(col[r + 256]), e2 = oz_exp(col[r + 512]), e3 = oz_exp(col[r + 768]);
            ex = max(ex, max(max(e0, e1), max(e2, e3)));
        }
        for (; r < m; r += 256) ex = max(ex, oz_exp(col[r]));
        ex = __reduce_max_sync(0xFFFFFFFFu, ex);
        if (lane == 0) sx[warp] = ex;
        __syncthreads();
        if (tid == 0) {
            int e = kZeroExp;
            for (int w = 0; w < 8; ++w) e = max(e, sx[w]);
            colexp[c] = (e >= kNonFinite) ? kNonFinite : (e == kZeroExp ? kZeroExp : e + 2);
        }
        __syncthreads();
    }
}

// out[j] = ||Af(0:m, j)||_2^2 of the FP32 working copy, accumulated in FP32
// with eight partial sums per thread and combined in FP64 (relative error
// below 1e-6: the norm only scales the stopping test); one block per column
template <int kTag> __global__ void __launch_bounds__(256) k_col_sumsq_f32(int m, int n, const float *Af, size_t ldf, double *out) {
    __shared__ double s[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        const float *col = Af + (size_t)c * ldf;
        float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int r = tid;
        for (; r + 7 * 256 < m; r += 8 * 256) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const float v = col[r + u * 256];
                acc[u] = fmaf(v, v, acc[u]);
            }
        }
        for (; r < m; r += 256) acc[0] = fmaf(col[r], col[r], acc[0]);
        double t = 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) t += (double)acc[u];
        t = warp_sum(t);
        if (lane == 0) s[warp] = t;
        __syncthreads();
        if (tid == 0) {
            double v = 0.0;
            for (int w = 0; w < 8; ++w) v += s[w];
            out[c] = v;
        }
        __syncthreads();
    }
}

// byte offset of element (r, c) inside a 16 x 16 block of packed A: row-major
// 128-byte rows whose 16-byte chunks (two elements) are rotated by r mod 8, so
// that eight threads reading one chunk each of eight rows hit distinct banks
__device__ __forceinline__ uint32_t blk_off(int r, int c) { return (uint32_t)(r * 128 + (((c >> 1) ^ (r & 7)) << 4) + ((c & 1) << 3)); }

// Packed digits of A relative to 2^e_k in 16 x 16 blocks: block (bi, bk) at
// byte (bk * nbr + bi) * 2048 of Ad, zero outside m x n (the grid covers
// whole 128-row tiles and 16-column blocks: nbr = 8 * ceil(m / 128), and the
// caller sizes the column blocks to 8 * ceil(n / 128)).  Af(0:m, 0:n) =
// (float) A when Af != nullptr (the working copy of the FP32 factorization).
// Thread (ml, g) of a block handles row ml of a 128-row tile and columns
// 8g..8g+7 of a 16-column block: coalesced reads along each column, one
// 16-byte chunk write per column pair.
template <int kTag> __global__ void __launch_bounds__(256) k_adigits(int m, int n, int nbr, int nbc, const double *A, size_t lda, const int *colexp, unsigned char *Ad, float *Af, size_t ldf) {
    const int ml = threadIdx.x & 127, g = threadIdx.x >> 7;
    const int ntile = nbr / 8;
    for (int bk = blockIdx.y; bk < nbc; bk += gridDim.y) {
        for (int rt = blockIdx.x; rt < ntile; rt += gridDim.x) {
            const int i = rt * 128 + ml;
            uint2 w[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = bk * 16 + 8 * g + e;
                w[e] = make_uint2(0u, 0u);
                if (i < m && k < n) {
                    const double v = A[i + (size_t)k * lda];
                    if (Af) Af[i + (size_t)k * ldf] = (float)v;
                    const int ek = colexp[k];
                    if (ek > kZeroExp && ek < kNonFinite) {
                        uint32_t u[kDig];
                        oz_fields(v, -ek, u);
                        w[e] = oz_pack(u);
                    }
                }
            }
            unsigned char *blk = Ad + ((size_t)bk * nbr + (size_t)(rt * 8 + (ml >> 4))) * kBlock;
            const int r = ml & 15;
#pragma unroll
            for (int e = 0; e < 8; e += 2) *reinterpret_cast<uint4 *>(blk + blk_off(r, 8 * g + e)) = make_uint4(w[e].x, w[e].y, w[e + 1].x, w[e + 1].y);
        }
    }
}

// Eight consecutive K values (kk = 8h .. 8h + 7) of right-hand side j of the
// other operand, scaled by 2^se[e], into the stack image img: digit q goes to
// block 7 - q, row 16 (7 - q) + j, as one 16-byte chunk per digit.
__device__ __forceinline__ void oz_stack_put8(unsigned char *img, int h, int j, const double (&v)[8], const int (&se)[8]) {
    uint32_t w[kDig][4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
        uint32_t ua[kDig], ub[kDig];
        oz_fields(v[e], se[e], ua);
        oz_fields(v[e + 1], se[e + 1], ub);
#pragma unroll
        for (int q = 0; q < kDig; ++q) w[q][e >> 1] = (uint32_t)oz_digit_f16(ua[q]) | ((uint32_t)oz_digit_f16(ub[q]) << 16);
    }
#pragma unroll
    for (int q = 0; q < kDig; ++q) *reinterpret_cast<uint4 *>(img + toff(16 * (7 - q) + j, 8 * h)) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
}

// x (n x nrhs, nrhs <= 16) for the residual: f_j = max_k (floor(log2 |x_kj|) + e_k) + 2,
// then the stack image of every 16-row step of x scaled by 2^(e_k - f_j).
// Every block computes f_j (x is small), then writes the images of its steps;
// block 0 stores f_j.  Thread (j, h) of a 32-thread group handles K half h.
template <int kTag> __global__ void __launch_bounds__(256) k_xstack(int n, int nrhs, const double *X, size_t ldx, const int *colexp, int *fexp, uint4 *XS) {
    __shared__ int sf[kRhs];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < kRhs) sf[tid] = kZeroExp;
    __syncthreads();
    int mx[kRhs];
#pragma unroll
    for (int j = 0; j < kRhs; ++j) mx[j] = kZeroExp;
    for (int k = tid; k < n; k += blockDim.x) {
        const int ek = colexp[k];
        double v[kRhs];
#pragma unroll
        for (int j = 0; j < kRhs; ++j) v[j] = (j < nrhs) ? X[k + ldx * (size_t)j] : 0.0;
#pragma unroll
        for (int j = 0; j < kRhs; ++j) {
            const int ex = oz_exp(v[j]);
            if (ex >= kNonFinite) mx[j] = kNonFinite;
            else if (ex > kZeroExp && ek > kZeroExp && ek < kNonFinite) mx[j] = max(mx[j], ex + ek + 2);
        }
    }
#pragma unroll
    for (int j = 0; j < kRhs; ++j) {
        const int r = __reduce_max_sync(0xFFFFFFFFu, mx[j]);
        if (lane == 0 && r > kZeroExp) atomicMax(&sf[j], r);
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid < kRhs) fexp[tid] = sf[tid];
    const int nsteps = (n + kKst - 1) / kKst;
    for (int idx = blockIdx.x * blockDim.x + tid; idx < nsteps * 32; idx += gridDim.x * blockDim.x) {
        const int s = idx >> 5, j = (idx >> 1) & 15, h = idx & 1;
        double v[8];
        int se[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = s * kKst + 8 * h + e;
            v[e] = 0.0;
            se[e] = 0;
            if (k < n && j < nrhs && sf[j] < kNonFinite) {
                const int ek = colexp[k];
                if (ek > kZeroExp && ek < kNonFinite) {
                    v[e] = X[k + ldx * (size_t)j];
                    se[e] = ek - sf[j];
                }
            }
        }
        oz_stack_put8(reinterpret_cast<unsigned char *>(XS + (size_t)s * 256), h, j, v, se);
    }
}

// r (m x nrhs, nrhs <= 16) for A^T r: f_j = max over the residual's CTAs of
// max_i floor(log2 |r_ij|), plus 2; then the stack image of every 16-row step
// of r scaled by 2^-f_j.  Block 0 stores f_j.
template <int kTag> __global__ void __launch_bounds__(256) k_rstack(int m, int nrhs, const double *R, size_t ldr, const int *rexp, int rexp_n, int *fexp, uint4 *RS) {
    __shared__ int sf[kRhs];
    const int tid = threadIdx.x;
    if (tid < kRhs) sf[tid] = kZeroExp;
    __syncthreads();
    int mx = kZeroExp;  // every index this thread visits has right-hand side tid % 16
    for (int idx = tid; idx < rexp_n * kRhs; idx += blockDim.x) mx = max(mx, rexp[idx]);
    atomicMax(&sf[tid & (kRhs - 1)], mx);
    __syncthreads();
    if (tid < kRhs) {
        const int f = sf[tid];
        sf[tid] = (f >= kNonFinite) ? kNonFinite : (f == kZeroExp ? kZeroExp : f + 2);
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid < kRhs) fexp[tid] = sf[tid];
    const int nsteps = (m + kKst - 1) / kKst;
    for (int idx = blockIdx.x * blockDim.x + tid; idx < nsteps * 32; idx += gridDim.x * blockDim.x) {
        const int s = idx >> 5, j = (idx >> 1) & 15, h = idx & 1;
        const bool live = j < nrhs && sf[j] > kZeroExp && sf[j] < kNonFinite;
        double v[8];
        int se[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = s * kKst + 8 * h + e;
            v[e] = (live && i < m) ? R[i + ldr * (size_t)j] : 0.0;
            se[e] = live ? -sf[j] : 0;
        }
        oz_stack_put8(reinterpret_cast<unsigned char *>(RS + (size_t)s * 256), h, j, v, se);
    }
}

// ---------------------------------------------------------------------------
// Work items.  Residual: item = 128 rows of A, K = all n columns.  A^T r:
// item = (128 columns of A, one range of range_rows rows); the item's
// partial sums go to partial slot (range index).  A CTA takes items
// blockIdx.x, blockIdx.x + gridDim.x, ...; a cursor walks their 16-K steps.
// ---------------------------------------------------------------------------
struct Cursor {
    int it, s, nsteps;
    int mt;      // residual: row tile; A^T r: column tile
    int q;       // A^T r: range index
    int k0, k1;  // K range of the item
};

__device__ __forceinline__ int oz_nitems(const Args &a) { return a.mode == kResidual ? (a.m + 127) / 128 : ((a.n + 127) / 128) * a.nranges; }

__device__ __forceinline__ void oz_item(const Args &a, int it, Cursor &c) {
    c.it = it;
    c.s = 0;
    if (a.mode == kResidual) {
        c.mt = it;
        c.q = 0;
        c.k0 = 0;
        c.k1 = a.n;
    } else {
        const int nct = (a.n + 127) / 128;
        c.mt = it % nct;
        c.q = it / nct;
        c.k0 = c.q * a.range_rows;
        c.k1 = min(a.m, c.k0 + a.range_rows);
    }
    c.nsteps = max(0, (c.k1 - c.k0 + kKst - 1) / kKst);
}
// first item of this CTA (the host guarantees that every item has a step)
__device__ __forceinline__ bool oz_first(const Args &a, Cursor &c, int nitems) {
    if ((int)blockIdx.x >= nitems) return false;
    oz_item(a, blockIdx.x, c);
    return c.nsteps > 0;
}
__device__ __forceinline__ bool oz_next_item(const Args &a, Cursor &c, int nitems) {
    const int it = c.it + (int)gridDim.x;
    if (it >= nitems) return false;
    oz_item(a, it, c);
    return c.nsteps > 0;
}
__device__ __forceinline__ bool oz_next(const Args &a, Cursor &c, int nitems) { return (++c.s < c.nsteps) ? true : oz_next_item(a, c, nitems); }

// the bulk copies of one step: its eight A blocks (residual: one contiguous
// block column piece; A^T r: eight blocks of a block row), completion counted
// on abar, and its stack image, counted on tbar
__device__ __forceinline__ void oz_load_a(const Args &a, const Cursor &c, unsigned char *dst, uint64_t *abar) {
    const int sb = (c.k0 + c.s * kKst) / kKst;
    mbar_expect_tx(abar, (uint32_t)kRawA);
    if (a.mode == kResidual) {
        bulk_g2s(dst, a.Ad + ((size_t)sb * a.nbr + (size_t)c.mt * 8) * kBlock, (uint32_t)kRawA, abar);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) bulk_g2s(dst + j * kBlock, a.Ad + ((size_t)(c.mt * 8 + j) * a.nbr + (size_t)sb) * kBlock, (uint32_t)kBlock, abar);
    }
}
__device__ __forceinline__ void oz_load_t(const Args &a, const Cursor &c, unsigned char *dst, uint64_t *tbar) {
    const int sb = (c.k0 + c.s * kKst) / kKst;
    mbar_expect_tx(tbar, (uint32_t)kStack);
    bulk_g2s(dst, a.XS + (size_t)sb * 256, (uint32_t)kStack, tbar);
}

// (a template only so that every translation unit may include it)
template <int kTag> __global__ void __launch_bounds__(kThreads, 1) k_oz(Args a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *ra0 = smem + kSmemA, *rt0 = smem + kSmemT;
    uint64_t *a_full = reinterpret_cast<uint64_t *>(smem + kSmemCtl);
    uint64_t *a_empty = a_full + kNA, *t_full = a_empty + kNA, *t_empty = t_full + kNT;
    uint64_t *stg_full = t_empty + kNT, *stg_empty = stg_full + kNS;
    uint64_t *acc_full = stg_empty + kNS, *acc_empty = acc_full + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);
    int *snf = reinterpret_cast<int *>(tmem_slot + 1);
    int *sexp = snf + 1;     // [16] f_j
    int *snan = sexp + 16;   // [16] right-hand side j produces NaN
    int *srmax = snan + 16;  // [16] residual: max exponent of r in this CTA
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nitems = oz_nitems(a);

    if (tid < kRhs) {
        sexp[tid] = a.fexp[tid];
        srmax[tid] = kZeroExp;
    }
    if (tid == 0) {
        *snf = 0;
        for (int i = 0; i < kNA; ++i) {
            tc::mbar_init(&a_full[i], 1);
            tc::mbar_init(&a_empty[i], kConvWarps / 2);  // the converter group of the step
        }
        for (int i = 0; i < kNT; ++i) {
            tc::mbar_init(&t_full[i], 1);
            tc::mbar_init(&t_empty[i], 1);  // the MMA commit
        }
        for (int i = 0; i < kNS; ++i) {
            tc::mbar_init(&stg_full[i], kConvWarps / 2);  // the converter group of the step
            tc::mbar_init(&stg_empty[i], 1);              // the MMA commit
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], 4);
        }
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, kTmemCols);
        tc::tmem_relinquish();
    }
    // an Inf or NaN in A makes every result NaN, one in the other operand its column
    for (int k = tid; k < a.n; k += kThreads)
        if (a.colexp[k] >= kNonFinite) *snf = 1;
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (tid < kRhs) snan[tid] = (*snf != 0 || sexp[tid] >= kNonFinite) ? 1 : 0;
    __syncthreads();

    if (warp == kLoadWarp || warp == kStackWarp) {
        // ------------------------------ the two loaders ------------------------------
        if (lane == 0) {
            const bool isA = (warp == kLoadWarp);
            const int nbuf = isA ? kNA : kNT;
            uint64_t *full = isA ? a_full : t_full, *empty = isA ? a_empty : t_empty;
            Cursor c;
            bool have = oz_first(a, c, nitems), ok = true;
            int t = 0;
            while (have) {
                const int b = t % nbuf;
                if (t >= nbuf && !tc::mbar_wait(&empty[b], (uint32_t)(((t / nbuf) - 1) & 1))) {
                    ok = false;
                    break;
                }
                if (isA) oz_load_a(a, c, ra0 + b * kRawA, &full[b]);
                else oz_load_t(a, c, rt0 + b * kStack, &full[b]);
                ++t;
                have = oz_next(a, c, nitems);
            }
            // no copy may still be in flight when the CTA exits
            for (int u = max(0, t - nbuf); u < t; ++u) tc::mbar_wait(&full[u % nbuf], (uint32_t)((u / nbuf) & 1));
            if (!ok) atomicExch(a.err, (int)kStatusBarrierTimeout);
        }
    } else if (warp < kConvWarps) {
        // ------------------------------- converters ------------------------------
        // group grp takes the steps t = grp, grp + 2, ...; thread (ml, g): row /
        // column ml of the 128-tile, K values 8g .. 8g + 7
        const int grp = warp >> 3, ml = tid & 127, g = (tid >> 7) & 1, r = ml & 15, blk = ml >> 4;
        Cursor c;
        bool have = oz_first(a, c, nitems), ok = true;
        if (have && grp == 1) have = oz_next(a, c, nitems);
        int t = grp;
        while (have) {
            const int b = t % kNA, st = t % kNS;
            if (!tc::mbar_wait(&a_full[b], (uint32_t)((t / kNA) & 1))) {
                ok = false;
                break;
            }
            const unsigned char *rb = ra0 + b * kRawA + blk * kBlock;
            uint32_t wd[8][2];  // the eight elements' packed digits (byte p = u_p xor 64)
            if (a.mode == kResidual) {
                // row r of the block, columns 8g .. 8g + 7
#pragma unroll
                for (int pr = 0; pr < 4; ++pr) {
                    const uint4 q4 = *reinterpret_cast<const uint4 *>(rb + blk_off(r, 8 * g + 2 * pr));
                    wd[2 * pr][0] = q4.x;
                    wd[2 * pr][1] = q4.y;
                    wd[2 * pr + 1][0] = q4.z;
                    wd[2 * pr + 1][1] = q4.w;
                }
            } else {
                // column r of the block, rows 8g .. 8g + 7
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const uint2 q2 = *reinterpret_cast<const uint2 *>(rb + blk_off(8 * g + e, r));
                    wd[e][0] = q2.x;
                    wd[e][1] = q2.y;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&a_empty[b]);
            // plane p, element pair (e, e + 1): the two bytes side by side in the
            // low bytes of two halves, 0x64 above them with the xor undone gives
            // the FP16 numbers 1024 + u; subtracting 1088 leaves d = u - 64 exactly
            uint32_t w[kDig][4];
            const __half2 k1088 = __floats2half2_rn(1088.0f, 1088.0f);
#pragma unroll
            for (int p = 0; p < kDig; ++p) {
                const uint32_t bp = (uint32_t)(p & 3), sel = bp | (bp << 4) | ((4u + bp) << 8) | ((4u + bp) << 12);
#pragma unroll
                for (int e = 0; e < 8; e += 2) {
                    const uint32_t x = (__byte_perm(wd[e][p >> 2], wd[e + 1][p >> 2], sel) & 0x00FF00FFu) ^ 0x64406440u;
                    const __half2 h = __hsub2(*reinterpret_cast<const __half2 *>(&x), k1088);
                    w[p][e >> 1] = *reinterpret_cast<const uint32_t *>(&h);
                }
            }
            if (t >= kNS && !tc::mbar_wait(&stg_empty[st], (uint32_t)(((t / kNS) - 1) & 1))) {
                ok = false;
                break;
            }
            tc::tc_fence_after();
            // plane p of stage st: columns stage + 8p .. 8p + 7 (K pairs); this
            // thread's K values 8g .. 8g + 7 are columns 4g .. 4g + 3 of its lane
            const uint32_t tcol = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(2 * kAccCols + st * kStageCols + 4 * g);
#pragma unroll
            for (int p = 0; p < kDig; ++p) tmem_st4(tcol + (uint32_t)(p * kPlaneCols), w[p][0], w[p][1], w[p][2], w[p][3]);
            tmem_wait_st();
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&stg_full[st]);
            t += 2;
            have = oz_next(a, c, nitems) && oz_next(a, c, nitems);
        }
        if (!ok && lane == 0) atomicExch(a.err, (int)kStatusBarrierTimeout);
    } else if (warp == kMmaWarp) {
        // ------------------------------- MMA issue -------------------------------
        // the whole warp runs the loop (so that the descriptors are warp-uniform
        // values) and one elected lane issues the tcgen05 instructions
        Cursor c;
        bool have = oz_first(a, c, nitems), ok = true;
        int t = 0, cc = 0;
        while (have) {
            const int st = t % kNS, bt = t % kNT, set = cc & 1;
            const bool first = (c.s % kChunkSteps) == 0;
            const bool last = (c.s % kChunkSteps) == kChunkSteps - 1 || c.s == c.nsteps - 1;
            bool w_ok = tc::mbar_wait(&stg_full[st], (uint32_t)((t / kNS) & 1)) && tc::mbar_wait(&t_full[bt], (uint32_t)((t / kNT) & 1));
            if (w_ok && first && cc >= 2) w_ok = tc::mbar_wait(&acc_empty[set], (uint32_t)(((cc >> 1) - 1) & 1));
            if (!__all_sync(0xFFFFFFFFu, w_ok)) {
                ok = false;
                break;
            }
            tc::tc_fence_after();
            const uint32_t ta = tmem + (uint32_t)(2 * kAccCols + st * kStageCols), sbk = tc::smem_u32(rt0 + bt * kStack), d = tmem + (uint32_t)(set * kAccCols);
            if (tc::elect_one()) {
#pragma unroll
                for (int p = 0; p < kDig; ++p) {
                    const uint64_t bd = tc::smem_desc(sbk + p * 512, 128, 256);
                    umma_f16_ta(d, ta + (uint32_t)(p * kPlaneCols), bd, idesc_f16(128, 16 * (kDig - p)), (first && p == 0) ? 0u : 1u);
                }
                tc::umma_commit(&stg_empty[st]);
                tc::umma_commit(&t_empty[bt]);
                if (last) tc::umma_commit(&acc_full[set]);
            }
            __syncwarp();
            if (last) ++cc;
            ++t;
            have = oz_next(a, c, nitems);
        }
        // every MMA issued has finished before the accumulators are released
        if (t > 0) tc::mbar_wait(&stg_empty[(t - 1) % kNS], (uint32_t)(((t - 1) / kNS) & 1));
        if (!ok && lane == 0) atomicExch(a.err, (int)kStatusBarrierTimeout);
    } else {
        // -------------------------------- drain --------------------------------
        const int qd = warp & 3, ml = qd * 32 + lane;
        int cc = 0;
        bool ok = true;
        Cursor c;
        bool have = oz_first(a, c, nitems);
        long long *acc_i = reinterpret_cast<long long *>(smem + kSmemAcc);  // [16][128]: sum_{L<=4} S_L 2^(7(4-L))
        float *acc_t = reinterpret_cast<float *>(smem + kSmemAcc + 128 * kRhs * 8);  // [16][128]: S_5 + 2^-7 S_6 + 2^-14 S_7
        while (have) {
#pragma unroll
            for (int j = 0; j < kRhs; ++j) {
                acc_i[j * 128 + ml] = 0;
                acc_t[j * 128 + ml] = 0.0f;
            }
            const int nch = (c.nsteps + kChunkSteps - 1) / kChunkSteps;
            for (int ch = 0; ch < nch; ++ch) {
                const int set = cc & 1;
                if (!tc::mbar_wait(&acc_full[set], (uint32_t)((cc >> 1) & 1))) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t tb = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(set * kAccCols);
#pragma unroll
                for (int jh = 0; jh < 2; ++jh) {
                    // column block b holds level 7 - b.  Levels 7..5 by Horner in FP32;
                    // levels 0..4 are exact integers below 2^24: Horner in 64-bit
                    // integers from level 0
                    float S[8], tl[8];
                    long long I[8];
                    tmem_ld8(tb + 8 * jh, S);
#pragma unroll
                    for (int u = 0; u < 8; ++u) tl[u] = S[u];
#pragma unroll
                    for (int b = 1; b < 3; ++b) {
                        tmem_ld8(tb + 16 * b + 8 * jh, S);
#pragma unroll
                        for (int u = 0; u < 8; ++u) tl[u] = fmaf(tl[u], 0x1p-7f, S[u]);
                    }
                    tmem_ld8(tb + 112 + 8 * jh, S);
#pragma unroll
                    for (int u = 0; u < 8; ++u) I[u] = (long long)__float2int_rn(S[u]);
#pragma unroll
                    for (int b = 6; b >= 3; --b) {
                        tmem_ld8(tb + 16 * b + 8 * jh, S);
#pragma unroll
                        for (int u = 0; u < 8; ++u) I[u] = I[u] * 128 + (long long)__float2int_rn(S[u]);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        acc_i[(8 * jh + u) * 128 + ml] += I[u];
                        acc_t[(8 * jh + u) * 128 + ml] += tl[u];
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[set]);
                ++cc;
            }
            // sum_L 2^(-7L) S_L = 2^-28 acc_i + 2^-35 acc_t
            double acc[kRhs];
#pragma unroll
            for (int j = 0; j < kRhs; ++j) acc[j] = fma((double)acc_t[j * 128 + ml], 0x1p-35, (double)acc_i[j * 128 + ml] * 0x1p-28);
            if (!ok) break;
            if (a.mode == kResidual) {
                const int i = c.mt * 128 + ml;
#pragma unroll
                for (int j = 0; j < kRhs; ++j) {
                    int ex = kZeroExp;
                    if (j < a.nrhs && i < a.m) {
                        const double r = snan[j] ? __longlong_as_double(0x7FF8000000000000LL) : a.B[i + a.ldb * (size_t)j] - scalbn(acc[j], sexp[j] - 14);
                        a.out[i + a.ldo * (size_t)j] = r;
                        ex = oz_exp(r);
                    }
                    ex = __reduce_max_sync(0xFFFFFFFFu, ex);
                    if (lane == 0 && ex > kZeroExp) atomicMax(&srmax[j], ex);
                }
            } else {
                const int k = c.mt * 128 + ml;
                if (k < a.n) {
                    const int ek = a.colexp[k];
                    double *o = a.out + (size_t)c.q * a.pstride + k;
#pragma unroll
                    for (int j = 0; j < kRhs; ++j)
                        if (j < a.nrhs) o[a.ldo * (size_t)j] = snan[j] ? __longlong_as_double(0x7FF8000000000000LL) : scalbn(acc[j], ek + sexp[j] - 14);
                }
            }
            have = oz_next_item(a, c, nitems);
        }
        if (!ok && lane == 0) atomicExch(a.err, (int)kStatusBarrierTimeout);
    }
    tc::tc_fence_before();
    __syncthreads();
    if (a.mode == kResidual && tid < kRhs) a.rexp_out[blockIdx.x * kRhs + tid] = srmax[tid];
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
}


} // namespace oz

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
constexpr int kOzMaxGrid = 256;

inline int oz_grid(int nitems) { return std::max(1, std::min({nitems, device_facts().sm_count, kOzMaxGrid})); }
inline int oz_groups(size_t nrhs) { return (int)((nrhs + oz::kRhs - 1) / oz::kRhs); }
// rows per partial of g = A^T r: about one item per SM, a multiple of 16 rows
inline int oz_range_rows(int m, int n) {
    const int nct = (n + 127) / 128;
    const int want = std::max(1, std::min(device_facts().sm_count, kOzMaxGrid) / nct);
    int rr = (m + want - 1) / want;
    rr = (rr + oz::kKst - 1) / oz::kKst * oz::kKst;
    return std::max(rr, oz::kKst);
}
inline int oz_nranges(int m, int n) { return (m + oz_range_rows(m, n) - 1) / oz_range_rows(m, n); }

// Device workspace of the FP64-accurate products (regions 256-byte aligned)
struct OzWork {
    int *colexp;        // n
    unsigned char *Ad;  // packed digits of A: nbr x nbc blocks of 16 x 16 elements (2 KB)
    uint4 *XS;          // stack images of x: ceil(n/16) x 256
    uint4 *RS;          // stack images of r: ceil(m/16) x 256
    int *fexp;          // 16
    int *rexp;          // groups x kOzMaxGrid x 16
    double *P;          // kOzMaxGrid x n x 16 partials of A^T r
    static size_t al(size_t b) { return (b + 255) / 256 * 256; }
    static int nbr(size_t m) { return (int)(8 * ((m + 127) / 128)); }
    static int nbc(size_t n) { return (int)(8 * ((n + 127) / 128)); }
    static size_t bytes(size_t m, size_t n, size_t nrhs) {
        return al(n * sizeof(int)) + al((size_t)nbr(m) * nbc(n) * oz::kBlock) + al((n + 15) / 16 * 4096) + al((m + 15) / 16 * 4096) + al(oz::kRhs * sizeof(int)) +
               al((size_t)oz_groups(nrhs) * kOzMaxGrid * oz::kRhs * sizeof(int)) + al((size_t)kOzMaxGrid * n * oz::kRhs * sizeof(double)) + 256;
    }
    void carve(Carver &cv, size_t m, size_t n, size_t nrhs) {
        colexp = cv.take<int>(n);
        Ad = cv.take<unsigned char>((size_t)nbr(m) * nbc(n) * oz::kBlock);
        XS = cv.take<uint4>((n + 15) / 16 * 256);
        RS = cv.take<uint4>((m + 15) / 16 * 256);
        fexp = cv.take<int>(oz::kRhs);
        rexp = cv.take<int>((size_t)oz_groups(nrhs) * kOzMaxGrid * oz::kRhs);
        P = cv.take<double>((size_t)kOzMaxGrid * n * oz::kRhs);
    }
};

inline int oz_attr() { return kernel_attr((const void *)oz::k_oz<0>, oz::kSmem); }

// once per A: column scales, the packed digits, and the FP32 copy Af when
// given (with ||Af(:,k)||^2 into sumsq when both are given)
inline int oz_prepare_a(int m, int n, const double *A, size_t lda, const OzWork &w, double *sumsq, float *Af, size_t ldf, cudaStream_t st) {
    oz::k_col_exp<0><<<(unsigned)std::min(n, 8192), 256, 0, st>>>(m, n, A, lda, w.colexp);
    RNPGPU_CHECK_LAUNCH();
    const int nbr = OzWork::nbr((size_t)m), nbc = OzWork::nbc((size_t)n);
    const dim3 grid((unsigned)std::min(nbr / 8, 65535), (unsigned)std::min(nbc, 65535));
    oz::k_adigits<0><<<grid, 256, 0, st>>>(m, n, nbr, nbc, A, lda, w.colexp, w.Ad, Af, ldf);
    RNPGPU_CHECK_LAUNCH();
    if (sumsq && Af) {
        oz::k_col_sumsq_f32<0><<<(unsigned)std::min(n, 8192), 256, 0, st>>>(m, n, Af, ldf, sumsq);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

// the same for columns [c0, c0 + w) only (c0 a multiple of 128; the last
// range also writes the zero blocks that pad the packed digits to whole
// 128-column groups): a matrix prepared range by range as it arrives
inline int oz_prepare_cols(int m, int n, int c0, int w, const double *A, size_t lda, const OzWork &ow, double *sumsq, float *Af, size_t ldf, cudaStream_t st) {
    if (w <= 0) return kOk;
    oz::k_col_exp<0><<<(unsigned)std::min(w, 8192), 256, 0, st>>>(m, w, A + (size_t)c0 * lda, lda, ow.colexp + c0);
    RNPGPU_CHECK_LAUNCH();
    const int nbr = OzWork::nbr((size_t)m);
    const int nbc = (c0 + w >= n) ? OzWork::nbc((size_t)n) - c0 / 16 : w / 16;
    const dim3 grid((unsigned)std::min(nbr / 8, 65535), (unsigned)std::min(nbc, 65535));
    oz::k_adigits<0><<<grid, 256, 0, st>>>(m, w, nbr, nbc, A + (size_t)c0 * lda, lda, ow.colexp + c0, ow.Ad + (size_t)(c0 / 16) * nbr * oz::kBlock,
                                           Af ? Af + (size_t)c0 * ldf : nullptr, ldf);
    RNPGPU_CHECK_LAUNCH();
    if (sumsq && Af) {
        oz::k_col_sumsq_f32<0><<<(unsigned)std::min(w, 8192), 256, 0, st>>>(m, w, Af + (size_t)c0 * ldf, ldf, sumsq + c0);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

// r = b - A x (m x nrhs), FP64-accurate, A prepared by oz_prepare_a
inline int oz_residual(int m, int n, int nrhs, const OzWork &w, const double *x, size_t ldx, const double *b, size_t ldb, double *r, size_t ldr, cudaStream_t st) {
    if (int rc = oz_attr()) return rc;
    int *err = device_status_ptr();
    if (err == nullptr) return kErrCuda;
    const int grid = oz_grid((m + 127) / 128);
    KScope ks("residual_fp64", st);
    for (int g0 = 0, grp = 0; g0 < nrhs; g0 += oz::kRhs, ++grp) {
        const int ng = std::min(oz::kRhs, nrhs - g0);
        const unsigned xgrid = (unsigned)std::max(1, std::min((n + 15) / 16 * 32 / 256, 64));
        oz::k_xstack<0><<<xgrid, 256, 0, st>>>(n, ng, x + ldx * (size_t)g0, ldx, w.colexp, w.fexp, w.XS);
        RNPGPU_CHECK_LAUNCH();
        oz::Args a{};
        a.mode = oz::kResidual;
        a.m = m;
        a.n = n;
        a.nrhs = ng;
        a.Ad = w.Ad;
        a.nbr = OzWork::nbr((size_t)m);
        a.XS = w.XS;
        a.fexp = w.fexp;
        a.B = b + ldb * (size_t)g0;
        a.ldb = ldb;
        a.out = r + ldr * (size_t)g0;
        a.ldo = ldr;
        a.colexp = w.colexp;
        a.rexp_out = w.rexp + (size_t)grp * kOzMaxGrid * oz::kRhs;
        a.err = err;
        oz::k_oz<0><<<grid, oz::kThreads, oz::kSmem, st>>>(a);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

// g = A^T r (n x nrhs), FP64-accurate; r must come from oz_residual (the
// exponents of its entries are in w.rexp)
inline int oz_normal(int m, int n, int nrhs, const OzWork &w, const double *r, size_t ldr, double *g, size_t ldg, cudaStream_t st) {
    if (int rc = oz_attr()) return rc;
    int *err = device_status_ptr();
    if (err == nullptr) return kErrCuda;
    const int rgrid = oz_grid((m + 127) / 128);
    const int rr = oz_range_rows(m, n), nr = oz_nranges(m, n);
    const int grid = oz_grid(((n + 127) / 128) * nr);
    const unsigned sgrid = (unsigned)std::max(1, std::min((m + 15) / 16 * 32 / 256, 2 * std::max(1, device_facts().sm_count)));
    KScope ks("normal_eq_fp64", st);
    for (int g0 = 0, grp = 0; g0 < nrhs; g0 += oz::kRhs, ++grp) {
        const int ng = std::min(oz::kRhs, nrhs - g0);
        oz::k_rstack<0><<<sgrid, 256, 0, st>>>(m, ng, r + ldr * (size_t)g0, ldr, w.rexp + (size_t)grp * kOzMaxGrid * oz::kRhs, rgrid, w.fexp, w.RS);
        RNPGPU_CHECK_LAUNCH();
        oz::Args a{};
        a.mode = oz::kNormal;
        a.m = m;
        a.n = n;
        a.nrhs = ng;
        a.Ad = w.Ad;
        a.nbr = OzWork::nbr((size_t)m);
        a.XS = w.RS;
        a.fexp = w.fexp;
        a.out = w.P;
        a.ldo = (size_t)n;
        a.pstride = (size_t)n * oz::kRhs;
        a.colexp = w.colexp;
        a.range_rows = rr;
        a.nranges = nr;
        a.err = err;
        oz::k_oz<0><<<grid, oz::kThreads, oz::kSmem, st>>>(a);
        RNPGPU_CHECK_LAUNCH();
        const dim3 gs((unsigned)((n + 63) / 64), (unsigned)ng);
        k_reduce_splits<double><<<gs, 256, 0, st>>>(w.P, (size_t)n, (size_t)n * oz::kRhs, nr, n, g + ldg * (size_t)g0, ldg);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

// r = b - A x and, when g != nullptr, g = A^T r, both FP64-accurate
inline int ls_residual(size_t m, size_t n, size_t nrhs, const double *a, size_t lda, const double *x, size_t ldx, const double *b, size_t ldb, double *r, size_t ldr, double *g,
                       size_t ldg, void *work, size_t *lwork_bytes) {
    if (lwork_bytes == nullptr) return -15;
    if (m == 0 || nrhs == 0) return kOk;
    if (lda < std::max<size_t>(m, 1)) return -5;
    if (ldx < std::max<size_t>(n, 1)) return -7;
    if (ldb < m) return -9;
    if (ldr < m) return -11;
    if (g != nullptr && ldg < std::max<size_t>(n, 1)) return -13;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX) return -1;
    const size_t need = OzWork::bytes(m, n, nrhs);
    if (work == nullptr || *lwork_bytes == 0) {
        *lwork_bytes = need;
        return kOk;
    }
    if (*lwork_bytes < need) return -15;
    if (b == nullptr) return -8;
    if (r == nullptr) return -10;
    cudaStream_t st = current_stream();
    if (n == 0) {
        if (r != b) RNPGPU_CHECK(cudaMemcpy2DAsync(r, ldr * sizeof(double), b, ldb * sizeof(double), m * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, st));
        return kOk;
    }
    if (a == nullptr) return -4;
    if (x == nullptr) return -6;
    Carver cv(work);
    OzWork w;
    w.carve(cv, m, n, nrhs);
    int rc;
    if ((rc = oz_prepare_a((int)m, (int)n, a, lda, w, nullptr, nullptr, 0, st))) return rc;
    if ((rc = oz_residual((int)m, (int)n, (int)nrhs, w, x, ldx, b, ldb, r, ldr, st))) return rc;
    if (g != nullptr && (rc = oz_normal((int)m, (int)n, (int)nrhs, w, r, ldr, g, ldg, st))) return rc;
    return kOk;
}

} // namespace rnpgpu
