// oz_gemm.cuh — the FP64 products of the mixed least-squares refinement,
// r = b - A x and g = A^T r, on the BF16 tensor cores by exact integer
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
//   d_p an integer in [-64, 64] (exact in BF16);
// * a digit product d_p D_q is an integer of magnitude <= 2^12; the products
//   of one level L = p + q go into one FP32 tensor-memory accumulator.  Over
//   512 K values a level L <= 4 stays below 5 * 2^12 * 2^9 < 2^24, so those
//   sums are exact integers; levels 5..7 weigh less than 2^-35 relative, where
//   FP32 rounding of their sums no longer matters; levels >= 8 are dropped;
// * the levels are combined in FP64 every 512 K values and at the end,
//   result = 2^scale * 2^-14 * sum_L 2^(-7L) S_L.
//
// The error is that of representing both operands to 2^-56 of their scales
// plus the dropped levels: about 2^-50 of sum_k 2^e_k |x_kj| 2^(f_j - e_k) —
// the accuracy of an FP64 dot product, independent of the condition of A.
//
// Tensor-core layout.  One accumulation D (128 TMEM lanes x 128 FP32 columns)
// per 128 rows of A (residual) or 128 columns of A (A^T r): lane = that row or
// column, column c = 16 b + j holds level 7 - b of right-hand side j.  The
// A tile's digits are eight K-major planes (the UMMA A operand, M = 128); the
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
// per element, byte p = (d_p + 64) xor 64, so that zero bytes mean zero
// digits (the padding to whole 128 x 128 tiles is zero).  The other operand
// (x, or r for A^T r) is small; k_xstack / k_rstack compute its scales f_j and
// write its digits directly as the BF16 digit-stack image of every 16-K step.
//
// CTA of k_oz: 8 producer warps (cp.async of the packed digits and the stack
// images NR - 1 steps ahead, byte -> BF16 expansion, 16-byte stores into the
// digit stage; one thread issues the eight tcgen05.mma per 16-K step and
// commits them to the stage's mbarrier) and 4 drain warps (tcgen05.ld of a
// finished accumulator, FP64 level combination, output), two accumulator sets
// so that the drain of one chunk overlaps the MMAs of the next.  Every wait is
// bounded.
#pragma once
#include "ls_kernels.cuh"
#include "qr_driver.cuh"

namespace rnpgpu {
namespace oz {

constexpr int kDig = 8;                          // digits per operand
constexpr int kKst = 16;                         // K values per step (one UMMA K)
constexpr int kChunkSteps = 32;                  // steps per exact accumulation chunk (512 K)
constexpr int kRhs = 16;                         // right-hand sides per launch
constexpr int kProd = 256;                       // producer threads (warps 0..7)
constexpr int kThreads = kProd + 128;            // + drain warps 8..11
constexpr int kNR = 6;                           // FP64 staging buffers (kNR - 1 steps ahead)
constexpr int kPlane = 128 * kKst * 2;           // one digit plane of the A tile (4 KB)
constexpr int kStack = kDig * kRhs * kKst * 2;   // digit stack of the other operand (4 KB)
constexpr int kStage = kDig * kPlane + kStack;   // 36 KB
constexpr int kRawA = kProd * 64;                // 8 packed elements per producer thread (16 KB)
constexpr int kRawX = kStack;                    // one stack image (16 bytes per producer thread)
constexpr int kSmemStages = 2 * kStage;
constexpr int kSmemRawA = kSmemStages;
constexpr int kSmemRawX = kSmemRawA + kNR * kRawA;
constexpr int kSmemCtl = kSmemRawX + kNR * kRawX;
constexpr int kSmem = kSmemCtl + 256;
constexpr int kZeroExp = -(1 << 20);             // scale of an all-zero column / vector
constexpr int kNonFinite = 1 << 20;              // an Inf or NaN was seen
constexpr unsigned long long kBias = 0x81020408102040ull;  // 64 * sum_q 128^q, q = 0..7

enum Mode : int { kResidual = 0, kNormal = 1 };

struct Args {
    int mode;
    int m, n, nrhs;             // nrhs <= 16
    const uint2 *Ad;            // packed digits of A, padded to whole 128 x 128 tiles
    size_t ldd;
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

// BF16 bits of a digit: an exact FP32 integer of magnitude <= 64 is its own top 16 bits
__device__ __forceinline__ uint16_t oz_digit_bf16(uint32_t u) { return (uint16_t)(__float_as_uint(oz_digit_value(u)) >> 16); }

// packed form of one element: byte p = u_p xor 64 (zero bytes = zero digits)
__device__ __forceinline__ uint2 oz_pack(const uint32_t (&u)[kDig]) {
    uint2 w;
    w.x = (u[0] | (u[1] << 8) | (u[2] << 16) | (u[3] << 24)) ^ 0x40404040u;
    w.y = (u[4] | (u[5] << 8) | (u[6] << 16) | (u[7] << 24)) ^ 0x40404040u;
    return w;
}

// byte offset of (row, k) in a K-major, no-swizzle BF16 tile with kKst = 16
// columns: core matrix (row/8, k/8) is 128 contiguous bytes
__device__ __forceinline__ uint32_t toff(int row, int k) { return (uint32_t)(((row >> 3) * 2 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2); }

template <int BYTES> __device__ __forceinline__ void cp_zfill(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src), "n"(BYTES), "r"(valid ? BYTES : 0) : "memory");
}
template <int N> __device__ __forceinline__ void cp_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) { asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory"); }
// barrier 1 over the producer warps, and-reduction of a flag
__device__ __forceinline__ int producers_and(int pred) {
    int r;
    asm volatile("{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.and.pred q, 1, %2, p;\nselp.s32 %0, 1, 0, q;\n}\n" : "=r"(r) : "r"(pred), "n"(kProd) : "memory");
    return r;
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
// when the column holds an Inf or NaN) and, when sumsq != nullptr,
// ||A(:,k)||_2^2 in FP64 (the same order of summation as k_col_sumsq); one
// block per column
template <int kTag> __global__ void __launch_bounds__(256) k_col_exp_sumsq(int m, int n, const double *A, size_t lda, int *colexp, double *sumsq) {
    __shared__ double s[8];
    __shared__ int sx[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        double acc = 0.0;
        int ex = kZeroExp;
        for (int r = tid; r < m; r += 256) {
            const double v = A[r + (size_t)c * lda];
            acc += v * v;
            ex = max(ex, oz_exp(v));
        }
        acc = warp_sum(acc);
        ex = __reduce_max_sync(0xFFFFFFFFu, ex);
        if (lane == 0) {
            s[warp] = acc;
            sx[warp] = ex;
        }
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            int e = kZeroExp;
            for (int w = 0; w < 8; ++w) {
                t += s[w];
                e = max(e, sx[w]);
            }
            colexp[c] = (e >= kNonFinite) ? kNonFinite : (e == kZeroExp ? kZeroExp : e + 2);
            if (sumsq) sumsq[c] = t;
        }
        __syncthreads();
    }
}

// Ad(0:m, 0:n) = packed digits of A relative to 2^e_k; Af(0:m, 0:n) =
// (float) A when Af != nullptr (the working copy of the FP32 factorization)
template <int kTag> __global__ void __launch_bounds__(256) k_adigits(int m, int n, const double *A, size_t lda, const int *colexp, uint2 *Ad, size_t ldd, float *Af, size_t ldf) {
    for (int c = blockIdx.y; c < n; c += gridDim.y) {
        const int ek = colexp[c];
        const bool live = ek > kZeroExp && ek < kNonFinite;
        for (int r = blockIdx.x * 256 + threadIdx.x; r < m; r += gridDim.x * 256) {
            const double v = A[r + (size_t)c * lda];
            if (Af) Af[r + (size_t)c * ldf] = (float)v;
            uint2 w = make_uint2(0u, 0u);
            if (live) {
                uint32_t u[kDig];
                oz_fields(v, -ek, u);
                w = oz_pack(u);
            }
            Ad[r + (size_t)c * ldd] = w;
        }
    }
}

// the digit stack image of one element of the other operand: digit q of
// right-hand side j at K offset kk goes to block 7 - q of the image
__device__ __forceinline__ void oz_stack_put(unsigned char *img, int kk, int j, double v, int se) {
    uint32_t u[kDig];
    oz_fields(v, se, u);
#pragma unroll
    for (int q = 0; q < kDig; ++q) *reinterpret_cast<uint16_t *>(img + toff(16 * (7 - q) + j, kk)) = oz_digit_bf16(u[q]);
}

// x (n x nrhs, nrhs <= 16) for the residual: f_j = max_k (floor(log2 |x_kj|) + e_k) + 2,
// then the stack image of every 16-row step of x scaled by 2^(e_k - f_j)
template <int kTag> __global__ void __launch_bounds__(1024) k_xstack(int n, int nrhs, const double *X, size_t ldx, const int *colexp, int *fexp, uint4 *XS) {
    __shared__ int sf[kRhs];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < kRhs) sf[tid] = kZeroExp;
    __syncthreads();
    int mx[kRhs];
#pragma unroll
    for (int j = 0; j < kRhs; ++j) mx[j] = kZeroExp;
    for (int k = tid; k < n; k += blockDim.x) {
        const int ek = colexp[k];
#pragma unroll
        for (int j = 0; j < kRhs; ++j) {
            if (j < nrhs) {
                const int ex = oz_exp(X[k + ldx * (size_t)j]);
                if (ex >= kNonFinite) mx[j] = kNonFinite;
                else if (ex > kZeroExp && ek > kZeroExp && ek < kNonFinite) mx[j] = max(mx[j], ex + ek + 2);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kRhs; ++j) {
        const int r = __reduce_max_sync(0xFFFFFFFFu, mx[j]);
        if (lane == 0 && r > kZeroExp) atomicMax(&sf[j], r);
    }
    __syncthreads();
    if (tid < kRhs) fexp[tid] = sf[tid];
    const int nsteps = (n + kKst - 1) / kKst;
    for (int idx = tid; idx < nsteps * 256; idx += blockDim.x) {
        const int s = idx >> 8, kk = idx & 15, j = (idx >> 4) & 15, k = s * kKst + kk;
        double v = 0.0;
        int se = 0;
        if (k < n && j < nrhs && sf[j] < kNonFinite) {
            const int ek = colexp[k];
            if (ek > kZeroExp && ek < kNonFinite) {
                v = X[k + ldx * (size_t)j];
                se = ek - sf[j];
            }
        }
        oz_stack_put(reinterpret_cast<unsigned char *>(XS + (size_t)s * 256), kk, j, v, se);
    }
}

// r (m x nrhs, nrhs <= 16) for A^T r: f_j = max over the residual's CTAs of
// max_i floor(log2 |r_ij|), plus 2; then the stack image of every 16-row step
// of r scaled by 2^-f_j.  CTA 0 writes f_j.
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
    const int nsteps = (m + kKst - 1) / kKst, kk = tid & 15, j = tid >> 4;
    for (int s = blockIdx.x; s < nsteps; s += gridDim.x) {
        const int i = s * kKst + kk;
        double v = 0.0;
        int se = 0;
        if (i < m && j < nrhs && sf[j] > kZeroExp && sf[j] < kNonFinite) {
            v = R[i + ldr * (size_t)j];
            se = -sf[j];
        }
        oz_stack_put(reinterpret_cast<unsigned char *>(RS + (size_t)s * 256), kk, j, v, se);
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

// issue the cp.async copies of one step owned by producer tid: eight packed
// elements of A (zero-filled outside A: zero bytes are zero digits) and 16
// bytes of the step's stack image
__device__ __forceinline__ void oz_prefetch(const Args &a, const Cursor &c, unsigned char *rawA, unsigned char *rawX, int tid) {
    const int kb = c.k0 + c.s * kKst;
    if (a.mode == kResidual) {
        const int ml = tid & 127, g = tid >> 7, i = c.mt * 128 + ml;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = kb + 8 * g + e;
            const bool ok = i < a.m && k < c.k1;
            cp_zfill<8>(rawA + ((e >> 1) * kProd + tid) * 16 + (e & 1) * 8, ok ? a.Ad + i + a.ldd * (size_t)k : a.Ad, ok);
        }
    } else {
        const int ml = tid >> 1, g = tid & 1, col = c.mt * 128 + ml;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = kb + 8 * g + e;
            const bool ok = col < a.n && i < c.k1;
            cp_zfill<8>(rawA + ((e >> 1) * kProd + tid) * 16 + (e & 1) * 8, ok ? a.Ad + i + a.ldd * (size_t)col : a.Ad, ok);
        }
    }
    cp_zfill<16>(rawX + tid * 16, a.XS + (size_t)(kb / kKst) * 256 + tid, true);
}

// (a template only so that every translation unit may include it)
template <int kTag> __global__ void __launch_bounds__(kThreads, 1) k_oz(Args a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *rawA0 = smem + kSmemRawA;
    unsigned char *rawX0 = smem + kSmemRawX;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kSmemCtl);  // 0,1 stage; 2,3 acc full; 4,5 acc empty
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 6);
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
        for (int i = 0; i < 4; ++i) tc::mbar_init(&bars[i], 1);
        tc::mbar_init(&bars[4], 4);
        tc::mbar_init(&bars[5], 4);
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, 256);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // producers: start the copies of the first kNR - 1 steps
    Cursor cv, pf;
    bool has_cv = false, has_pf = false;
    if (tid < kProd) {
        has_cv = oz_first(a, cv, nitems);
        pf = cv;
        has_pf = has_cv;
        for (int u = 0; u < kNR - 1; ++u) {
            if (has_pf) {
                oz_prefetch(a, pf, rawA0 + u * kRawA, rawX0 + u * kRawX, tid);
                has_pf = oz_next(a, pf, nitems);
            }
            cp_async_commit();
        }
    }
    // an Inf or NaN in A makes every result NaN, one in the other operand its column
    for (int k = tid; k < a.n; k += kThreads)
        if (a.colexp[k] >= kNonFinite) *snf = 1;
    __syncthreads();
    if (tid < kRhs) snan[tid] = (*snf != 0 || sexp[tid] >= kNonFinite) ? 1 : 0;
    __syncthreads();

    if (tid < kProd) {
        // ------------------------------ producers ------------------------------
        bool ok = true;
        int t = 0, cc = 0, last_commit = -1;
        const int ml = (a.mode == kResidual) ? (tid & 127) : (tid >> 1);
        const int g = (a.mode == kResidual) ? (tid >> 7) : (tid & 1);
        while (has_cv) {
            // keep kNR - 1 steps of copies in flight
            if (has_pf) {
                const int b = (t + kNR - 1) % kNR;
                oz_prefetch(a, pf, rawA0 + b * kRawA, rawX0 + b * kRawX, tid);
                has_pf = oz_next(a, pf, nitems);
            }
            cp_async_commit();
            cp_wait_group<kNR - 1>();
            const int rb = t % kNR;
            const unsigned char *ra = rawA0 + rb * kRawA;
            uint32_t wd[8][2];  // packed digits of the eight elements, bytes decoded to u = d + 64
#pragma unroll
            for (int pr = 0; pr < 4; ++pr) {
                const uint4 q4 = *reinterpret_cast<const uint4 *>(ra + (pr * kProd + tid) * 16);
                wd[2 * pr][0] = q4.x ^ 0x40404040u;
                wd[2 * pr][1] = q4.y ^ 0x40404040u;
                wd[2 * pr + 1][0] = q4.z ^ 0x40404040u;
                wd[2 * pr + 1][1] = q4.w ^ 0x40404040u;
            }
            const uint4 xs = *reinterpret_cast<const uint4 *>(rawX0 + rb * kRawX + tid * 16);
            // plane p, element pair (e, e + 1): two BF16 digits in one word
            uint32_t w[kDig][4];
#pragma unroll
            for (int p = 0; p < kDig; ++p) {
                const uint32_t sel = 0x7440u | (uint32_t)(p & 3);
#pragma unroll
                for (int e = 0; e < 8; e += 2) {
                    const float fa = __uint_as_float(__byte_perm(wd[e][p >> 2], 0x4B000000u, sel)) - 8388672.0f;
                    const float fb = __uint_as_float(__byte_perm(wd[e + 1][p >> 2], 0x4B000000u, sel)) - 8388672.0f;
                    w[p][e >> 1] = __byte_perm(__float_as_uint(fa), __float_as_uint(fb), 0x7632);
                }
            }
            // the MMAs of step t - 2 read this stage
            if (t >= 2 && ok) ok = tc::mbar_wait(&bars[t & 1], (uint32_t)(((t >> 1) - 1) & 1));
            unsigned char *stg = smem + (t & 1) * kStage;
#pragma unroll
            for (int p = 0; p < kDig; ++p)
                *reinterpret_cast<uint4 *>(stg + p * kPlane + toff(ml, 8 * g)) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
            *reinterpret_cast<uint4 *>(stg + kDig * kPlane + tid * 16) = xs;
            tc::fence_proxy_async();
            if (!producers_and(ok ? 1 : 0)) {
                ok = false;
                break;
            }
            const bool first = (cv.s % kChunkSteps) == 0;
            const bool last = (cv.s % kChunkSteps) == kChunkSteps - 1 || cv.s == cv.nsteps - 1;
            if (tid == 0) {
                const int set = cc & 1;
                if (first && cc >= 2) ok = tc::mbar_wait(&bars[4 + set], (uint32_t)(((cc >> 1) - 1) & 1));
                if (ok) {
                    tc::tc_fence_after();
                    const uint32_t sb = tc::smem_u32(stg), d = tmem + (uint32_t)(set * 128);
#pragma unroll
                    for (int p = 0; p < kDig; ++p) {
                        const uint64_t ad = tc::smem_desc(sb + p * kPlane, 128, 256);
                        const uint64_t bd = tc::smem_desc(sb + kDig * kPlane + p * 512, 128, 256);
                        tc::umma_bf16(d, ad, bd, tc::idesc_bf16(128, 16 * (kDig - p)), (first && p == 0) ? 0u : 1u);
                    }
                    tc::umma_commit(&bars[t & 1]);
                    last_commit = t;
                    if (last) tc::umma_commit(&bars[2 + set]);
                }
            }
            if (last) ++cc;
            ++t;
            has_cv = oz_next(a, cv, nitems);
        }
        cp_async_wait_all();
        // every MMA issued has finished before the accumulators are released
        if (tid == 0 && last_commit >= 0) tc::mbar_wait(&bars[last_commit & 1], (uint32_t)((last_commit >> 1) & 1));
        if (!ok && tid == 0) atomicExch(a.err, (int)kStatusBarrierTimeout);
    } else {
        // -------------------------------- drain --------------------------------
        const int qd = warp & 3, ml = qd * 32 + lane;
        int cc = 0;
        bool ok = true;
        Cursor c;
        bool have = oz_first(a, c, nitems);
        while (have) {
            double acc[kRhs];
#pragma unroll
            for (int j = 0; j < kRhs; ++j) acc[j] = 0.0;
            const int nch = (c.nsteps + kChunkSteps - 1) / kChunkSteps;
            for (int ch = 0; ch < nch; ++ch) {
                const int set = cc & 1;
                if (!tc::mbar_wait(&bars[2 + set], (uint32_t)((cc >> 1) & 1))) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t tb = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(set * 128);
#pragma unroll
                for (int jh = 0; jh < 2; ++jh) {
                    // Horner over the levels, 7 (column block 0) down to 0 (block 7):
                    // levels 7..5 in FP32, then FP64
                    float S[8], tl[8];
                    double h[8];
                    tmem_ld8(tb + 8 * jh, S);
#pragma unroll
                    for (int u = 0; u < 8; ++u) tl[u] = S[u];
#pragma unroll
                    for (int b = 1; b < 3; ++b) {
                        tmem_ld8(tb + 16 * b + 8 * jh, S);
#pragma unroll
                        for (int u = 0; u < 8; ++u) tl[u] = fmaf(tl[u], 0x1p-7f, S[u]);
                    }
                    tmem_ld8(tb + 48 + 8 * jh, S);
#pragma unroll
                    for (int u = 0; u < 8; ++u) h[u] = fma((double)tl[u], 0x1p-7, (double)S[u]);
#pragma unroll
                    for (int b = 4; b < 8; ++b) {
                        tmem_ld8(tb + 16 * b + 8 * jh, S);
#pragma unroll
                        for (int u = 0; u < 8; ++u) h[u] = fma(h[u], 0x1p-7, (double)S[u]);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[8 * jh + u] += h[u];
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&bars[4 + set]);
                ++cc;
            }
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
        tc::tmem_dealloc(tmem, 256);
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
    int *colexp;  // n
    uint2 *Ad;    // m x n packed digits of A (leading dimension m)
    uint4 *XS;    // stack images of x: ceil(n/16) x 256
    uint4 *RS;    // stack images of r: ceil(m/16) x 256
    int *fexp;    // 16
    int *rexp;    // groups x kOzMaxGrid x 16
    double *P;    // kOzMaxGrid x n x 16 partials of A^T r
    static size_t al(size_t b) { return (b + 255) / 256 * 256; }
    static size_t bytes(size_t m, size_t n, size_t nrhs) {
        return al(n * sizeof(int)) + al(m * n * sizeof(uint2)) + al((n + 15) / 16 * 4096) + al((m + 15) / 16 * 4096) + al(oz::kRhs * sizeof(int)) +
               al((size_t)oz_groups(nrhs) * kOzMaxGrid * oz::kRhs * sizeof(int)) + al((size_t)kOzMaxGrid * n * oz::kRhs * sizeof(double)) + 256;
    }
    void carve(Carver &cv, size_t m, size_t n, size_t nrhs) {
        colexp = cv.take<int>(n);
        Ad = cv.take<uint2>(m * n);
        XS = cv.take<uint4>((n + 15) / 16 * 256);
        RS = cv.take<uint4>((m + 15) / 16 * 256);
        fexp = cv.take<int>(oz::kRhs);
        rexp = cv.take<int>((size_t)oz_groups(nrhs) * kOzMaxGrid * oz::kRhs);
        P = cv.take<double>((size_t)kOzMaxGrid * n * oz::kRhs);
    }
};

inline int oz_attr() {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, []() { attr = cudaFuncSetAttribute((const void *)oz::k_oz<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::kSmem); });
    RNPGPU_CHECK(attr);
    return kOk;
}

// once per A: column scales (and ||A(:,k)||^2 into sumsq when given), the
// packed digits, and the FP32 copy Af when given
inline int oz_prepare_a(int m, int n, const double *A, size_t lda, const OzWork &w, double *sumsq, float *Af, size_t ldf, cudaStream_t st) {
    oz::k_col_exp_sumsq<0><<<(unsigned)std::min(n, 4096), 256, 0, st>>>(m, n, A, lda, w.colexp, sumsq);
    RNPGPU_CHECK_LAUNCH();
    const dim3 grid((unsigned)std::min((m + 255) / 256, 2048), (unsigned)std::min(n, 65535));
    oz::k_adigits<0><<<grid, 256, 0, st>>>(m, n, A, lda, w.colexp, w.Ad, (size_t)m, Af, ldf);
    RNPGPU_CHECK_LAUNCH();
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
        oz::k_xstack<0><<<1, 1024, 0, st>>>(n, ng, x + ldx * (size_t)g0, ldx, w.colexp, w.fexp, w.XS);
        RNPGPU_CHECK_LAUNCH();
        oz::Args a{};
        a.mode = oz::kResidual;
        a.m = m;
        a.n = n;
        a.nrhs = ng;
        a.Ad = w.Ad;
        a.ldd = (size_t)m;
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
    const unsigned sgrid = (unsigned)std::min((m + 15) / 16, 2 * std::max(1, device_facts().sm_count));
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
        a.ldd = (size_t)m;
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
        const dim3 gs((unsigned)std::min((n + 255) / 256, 2048), (unsigned)ng);
        k_sum_partials<double><<<gs, 256, 0, st>>>(w.P, (size_t)n, (size_t)n * oz::kRhs, nr, n, ng, g + ldg * (size_t)g0, ldg);
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
