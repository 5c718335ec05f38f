// rnp_common.cuh — scalar types, reductions and the bounded grid barrier
// shared by every QR kernel of the GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace rnpgpu {

// ---------------------------------------------------------------------------
// Complex scalar, layout-compatible with std::complex<R> (re, im).
// ---------------------------------------------------------------------------
template <class R> struct alignas(2 * sizeof(R)) cplx {
    R x, y;
    cplx() = default;
    __host__ __device__ cplx(R a) : x(a), y(R(0)) {}
    __host__ __device__ cplx(R a, R b) : x(a), y(b) {}
};
template <class R> __host__ __device__ inline cplx<R> operator+(cplx<R> a, cplx<R> b) { return cplx<R>(a.x + b.x, a.y + b.y); }
template <class R> __host__ __device__ inline cplx<R> operator-(cplx<R> a, cplx<R> b) { return cplx<R>(a.x - b.x, a.y - b.y); }
template <class R> __host__ __device__ inline cplx<R> operator-(cplx<R> a) { return cplx<R>(-a.x, -a.y); }
template <class R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, cplx<R> b) { return cplx<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <class R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, R b) { return cplx<R>(a.x * b, a.y * b); }
template <class R> __host__ __device__ inline cplx<R> operator*(R b, cplx<R> a) { return cplx<R>(a.x * b, a.y * b); }
template <class R> __host__ __device__ inline cplx<R> operator/(cplx<R> a, R b) { return cplx<R>(a.x / b, a.y / b); }
// a/b by Smith's algorithm (Smith, CACM 5(8), 1962)
template <class R> __host__ __device__ inline cplx<R> operator/(cplx<R> a, cplx<R> b) {
    if ((b.y < 0 ? -b.y : b.y) <= (b.x < 0 ? -b.x : b.x)) {
        R r = b.y / b.x, d = b.x + b.y * r;
        return cplx<R>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    R r = b.x / b.y, d = b.y + b.x * r;
    return cplx<R>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
template <class R> __host__ __device__ inline bool operator==(cplx<R> a, cplx<R> b) { return a.x == b.x && a.y == b.y; }
template <class R> __host__ __device__ inline bool operator!=(cplx<R> a, cplx<R> b) { return !(a == b); }

typedef cplx<float> cf32;
typedef cplx<double> cf64;

// ---------------------------------------------------------------------------
// Scalar traits.  AccR is the real type used for Householder norms and
// beta/tau: FP64 for every scalar type (the FP32 forms keep the norm and the
// beta scaling in FP64).
// ---------------------------------------------------------------------------
template <class T> struct Tr;
template <> struct Tr<double> {
    typedef double R;
    static constexpr bool is_complex = false;
    __host__ __device__ static double conj(double v) { return v; }
    __host__ __device__ static double re(double v) { return v; }
    __host__ __device__ static double im(double) { return 0.0; }
    __host__ __device__ static double make(double a, double) { return a; }
};
template <> struct Tr<float> {
    typedef float R;
    static constexpr bool is_complex = false;
    __host__ __device__ static float conj(float v) { return v; }
    __host__ __device__ static float re(float v) { return v; }
    __host__ __device__ static float im(float) { return 0.0f; }
    __host__ __device__ static float make(float a, float) { return a; }
};
template <class Rr> struct Tr<cplx<Rr> > {
    typedef Rr R;
    static constexpr bool is_complex = true;
    __host__ __device__ static cplx<Rr> conj(cplx<Rr> v) { return cplx<Rr>(v.x, -v.y); }
    __host__ __device__ static Rr re(cplx<Rr> v) { return v.x; }
    __host__ __device__ static Rr im(cplx<Rr> v) { return v.y; }
    __host__ __device__ static cplx<Rr> make(Rr a, Rr b) { return cplx<Rr>(a, b); }
};

// fused multiply-add c + a*b for every scalar type
__device__ __forceinline__ double fmac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmac(float a, float b, float c) { return fmaf(a, b, c); }
template <class R> __device__ __forceinline__ cplx<R> fmac(cplx<R> a, cplx<R> b, cplx<R> c) {
    return cplx<R>(fmac(-a.y, b.y, fmac(a.x, b.x, c.x)), fmac(a.y, b.x, fmac(a.x, b.y, c.y)));
}

// ---------------------------------------------------------------------------
// Warp / block sums
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double shfl_xor_t(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float shfl_xor_t(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
template <class R> __device__ __forceinline__ cplx<R> shfl_xor_t(cplx<R> v, int o) { return cplx<R>(shfl_xor_t(v.x, o), shfl_xor_t(v.y, o)); }
// A warp's 16 sums at once: a butterfly that halves the entries at each of
// four steps, then adds lane pairs; each even lane ends with the total of
// one entry, whose index it returns (v[0] holds it).
template <class T> __device__ __forceinline__ int warp_reduce16(T (&v)[16], int lane) {
#pragma unroll
    for (int lvl = 0; lvl < 4; ++lvl) {
        const int o = 16 >> lvl, n = 8 >> lvl;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const T send = up ? v[i] : v[i + n], keep = up ? v[i + n] : v[i];
            v[i] = keep + shfl_xor_t(send, o);
        }
    }
    v[0] = v[0] + shfl_xor_t(v[0], 1);
    return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}
template <class R> __device__ __forceinline__ cplx<R> warp_sum(cplx<R> v) {
    return cplx<R>(warp_sum(v.x), warp_sum(v.y));
}
__device__ __forceinline__ double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
template <class R> __device__ __forceinline__ cplx<R> shfl(cplx<R> v, int src) { return cplx<R>(shfl(v.x, src), shfl(v.y, src)); }
__device__ __forceinline__ double abs2(double v) { return v * v; }
__device__ __forceinline__ double abs2(float v) { return (double)v * (double)v; }
template <class R> __device__ __forceinline__ double abs2(cplx<R> v) { return (double)v.x * (double)v.x + (double)v.y * (double)v.y; }

// ---------------------------------------------------------------------------
// Safe 2-norm accumulation without divisions (three accumulators for tiny,
// medium and huge magnitudes, after Blue 1978 and Anderson, ACM TOMS
// Algorithm 978, 2017).  The thresholds and scale factors follow from the
// IEEE double format (minexponent -1021, maxexponent 1024, 53 digits):
//   tsml = 2^ceil((-1021-1)/2)       = 2^-511
//   tbig = 2^floor((1024-53+1)/2)    = 2^486
//   ssml = 2^-floor((-1021-53)/2)    = 2^537
//   sbig = 2^-ceil((1024+53-1)/2)    = 2^-538
// Squares of FP32 values never leave the double range, so FP32 inputs use
// the medium accumulator only.
// ---------------------------------------------------------------------------
struct NormAcc {
    double sml, med, big;
    __device__ __forceinline__ void zero() { sml = 0.0; med = 0.0; big = 0.0; }
    __device__ __forceinline__ void add(double v) {
        // 2^-511 <= |v| < 2^486 (the medium range, all but extreme data),
        // told from the exponent bits on the integer pipe: one FP64
        // instruction for the common case, the same accumulator as below
        const int e = (__double2hiint(v) >> 20) & 0x7ff;
        if (e >= 1023 - 511 && e < 1023 + 486) {
            med = fma(v, v, med);
            return;
        }
        const double tsml = 0x1p-511, tbig = 0x1p486, ssml = 0x1p537, sbig = 0x1p-538;
        double a = fabs(v);
        if (a > tbig) {
            double s = a * sbig;
            big = fma(s, s, big);
        } else if (a < tsml) {
            double s = a * ssml;
            sml = fma(s, s, sml);
        } else {
            med = fma(a, a, med);
        }
    }
    __device__ __forceinline__ void add(float v) {
        double a = (double)v;
        med = fma(a, a, med);
    }
    template <class R> __device__ __forceinline__ void add(cplx<R> v) { add(v.x); add(v.y); }
    __device__ __forceinline__ void merge(const NormAcc &o) { sml += o.sml; med += o.med; big += o.big; }
    // the extreme-range accumulators only when some lane holds one
    __device__ __forceinline__ void warp_reduce() {
        if (__any_sync(0xffffffffu, sml != 0.0 || big != 0.0)) {
            sml = warp_sum(sml);
            big = warp_sum(big);
        }
        med = warp_sum(med);
    }
    __device__ double result() const { return result_scaled(1.0); }
    // mult * ||x|| for a power-of-two mult, without rounding through the
    // subnormal range when ||x|| itself is subnormal
    __device__ double result_scaled(double mult) const {
        const double ssml = 0x1p537, sbig = 0x1p-538;
        double scl, sumsq;
        if (big > 0.0) {
            double b = big;
            if (med > 0.0 || med != med) b += (med * sbig) * sbig;
            scl = 1.0 / sbig;
            sumsq = b;
        } else if (sml > 0.0) {
            if (med > 0.0 || med != med) {
                double ymed = sqrt(med), ysml = sqrt(sml) / ssml;
                double ymin = ymed < ysml ? ymed : ysml, ymax = ymed < ysml ? ysml : ymed;
                double q = ymin / ymax;
                scl = 1.0;
                sumsq = ymax * ymax * (1.0 + q * q);
            } else {
                scl = 1.0 / ssml;
                sumsq = sml;
            }
        } else {
            scl = 1.0;
            sumsq = med;
        }
        return (scl * mult) * sqrt(sumsq);
    }
};

// sqrt(x^2+y^2+z^2) without unnecessary overflow (RNP/Types.hpp:73-92)
// The components are scaled by the power of two nearest below max|.| (exact)
// instead of divided by the max: the same overflow protection without
// divisions, which are long instruction sequences on the FP64 pipe.
__device__ __forceinline__ double hypot3(double x, double y, double z) {
    double xa = fabs(x), ya = fabs(y), za = fabs(z);
    double w = fmax(fmax(xa, ya), za);
    if (xa != xa || ya != ya || za != za) return xa + ya + za;
    if (w == 0.0) return xa + ya + za;
    if (w < 0x1p-1000 || w > 0x1p1000) {
        // extreme magnitudes (2^-e would leave the double range): divide
        xa /= w; ya /= w; za /= w;
        return w * sqrt(xa * xa + ya * ya + za * za);
    }
    int e;
    frexp(w, &e);
    const double sc = ldexp(1.0, -e);
    xa *= sc; ya *= sc; za *= sc;
    return ldexp(sqrt(xa * xa + ya * ya + za * za), e);
}

// Error-free FP32 accumulation (TwoProduct by FMA, TwoSum): (hi, lo) carries a
// sum to about 2^-48 relative, on the FP32 pipe.
__device__ __forceinline__ void df_add(float &hi, float &lo, float x) {
    const float s = hi + x, bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}
__device__ __forceinline__ void df_add_prod(float &hi, float &lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    df_add(hi, lo, p);
    lo += e;
}
// FP32 hi + lo pairs (double-float arithmetic after Dekker, "A floating-point
// technique for extending the available precision", 1971): about 2^-44
// relative, on the FP32 pipe
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 f2_norm(float h, float l) {
    const float s = h + l;
    return F2{s, l - (s - h)};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const float s = a.h + b.h, bp = s - a.h;
    const float e = ((a.h - (s - bp)) + (b.h - bp)) + (a.l + b.l);
    return f2_norm(s, e);
}
__device__ __forceinline__ F2 f2_neg(F2 a) { return F2{-a.h, -a.l}; }
__device__ __forceinline__ F2 f2_mul(F2 a, float c) {
    const float p = a.h * c;
    return f2_norm(p, fmaf(a.l, c, fmaf(a.h, c, -p)));
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = a.h * b.h;
    return f2_norm(p, fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p))));
}
__device__ __forceinline__ F2 f2_sq(float a) {
    const float p = a * a;
    return F2{p, fmaf(a, a, -p)};
}

__device__ __forceinline__ void df_warp_sum(float &hi, float &lo) {
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
        df_add(hi, lo, oh);
        lo += ol;
    }
}

// Asynchronous global -> shared copies (cp.async, 4/8/16 bytes, cached in
// L1); both addresses aligned to the copy size.
template <int BYTES> __device__ __forceinline__ void cp_async(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)), "l"(gsrc), "n"(BYTES) : "memory");
}
// 16 bytes, not cached in L1 (streamed operands)
__device__ __forceinline__ void cp_async_cg16(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// 1/(a+ib) by Smith's algorithm (Smith, CACM 5(8), 1962)
__device__ __forceinline__ void crecip(double a, double b, double &rx, double &ry) {
    if (fabs(b) <= fabs(a)) {
        double r = b / a, d = a + b * r;
        rx = 1.0 / d;
        ry = -r / d;
    } else {
        double r = a / b, d = b + a * r;
        rx = r / d;
        ry = -1.0 / d;
    }
}

// ---------------------------------------------------------------------------
// Bounded grid barrier for cooperative launches.  The counter is zeroed by
// the host before the launch; every barrier generation adds one arrival per
// block.  A wait that exceeds kSpinLimit cycles (about 2 s at 2 GHz) sets the
// launch's error word and the kernel returns instead of hanging; a block that
// sees the error word set stops waiting too.
// ---------------------------------------------------------------------------
static constexpr long long kSpinLimit = 4000000000LL;

enum DeviceStatus : int { kStatusOk = 0, kStatusBarrierTimeout = 1 };

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile(const int *p) {
    int v;
    asm volatile("ld.volatile.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct GridBarrier {
    unsigned *counter;
    int *err;
    unsigned nblocks;
    unsigned gen;
    long long spin_limit = kSpinLimit;
    int *status = nullptr;  // library-wide status word, also set on a timeout
    // arrive + wait; returns false when this launch must stop (timeout or an
    // error elsewhere)
    __device__ bool sync() {
        arrive();
        return wait();
    }
    // split form: work between arrive() and wait() overlaps the barrier;
    // it must not touch what other blocks read after the barrier.  The
    // block's writes are ordered before thread 0's release by the block
    // barrier, and the release/acquire pair carries them to the waiting
    // blocks (no separate fence).
    __device__ void arrive() {
        __syncthreads();
        if (nblocks > 1 && threadIdx.x == 0) {
            ++gen;
            red_release_add(counter, 1u);
        }
    }
    __device__ bool wait() {
        __shared__ int s_ok;
        if (nblocks > 1) {
            if (threadIdx.x == 0) {
                const unsigned target = gen * nblocks;
                int ok = 1;
                const long long t0 = clock64();
                for (unsigned it = 1; ld_acquire(counter) < target; ++it) {
                    if ((it & 63u) == 0) {  // the error word and the time limit, now and then
                        if (ld_volatile(err) != 0) { ok = 0; break; }
                        if (clock64() - t0 > spin_limit) {
                            atomicExch(err, (int)kStatusBarrierTimeout);
                            if (status) atomicExch(status, (int)kStatusBarrierTimeout);
                            ok = 0;
                            break;
                        }
                    }
                }
                s_ok = ok;
            }
            __syncthreads();
            return s_ok != 0;
        }
        __syncthreads();
        return true;
    }
};

} // namespace rnpgpu
