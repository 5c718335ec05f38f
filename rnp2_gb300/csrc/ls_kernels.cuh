// ls_kernels.cuh — kernels of the least-squares layer built on the QR path:
// upper-triangular solve (the reference's BLAS::SolveTrM "L","U","N","N",
// RNP/BLAS/BLAS_mix.hpp:2096-2113 -> dtrsm_), precision conversion, column
// norms and the FP64 accumulation of refinement corrections.
#pragma once
#include "qr_kernels.cuh"

namespace rnpgpu {

// X = R^{-1} Y in place (Y is n x nrhs with leading dimension ldb), R upper
// triangular non-unit (leading dimension ldr).  One block per right-hand
// side; each 32 x 32 diagonal block is staged in shared memory and solved by
// one warp with shuffles, the rows above are updated by the whole block.
template <class T> __global__ void __launch_bounds__(512) k_trsm_upper(int n, int nrhs, const T *R, size_t ldr, T *B, size_t ldb) {
    __shared__ T xs[32];
    __shared__ T sR[32][33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int col = blockIdx.x; col < nrhs; col += gridDim.x) {
        T *y = B + (size_t)col * ldb;
        for (int i1 = n; i1 > 0; i1 -= 32) {
            const int i0 = max(0, i1 - 32), nbk = i1 - i0;
            for (int idx = tid; idx < nbk * nbk; idx += blockDim.x) {
                const int r = idx % nbk, c = idx / nbk;
                sR[r][c] = (r <= c) ? R[(i0 + r) + (size_t)(i0 + c) * ldr] : T(0);
            }
            __syncthreads();
            if (warp == 0) {
                T yv = (lane < nbk) ? y[i0 + lane] : T(0);
                for (int i = nbk - 1; i >= 0; --i) {
                    if (lane == i) yv = yv / sR[i][i];
                    const T xi = shfl(yv, i);
                    if (lane < i) yv = yv - sR[lane][i] * xi;
                }
                if (lane < nbk) {
                    y[i0 + lane] = yv;
                    xs[lane] = yv;
                }
            }
            __syncthreads();
            // rows above: 32 independent loads in flight per thread
            for (int r = tid; r < i0; r += blockDim.x) {
                T a[4] = {T(0), T(0), T(0), T(0)};
                if (nbk == 32 && sizeof(T) <= 8) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) a[c & 3] = fmac(R[r + (size_t)(i0 + c) * ldr], xs[c], a[c & 3]);
                } else {
                    for (int c = 0; c < nbk; ++c) a[0] = fmac(R[r + (size_t)(i0 + c) * ldr], xs[c], a[0]);
                }
                y[r] = y[r] - ((a[0] + a[1]) + (a[2] + a[3]));
            }
            __syncthreads();
        }
    }
}

// Y = R^{-H} G in place: forward substitution with the conjugate transpose of
// an upper triangular R (the lower triangular system R^H y = g).
template <class T> __global__ void __launch_bounds__(512) k_trsm_upper_ct(int n, int nrhs, const T *R, size_t ldr, T *B, size_t ldb) {
    __shared__ T xs[32];
    __shared__ T sR[32][33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int col = blockIdx.x; col < nrhs; col += gridDim.x) {
        T *y = B + (size_t)col * ldb;
        for (int i0 = 0; i0 < n; i0 += 32) {
            const int nbk = min(32, n - i0), i1 = i0 + nbk;
            for (int idx = tid; idx < nbk * nbk; idx += blockDim.x) {
                const int r = idx % nbk, c = idx / nbk;
                sR[r][c] = (r <= c) ? R[(i0 + r) + (size_t)(i0 + c) * ldr] : T(0);
            }
            __syncthreads();
            if (warp == 0) {
                T yv = (lane < nbk) ? y[i0 + lane] : T(0);
                for (int i = 0; i < nbk; ++i) {
                    if (lane == i) yv = yv / Tr<T>::conj(sR[i][i]);
                    const T xi = shfl(yv, i);
                    if (lane > i && lane < nbk) yv = yv - Tr<T>::conj(sR[i][lane]) * xi;
                }
                if (lane < nbk) {
                    y[i0 + lane] = yv;
                    xs[lane] = yv;
                }
            }
            __syncthreads();
            for (int r = i1 + tid; r < n; r += blockDim.x) {
                const T *rc = R + (size_t)r * ldr + i0;
                T a[4] = {T(0), T(0), T(0), T(0)};
                if (nbk == 32 && sizeof(T) <= 8) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) a[c & 3] = fmac(Tr<T>::conj(rc[c]), xs[c], a[c & 3]);
                } else {
                    for (int c = 0; c < nbk; ++c) a[0] = fmac(Tr<T>::conj(rc[c]), xs[c], a[0]);
                }
                y[r] = y[r] - ((a[0] + a[1]) + (a[2] + a[3]));
            }
            __syncthreads();
        }
    }
}

// The same solves for n <= 512 and elements of at most 8 bytes, with the
// latencies hidden: R y = b by back substitution (CT = false) or R^H y = b by
// forward substitution (CT = true), one block per right-hand side, 32 rows a
// step.  The right-hand side stays in shared memory; the next diagonal block
// is loaded by warps 1..15 while warp 0 solves the current one (two buffers),
// the reciprocals of the diagonal are formed by all lanes at once, and every
// thread loads the 32 coefficients of its row's update before the barrier
// that waits for the block solve.  With Dinv (the inverses of R's 32 x 32
// diagonal blocks, k_trinv_diag) the block solve is one product by the
// block's inverse (32 independent sums instead of a 32-step chain).
constexpr int kTrsmSmallMax = 512;
template <class T, bool CT> __global__ void __launch_bounds__(512) k_trsm_small(int n, int nrhs, const T *R, size_t ldr, T *B, size_t ldb, const T *Dinv) {
    __shared__ T sy[kTrsmSmallMax];
    __shared__ T sD[2][32][33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nblk = (n + 31) / 32;
    auto first_row = [&](int s) { return 32 * (CT ? s : nblk - 1 - s); };
    auto load_diag = [&](int s, int buf, int t0, int nt) {
        const int i0 = first_row(s), nbk = min(32, n - i0);
        const T *D = Dinv ? Dinv + (size_t)(i0 / 32) * 1024 : nullptr;
        for (int idx = t0; idx < 32 * 32; idx += nt) {
            const int r = idx & 31, c = idx >> 5;
            sD[buf][r][c] = (r < nbk && c < nbk && r <= c) ? (D ? D[r + 32 * c] : R[(i0 + r) + (size_t)(i0 + c) * ldr]) : T(0);
        }
    };
    for (int col = blockIdx.x; col < nrhs; col += gridDim.x) {
        T *y = B + (size_t)col * ldb;
        // the unrolled updates read whole 32-entry blocks of sy: the entries
        // past n are zeros (0 * stale shared memory could be NaN)
        for (int i = tid; i < 32 * nblk; i += blockDim.x) sy[i] = (i < n) ? y[i] : T(0);
        load_diag(0, 0, tid, blockDim.x);
        __syncthreads();
        // this thread's 32 update coefficients of step s (row r = tid)
        auto load_coef = [&](int s, T (&cf)[32]) {
            const int i0 = first_row(s), nbk = min(32, n - i0), r = tid;
            const bool upd = CT ? (r >= i0 + nbk && r < n) : (r < i0);
            if (upd) {
#pragma unroll
                for (int c = 0; c < 32; ++c) cf[c] = (c < nbk) ? (CT ? Tr<T>::conj(R[(i0 + c) + (size_t)r * ldr]) : R[r + (size_t)(i0 + c) * ldr]) : T(0);
            }
        };
        // 4-byte elements: the next step's coefficients are loaded during
        // this step (their latency was most of a step)
        constexpr bool kPref = sizeof(T) == 4;
        T coef[32];
        if (kPref) load_coef(0, coef);
        for (int s = 0; s < nblk; ++s) {
            const int i0 = first_row(s), nbk = min(32, n - i0), buf = s & 1;
            const int r = tid;
            const bool upd = CT ? (r >= i0 + nbk && r < n) : (r < i0);
            T coefn[kPref ? 32 : 1];
            if constexpr (kPref) {
                if (s + 1 < nblk) load_coef(s + 1, coefn);
            } else {
                load_coef(s, coef);
            }
            if (warp == 0 && Dinv) {
                // y_B <- D_B^-1 y_B (CT: D_B^-H y_B), entries past n zero
                T acc = T(0);
#pragma unroll 8
                for (int c = 0; c < 32; ++c) acc = fmac(CT ? Tr<T>::conj(sD[buf][c][lane]) : sD[buf][lane][c], sy[i0 + c], acc);
                __syncwarp();
                if (lane < nbk) sy[i0 + lane] = acc;
            } else if (warp == 0) {
                T yv = (lane < nbk) ? sy[i0 + lane] : T(0);
                const T d = (lane < nbk) ? (CT ? Tr<T>::conj(sD[buf][lane][lane]) : sD[buf][lane][lane]) : T(1);
                const T dinv = T(1) / d;
                if (!CT) {
                    for (int i = nbk - 1; i >= 0; --i) {
                        if (lane == i) yv = yv * dinv;
                        const T xi = shfl(yv, i);
                        if (lane < i) yv = yv - sD[buf][lane][i] * xi;
                    }
                } else {
                    for (int i = 0; i < nbk; ++i) {
                        if (lane == i) yv = yv * dinv;
                        const T xi = shfl(yv, i);
                        if (lane > i && lane < nbk) yv = yv - Tr<T>::conj(sD[buf][i][lane]) * xi;
                    }
                }
                if (lane < nbk) sy[i0 + lane] = yv;
            } else if (s + 1 < nblk) {
                load_diag(s + 1, buf ^ 1, tid - 32, blockDim.x - 32);
            }
            __syncthreads();
            if (upd) {
                T a[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int c = 0; c < 32; ++c) a[c & 3] = fmac(coef[c], sy[i0 + c], a[c & 3]);
                sy[r] = sy[r] - ((a[0] + a[1]) + (a[2] + a[3]));
            }
            if constexpr (kPref) {
#pragma unroll
                for (int c = 0; c < 32; ++c) coef[c] = coefn[c];
            }
            __syncthreads();
        }
        for (int i = tid; i < n; i += blockDim.x) y[i] = sy[i];
        __syncthreads();
    }
}

// Dinv: the inverse of every 32 x 32 diagonal block of the upper triangular
// R (n x n), block b at Dinv + b * 1024 (column-major, zero below the
// diagonal and past n).  One warp per block; lane j forms column j of the
// inverse by back substitution.
template <class T> __global__ void __launch_bounds__(32) k_trinv_diag(int n, const T *R, size_t ldr, T *Dinv) {
    __shared__ T sU[32][33], sX[32][33];
    const int b = blockIdx.x, j = threadIdx.x, i0 = 32 * b, nb = min(32, n - i0);
    for (int r = 0; r < 32; ++r) sU[r][j] = (r < nb && j < nb && r <= j) ? R[(i0 + r) + (size_t)(i0 + j) * ldr] : T(0);
    __syncwarp();
    for (int i = 31; i >= 0; --i) {
        T x = T(0);
        if (j < nb && i <= j) {
            T acc = (i == j) ? T(1) : T(0);
            for (int k = i + 1; k <= j; ++k) acc = fmac(-sU[i][k], sX[k][j], acc);
            x = acc / sU[i][i];
        }
        sX[i][j] = x;
        __syncwarp();
    }
    for (int r = 0; r < 32; ++r) Dinv[(size_t)b * 1024 + r + 32 * j] = sX[r][j];
}

template <class Tin, class Tout> __device__ __forceinline__ Tout convert_scalar(Tin v);
template <> __device__ __forceinline__ float convert_scalar<double, float>(double v) { return (float)v; }
template <> __device__ __forceinline__ double convert_scalar<float, double>(float v) { return (double)v; }
template <> __device__ __forceinline__ double convert_scalar<double, double>(double v) { return v; }
template <> __device__ __forceinline__ float convert_scalar<float, float>(float v) { return v; }
template <> __device__ __forceinline__ cf32 convert_scalar<cf64, cf32>(cf64 v) { return cf32((float)v.x, (float)v.y); }
template <> __device__ __forceinline__ cf64 convert_scalar<cf32, cf64>(cf32 v) { return cf64((double)v.x, (double)v.y); }
template <> __device__ __forceinline__ cf64 convert_scalar<cf64, cf64>(cf64 v) { return v; }
template <> __device__ __forceinline__ cf32 convert_scalar<cf32, cf32>(cf32 v) { return v; }

// B(0:m, 0:n) = (Tout) A(0:m, 0:n)
template <class Tin, class Tout> __global__ void __launch_bounds__(256) k_convert(int m, int n, const Tin *A, size_t lda, Tout *B, size_t ldb) {
    for (int c = blockIdx.y; c < n; c += gridDim.y)
        for (int r = blockIdx.x * 256 + threadIdx.x; r < m; r += gridDim.x * 256)
            B[r + (size_t)c * ldb] = convert_scalar<Tin, Tout>(A[r + (size_t)c * lda]);
}

// X(0:n, j) += (Th) D(0:n, j)
template <class Tl, class Th> __global__ void __launch_bounds__(256) k_add_correction(int n, int nrhs, const Tl *D, size_t ldd, Th *X, size_t ldx) {
    for (int c = blockIdx.y; c < nrhs; c += gridDim.y)
        for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256)
            X[r + (size_t)c * ldx] = X[r + (size_t)c * ldx] + convert_scalar<Tl, Th>(D[r + (size_t)c * ldd]);
}

// out[j] = ||A(0:m, j)||_2^2 accumulated in FP64 (error metrics only)
template <class T> __global__ void __launch_bounds__(256) k_col_sumsq(int m, int n, const T *A, size_t lda, double *out) {
    __shared__ double s[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        double acc = 0.0;
        for (int r = tid; r < m; r += 256) acc += abs2(A[r + (size_t)c * lda]);
        acc = warp_sum(acc);
        if (lane == 0) s[warp] = acc;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < 8; ++w) t += s[w];
            out[c] = t;
        }
        __syncthreads();
    }
}

// out(0:rows, 0:cols) = sum over q < nsplit of P_q  (P_q = P + q*pstride)
template <class T> __global__ void __launch_bounds__(256) k_sum_partials(const T *P, size_t ldp, size_t pstride, int nsplit, int rows, int cols, T *out, size_t ldo) {
    for (int c = blockIdx.y; c < cols; c += gridDim.y)
        for (int r = blockIdx.x * 256 + threadIdx.x; r < rows; r += gridDim.x * 256) {
            T a[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = T(0);
            int q = 0;
            for (; q + 8 <= nsplit; q += 8) {
#pragma unroll
                for (int u = 0; u < 8; ++u) a[u] = a[u] + P[(size_t)(q + u) * pstride + r + (size_t)c * ldp];
            }
            for (int u = 0; q < nsplit; ++q, ++u) a[u] = a[u] + P[(size_t)q * pstride + r + (size_t)c * ldp];
            out[r + (size_t)c * ldo] = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
        }
}

} // namespace rnpgpu
