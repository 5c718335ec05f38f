// matgen.cuh — RNP::MatrixGen::RandomMatrix (RNP/MatrixGen.hpp:120-272) and
// GenerateDiagonal (:31-109) on the GPU, for real types (the reference's
// RandomMatrix compiles for real types only).
//
// The reference sets A = diag(d) and then, for i = min(m,n)-1 down to 0,
// applies a Householder reflector drawn from a Normal01 vector from the left
// to rows i.. and another from the right to columns i.. (symmetric cases:
// one reflector from both sides).  A reflector at step i only touches rows
// and columns >= i, where A is still zero outside the block that earlier
// steps filled, so
//     nonsymmetric:  A = (H_0 H_1 ... H_{k-1}) D (G_{k-1} ... G_0)
//     symmetric:     A = (H_0 ... H_{n-1}) D (H_{n-1} ... H_0)
// i.e. Q D Q_R^H for the QR-style reflector products Q = H_0 ... H_{k-1}:
// here every random vector is drawn at once (each from its own position in
// the generator's stream), its reflector formed by one block per vector and
// stored as a QR reflector column, and D is multiplied by the two blocked
// MultQ calls of the QR path.
//
// The generator is the reference's 48-bit multiplicative congruential one
// (RNP/Random.hpp:45-183, multiplier 33952834046453, modulus 2^48): the t-th
// uniform after a seed s is s * a^(t+1) mod 2^48, computed directly with
// 64-bit integer products (2^48 divides 2^64), so every uniform is
// bit-identical to the reference's; Normal01 = sqrt(-2 log1p(-u1)) cos(2 pi
// u2) (RNP/Random.hpp:190-193) is evaluated in double.
#pragma once
#include "qr_driver.cuh"

namespace rnpgpu {
namespace mg {

constexpr uint64_t kA = 33952834046453ULL;
constexpr uint64_t kMask = (1ULL << 48) - 1;

__host__ __device__ inline uint64_t powmod(uint64_t e) {
    // a^e mod 2^48
    uint64_t r = 1, b = kA;
    while (e) {
        if (e & 1) r = (r * b) & kMask;
        b = (b * b) & kMask;
        e >>= 1;
    }
    return r;
}
// the t-th uniform (0-based) after the state s
template <class R> __device__ inline R uniform_at(uint64_t s, uint64_t t) {
    const uint64_t x = (s * powmod(t + 1)) & kMask;
    const R it1 = (R)(double)((x >> 36) & 4095), it2 = (R)(double)((x >> 24) & 4095), it3 = (R)(double)((x >> 12) & 4095), it4 = (R)(double)(x & 4095);
    const R q = R(1) / R(4096);
    const R v = (it1 + (it2 + (it3 + it4 * q) * q) * q) * q;
    return R(1) - v;
}
template <class R> __device__ inline R normal_at(uint64_t s, uint64_t t) {
    const R u1 = uniform_at<R>(s, t), u2 = uniform_at<R>(s, t + 1);
    const R ang = (R)6.28318530717958647692528676656 * u2;  // in R, as the reference
    return (R)(sqrt(-2.0 * log1p(-(double)u1)) * cos((double)ang));
}

inline uint64_t seed_state(const int *iseed) {
    return ((uint64_t)(iseed[0] & 4095) << 36) | ((uint64_t)(iseed[1] & 4095) << 24) | ((uint64_t)(iseed[2] & 4095) << 12) | (uint64_t)((iseed[3] | 1) & 4095);
}
inline void state_seed(uint64_t s, int *iseed) {
    iseed[0] = (int)((s >> 36) & 4095);
    iseed[1] = (int)((s >> 24) & 4095);
    iseed[2] = (int)((s >> 12) & 4095);
    iseed[3] = (int)(s & 4095);
}
// uniforms consumed by GenerateVector(dist, n) (RNP/Random.hpp:262-320)
__host__ __device__ inline uint64_t draws(int dist, uint64_t n) {
    if (dist == 2) return 2 * n;
    if (dist == 3 || dist == 4) return 128 * ((n + 63) / 64);
    return n;
}

// GenerateDiagonal (RNP/MatrixGen.hpp:31-109) in one block: modes 1-6 (mode
// 0 copies d_in), the reference's "reverse" loop (it swaps every pair twice,
// leaving d as it was), random signs for the Hermitian case, the scaling to
// a largest magnitude dscale; writes dw and, when given, d_out.
template <class R> __global__ void __launch_bounds__(256) k_mg_diag(int dist, int mode, int randsign, R cond, R dscale, int n, const R *d_in, R *dw, R *d_out, uint64_t s) {
    __shared__ R s_max[256];
    const int tid = threadIdx.x;
    const R rcond = R(1) / cond;
    const uint64_t sign0 = mode == 5 ? (uint64_t)n : mode == 6 ? draws(dist, (uint64_t)n) : 0;
    R mx = R(0);
    for (int i = tid; i < n; i += 256) {
        R v;
        switch (mode) {
        case 1: v = i == 0 ? R(1) : rcond; break;
        case 2: v = i + 1 < n ? R(1) : rcond; break;
        case 3: v = pow(rcond, R(i) / R(n - 1)); break;
        case 4: {
            const R t = R(i) / R(n - 1);
            v = (R(1) - t) + t * rcond;
            break;
        }
        case 5: v = pow(rcond, uniform_at<R>(s, (uint64_t)i)); break;
        case 6:
            if (dist == 0) v = uniform_at<R>(s, (uint64_t)i);
            else if (dist == 1) v = R(2) * uniform_at<R>(s, (uint64_t)i) - R(1);
            else if (dist == 2) v = normal_at<R>(s, 2 * (uint64_t)i);
            else {
                const uint64_t t = 128 * (uint64_t)(i / 64) + 2 * (uint64_t)(i % 64);
                const R u = uniform_at<R>(s, t);
                v = dist == 3 ? R(2) * u - R(1) : ((R(2) * u < R(1)) ? R(-1) : R(1));
            }
            break;
        default: v = d_in[i]; break;
        }
        if (randsign && R(2) * uniform_at<R>(s, sign0 + (uint64_t)i) > R(1)) v = -v;
        dw[i] = v;
        mx = fmax(mx, fabs(v));
    }
    s_max[tid] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (tid < o) s_max[tid] = fmax(s_max[tid], s_max[tid + o]);
        __syncthreads();
    }
    const bool scale = mode != 0 && mode != 6;
    const R f = scale ? dscale / s_max[0] : R(1);
    for (int i = tid; i < n; i += 256) {
        const R v = scale ? dw[i] * f : dw[i];
        dw[i] = v;
        if (d_out) d_out[i] = v;
    }
}

// One block per reflector (RNP/MatrixGen.hpp:164-181, 196-208, 228-238):
// vector j (step i = pos[j]) of length len = rows - i, drawn from stream
// position off[j]; u = w / (w0 + wa) with u0 = 1 stored in column i of V
// from row i (unit diagonal implicit, zeros above), tau = (w0 + wa) / wa,
// wa = ||w|| w0 / |w0|.
struct MgVec {
    int i, len;
    uint64_t off;
    int side;  // 0: left (V_L), 1: right (V_R)
};
template <class R> __global__ void __launch_bounds__(256) k_mg_reflect(const MgVec *vecs, uint64_t s, R *VL, size_t ldl, R *tauL, R *VR, size_t ldr, R *tauR) {
    __shared__ double s_red[256];
    __shared__ R s_w0, s_scale;
    const MgVec v = vecs[blockIdx.x];
    const int tid = threadIdx.x;
    R *V = v.side ? VR : VL;
    const size_t ld = v.side ? ldr : ldl;
    R *col = V + (size_t)v.i * ld;
    // draw into the column (rows i .. i+len-1), zero the rows above
    for (int r = tid; r < v.i; r += 256) col[r] = R(0);
    double mx = 0.0;
    for (int j = tid; j < v.len; j += 256) {
        const R x = normal_at<R>(s, v.off + 2 * (uint64_t)j);
        col[v.i + j] = x;
        mx = fmax(mx, fabs((double)x));
    }
    s_red[tid] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (tid < o) s_red[tid] = fmax(s_red[tid], s_red[tid + o]);
        __syncthreads();
    }
    const double big = s_red[0];
    __syncthreads();
    // scaled sum of squares (the reference's Norm2, RNP/BLAS/BLAS_mix.hpp:725-760)
    double ss = 0.0;
    if (big > 0.0)
        for (int j = tid; j < v.len; j += 256) {
            const double q = (double)col[v.i + j] / big;
            ss += q * q;
        }
    s_red[tid] = ss;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (tid < o) s_red[tid] += s_red[tid + o];
        __syncthreads();
    }
    if (tid == 0) {
        const R wn = (R)(big * sqrt(s_red[0]));
        const R w0 = col[v.i];
        const R wa = (wn / fabs(w0)) * w0;
        R tau = R(0), sc = R(1);
        if (wn != R(0)) {
            const R wb = w0 + wa;
            sc = R(1) / wb;
            tau = wb / wa;
        }
        (v.side ? tauR : tauL)[v.i] = tau;
        s_w0 = tau != R(0) ? R(1) : w0;
        s_scale = sc;
    }
    __syncthreads();
    const R sc = s_scale;
    for (int j = tid + 1; j < v.len; j += 256) col[v.i + j] *= sc;
    if (tid == 0) col[v.i] = s_w0;
}

// A = diag(d) (m x n)
template <class R> __global__ void k_mg_setdiag(int m, int n, const R *d, R *A, size_t lda) {
    for (int c = blockIdx.y; c < n; c += gridDim.y)
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) A[r + (size_t)c * lda] = (r == c) ? d[r] : R(0);
}
// upper triangle from the lower (RNP/MatrixGen.hpp:218-223)
template <class R> __global__ void k_mg_symmetrize(int n, R *A, size_t lda) {
    for (int c = blockIdx.y; c < n; c += gridDim.y)
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < c; r += gridDim.x * blockDim.x) A[r + (size_t)c * lda] = A[c + (size_t)r * lda];
}

} // namespace mg

// Workspace (elements of R): the diagonal, the left and right reflector
// matrices and their tau, the vector descriptors, and the MultQ workspace.
template <class R> size_t random_matrix_bytes(int sym, size_t m, size_t n) {
    const size_t k = std::min(m, n);
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t q1 = 0, q2 = 0;
    unmqr<R>("L", "N", m, n, k, nullptr, std::max<size_t>(m, 1), nullptr, nullptr, std::max<size_t>(m, 1), &q1, nullptr);
    unmqr<R>("R", "C", m, n, k, nullptr, std::max<size_t>(n, 1), nullptr, nullptr, std::max<size_t>(m, 1), &q2, nullptr);
    const size_t nvec = 2 * k;
    return al(k * sizeof(R)) + al(m * k * sizeof(R)) + al(k * sizeof(R)) + (sym == 0 ? al(n * k * sizeof(R)) + al(k * sizeof(R)) : 0) + al(nvec * sizeof(mg::MgVec)) +
           al(std::max(q1, q2) * sizeof(R)) + 256;
}

// RNP::MatrixGen::RandomMatrix: sym 0 Nonsymmetric, 1 Hermitian, 2 Hermitian
// positive definite, 3 Symmetric; dist and mode as RNP::Random::Distribution
// and MatrixGen::DiagonalMode; d (device) is read for mode 0 (Given) and
// written otherwise when given; iseed (host, 4 ints) is advanced past every
// number drawn, as the reference leaves it.
template <class R>
int random_matrix(int sym, int dist, int mode, int reverse, R cond, R dmax, R *d, size_t m, size_t n, R *a, size_t lda, int *iseed, size_t *lwork, R *work) {
    (void)reverse;  // the reference's reverse loop leaves d unchanged
    if (lwork == nullptr) return -13;
    if (sym < 0 || sym > 3) return -1;
    if (dist < 0 || dist > 4) return -2;
    if (mode < 0 || mode > 6) return -3;
    if (sym != 0 && m != n) return -8;
    const size_t k = std::min(m, n);
    if (k == 0) {
        if (work == nullptr || *lwork == 0) *lwork = 1;
        return kOk;
    }
    if (lda < std::max<size_t>(1, m)) return -11;
    if (m > (size_t)INT32_MAX / 2 || n > (size_t)INT32_MAX / 2) return -8;
    const size_t need = elems_for<R>(random_matrix_bytes<R>(sym, m, n));
    if (work == nullptr || *lwork == 0) {
        *lwork = need;
        return kOk;
    }
    if (mode == 0 && d == nullptr) return -7;
    if (a == nullptr) return -10;
    if (iseed == nullptr) return -12;
    if (*lwork < need) return -13;
    cudaStream_t st = current_stream();
    Carver cv(work);
    R *dw = cv.take<R>(k);
    R *VL = cv.take<R>(m * k);
    R *tauL = cv.take<R>(k);
    R *VR = sym == 0 ? cv.take<R>(n * k) : nullptr;
    R *tauR = sym == 0 ? cv.take<R>(k) : nullptr;
    mg::MgVec *vecs = cv.take<mg::MgVec>(2 * k);
    R *wrest = cv.take<R>(0);
    const size_t lwq = *lwork - (size_t)(wrest - work);

    // the generator's stream: the diagonal's draws, the signs, then the
    // reflectors in the reference's order (i descending; left before right)
    const uint64_t s0 = mg::seed_state(iseed);
    uint64_t t = 0;
    if (mode == 5) t += k;
    if (mode == 6) t += mg::draws(dist, k);
    if (sym == 1) t += k;
    std::vector<mg::MgVec> hv;
    hv.reserve(2 * k);
    const size_t nref = sym == 0 ? k : n;
    for (size_t ii = nref; ii-- > 0;) {
        if (sym == 0) {
            if (ii + 1 < m) {
                hv.push_back(mg::MgVec{(int)ii, (int)(m - ii), t, 0});
                t += 2 * (m - ii);
            }
            if (ii + 1 < n) {
                hv.push_back(mg::MgVec{(int)ii, (int)(n - ii), t, 1});
                t += 2 * (n - ii);
            }
        } else {
            hv.push_back(mg::MgVec{(int)ii, (int)(n - ii), t, 0});
            t += 2 * (n - ii);
        }
    }
    KScope ks("random_matrix", st);
    // left reflector columns not drawn (a vector of length 1) stay identity
    RNPGPU_CHECK(cudaMemsetAsync(tauL, 0, k * sizeof(R), st));
    if (tauR) RNPGPU_CHECK(cudaMemsetAsync(tauR, 0, k * sizeof(R), st));
    RNPGPU_CHECK(cudaMemsetAsync(VL, 0, m * k * sizeof(R), st));
    if (VR) RNPGPU_CHECK(cudaMemsetAsync(VR, 0, n * k * sizeof(R), st));
    RNPGPU_CHECK(cudaMemcpyAsync(vecs, hv.data(), hv.size() * sizeof(mg::MgVec), cudaMemcpyHostToDevice, st));
    mg::k_mg_diag<R><<<1, 256, 0, st>>>(dist, mode, sym == 1 ? 1 : 0, cond, dmax, (int)k, d, dw, mode == 0 ? nullptr : d, s0);
    RNPGPU_CHECK_LAUNCH();
    if (!hv.empty()) {
        mg::k_mg_reflect<R><<<(unsigned)hv.size(), 256, 0, st>>>(vecs, s0, VL, m, tauL, VR, n, tauR);
        RNPGPU_CHECK_LAUNCH();
    }
    const dim3 g2((unsigned)std::min<size_t>((m + 255) / 256, 1024), (unsigned)std::min<size_t>(n, 4096));
    mg::k_mg_setdiag<R><<<g2, 256, 0, st>>>((int)m, (int)n, dw, a, lda);
    RNPGPU_CHECK_LAUNCH();
    int rc;
    size_t lw = lwq;
    if ((rc = unmqr<R>("L", "N", m, n, k, VL, m, tauL, a, lda, &lw, wrest))) return rc < 0 ? -13 : rc;
    lw = lwq;
    if (sym == 0) rc = unmqr<R>("R", "C", m, n, k, VR, n, tauR, a, lda, &lw, wrest);
    else rc = unmqr<R>("R", "C", m, n, k, VL, m, tauL, a, lda, &lw, wrest);
    if (rc) return rc < 0 ? -13 : rc;
    if (sym != 0) {
        mg::k_mg_symmetrize<R><<<g2, 256, 0, st>>>((int)n, a, lda);
        RNPGPU_CHECK_LAUNCH();
    }
    // the reference leaves iseed past every number it drew
    mg::state_seed((s0 * mg::powmod(t)) & mg::kMask, iseed);
    // the descriptors are read by the reflector kernel: keep the host copy
    // alive until that copy has been made
    RNPGPU_CHECK(cudaStreamSynchronize(st));
    return kOk;
}

} // namespace rnpgpu
