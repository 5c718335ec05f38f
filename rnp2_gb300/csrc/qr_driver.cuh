// qr_driver.cuh — host side of the blocked Householder QR on one GB300.
//
// Mirrors RNP::LA::QR (RNP/LA/QR.hpp): Factor (geqrf), Factor_unblocked
// (geqr2), MultQ (unmqr/ormqr), MultQ_unblocked (unm2r), GenerateQ
// (ungqr/orgqr) and GenerateQ_unblocked (ung2r), with caller-owned device
// work blocks and RNP's *lwork query.  All pointers are device pointers; work
// is enqueued on the library's current stream and the calls return without
// synchronizing.
#pragma once
#include "qr_kernels.cuh"
#include "panel_cqr.cuh"
#include "update_f32.cuh"
#include "multq_thin.cuh"
#include "tc_gemm.cuh"
#include <algorithm>
#include <type_traits>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <mutex>

namespace rnpgpu {

// status codes of the C ABI
enum : int { kOk = 0, kErrCuda = 1, kErrDevice = 2 };

// ---------------------------------------------------------------------------
// Library context: current stream (per thread), last error, device facts.
// ---------------------------------------------------------------------------
struct DeviceFacts {
    int sm_count = 0;
    int panel_max_blocks[4] = {0, 0, 0, 0};  // per scalar type index
};
cudaStream_t current_stream();
void set_last_error(const char *msg);
const DeviceFacts &device_facts();
int *device_status_ptr();  // library-wide device status word

// Kernel attributes per launch site's kernel (api_context.cu): raise the
// dynamic shared memory limit to dyn_smem (and prefer the largest shared
// memory carveout); blocks of a kernel one SM holds (cached).
int kernel_attr(const void *kern, int dyn_smem, bool max_carveout = false);
int kernel_blocks_per_sm(const void *kern, int threads, size_t dyn_smem);
int kernel_max_cluster(const void *kern, int threads, size_t dyn_smem, int want);

// Launch accounting and optional per-kernel-class timing (CUDA events on the
// launching stream; only while rnpgpu_timing_enable(1) is in effect).
void note_launch();
void ktimer_begin(const char *name, cudaStream_t st);
void ktimer_end(cudaStream_t st);
struct KScope {
    cudaStream_t st;
    KScope(const char *name, cudaStream_t s) : st(s) { ktimer_begin(name, s); }
    ~KScope() { ktimer_end(st); }
};
template <class T> struct TypeName;
template <> struct TypeName<float> { static constexpr const char *v = "f32"; };
template <> struct TypeName<double> { static constexpr const char *v = "f64"; };
template <> struct TypeName<cf32> { static constexpr const char *v = "c32"; };
template <> struct TypeName<cf64> { static constexpr const char *v = "c64"; };

template <class T> struct TypeIndex;
template <> struct TypeIndex<float> { static constexpr int v = 0; };
template <> struct TypeIndex<double> { static constexpr int v = 1; };
template <> struct TypeIndex<cf32> { static constexpr int v = 2; };
template <> struct TypeIndex<cf64> { static constexpr int v = 3; };

#define RNPGPU_CHECK(call)                                                  \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            set_last_error(cudaGetErrorString(e_));                         \
            return kErrCuda;                                                \
        }                                                                   \
    } while (0)
#define RNPGPU_CHECK_LAUNCH()            \
    do {                                 \
        note_launch();                   \
        RNPGPU_CHECK(cudaGetLastError()); \
    } while (0)

// Tuning (RNP/LA/QR.hpp:41-51 keeps nb=32, nbmin=2, crossover=128 for the
// CPU).  On the GPU every column block goes through the blocked path: the
// unblocked tail of the CPU code would run level-2 work on one thread block.
struct GpuTuning {
    static constexpr size_t nb = kPanelMaxCols;
};

// ---------------------------------------------------------------------------
// Workspace carving: regions aligned to 256 bytes inside the caller's block.
// ---------------------------------------------------------------------------
struct Carver {
    char *base;
    size_t off;
    explicit Carver(void *p) : base((char *)p), off(0) {
        size_t mis = (size_t)(uintptr_t)base & 255;
        if (mis) off = 256 - mis;
    }
    template <class U> U *take(size_t count) {
        U *p = base ? (U *)(base + off) : nullptr;
        off += (count * sizeof(U) + 255) & ~(size_t)255;
        return p;
    }
};
// bytes -> elements of T, with the 256-byte alignment slack
template <class T> size_t elems_for(size_t bytes) { return (bytes + 256 + sizeof(T) - 1) / sizeof(T); }

// ---------------------------------------------------------------------------
// Contraction launcher
// ---------------------------------------------------------------------------
template <int BN> int launch_gemm_tc_bn(const GemmArgs<float> &g, int nsplit, cudaStream_t st) {
    if (int rc = kernel_attr((const void *)tc::k_gemm_tc<BN>, tc::SmemLayout<BN>::kBytes)) return rc;
    int *err = device_status_ptr();
    if (err == nullptr) return kErrCuda;
    dim3 grid((g.M + tc::kBM - 1) / tc::kBM, (g.N + BN - 1) / BN, nsplit);
    tc::k_gemm_tc<BN><<<grid, tc::kThreads, tc::SmemLayout<BN>::kBytes, st>>>(g, err);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// FP32 updates with a short contraction (the rank-32 trailing and MultQ
// updates C -= V W^H, K <= 64) and at least one full 128-row tile run on the
// tensor cores (three-term BF16 split).  The long reduction W = C^H V of the
// trailing update goes to the persistent tensor-core kernel below, which
// accumulates at most a few hundred rows per block in TMEM and sums the
// per-block partials in FP32 afterwards; other long reductions stay on FP32
// FMA, whose round-to-nearest accumulation over long K is more accurate than
// one tensor-core accumulator.
inline bool use_tensor_cores(const GemmArgs<float> &g) { return g.M >= 128 && g.K >= 16 && g.K <= 64; }
template <class T> bool use_tensor_cores(const GemmArgs<T> &) { return false; }

// The trailing update C -= V W^T (V unit-lower, K <= 32, N <= 512) goes to
// the FP32 rank-32 update kernel (update_f32.cuh).
inline bool is_trailing_update(const GemmArgs<float> &g, int nsplit) {
    return nsplit == 1 && g.opA == kOpN && g.vunitA && (g.opB == kOpC || g.opB == kOpT) && !g.vunitB && g.beta_mode == kBetaOne && g.alpha == -1.0f && g.K <= 32 &&
           g.N <= kUpdMaxN && g.M >= 128;
}
// two blocks of the update kernel per SM (96 KB of shared memory each: the
// largest carveout), as many blocks as SMs hold: each walks its row tiles
inline int launch_update_f32(const GemmArgs<float> &g, cudaStream_t st) {
    if (int rc = kernel_attr((const void *)k_update_f32<true>, (int)kUfSmem, true)) return rc;
    if (int rc = kernel_attr((const void *)k_update_f32<false>, (int)kUfSmem, true)) return rc;
    UpdArgs u;
    u.V = g.A; u.ldv = g.lda; u.W = g.B; u.ldw = g.ldb; u.C = g.D; u.ldc = g.ldd;
    u.M = g.M; u.N = g.N; u.K = g.K;
    const int ntiles = (g.M + kUfRows - 1) / kUfRows, gy = (g.N + kUfCols - 1) / kUfCols;
    const int gx = std::max(1, std::min(ntiles, device_facts().sm_count * 2 / gy));
    const bool vec = ((uintptr_t)g.D % 16 == 0) && (g.ldd % 4 == 0);
    if (vec) k_update_f32<true><<<dim3(gx, gy), kUfThreads, kUfSmem, st>>>(u);
    else k_update_f32<false><<<dim3(gx, gy), kUfThreads, kUfSmem, st>>>(u);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// W partials P_g = C^T V (g < nsplit, leading dimension N, stride N*K) on the
// FP32 pipe (update_f32.cuh), one partial per split of the rows; nsplit <=
// maxsplit.
inline bool w_partials_ok(int M, int N, int K) { return M >= 1024 && N <= kUpdMaxN && K <= 32; }
inline int launch_w_partials(const float *C, size_t ldc, const float *V, size_t ldv, float *P, int M, int N, int K, int maxsplit, int &nsplit, cudaStream_t st) {
    if (int rc = kernel_attr((const void *)k_w_f32<true>, (int)kWfSmem, true)) return rc;
    if (int rc = kernel_attr((const void *)k_w_f32<false>, (int)kWfSmem, true)) return rc;
    const int nkb = (M + 127) / 128;
    nsplit = std::max(1, std::min(std::min(nkb, maxsplit), device_facts().sm_count));
    UpdArgs u;
    u.V = V; u.ldv = ldv; u.W = nullptr; u.ldw = 0; u.C = const_cast<float *>(C); u.ldc = ldc; u.M = M; u.N = N; u.K = K;
    const int rps = ((M + nsplit - 1) / nsplit + 3) / 4 * 4;  // a multiple of 4: aligned row quads
    nsplit = (M + rps - 1) / rps;
    const dim3 grid(nsplit, (N + kWfCols - 1) / kWfCols);
    const bool vec = ((uintptr_t)C % 16 == 0) && (ldc % 4 == 0);
    if (vec) k_w_f32<true><<<grid, kUfThreads, kWfSmem, st>>>(u, P, rps);
    else k_w_f32<false><<<grid, kUfThreads, kWfSmem, st>>>(u, P, rps);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}
template <class T> int launch_w_partials(const T *, size_t, const T *, size_t, T *, int, int, int, int, int &, cudaStream_t) { return kErrDevice; }

inline int launch_gemm_tc(const GemmArgs<float> &g, int nsplit, cudaStream_t st) {
    if (is_trailing_update(g, nsplit)) return launch_update_f32(g, st);
    if (g.N <= 32) return launch_gemm_tc_bn<32>(g, nsplit, st);
    return launch_gemm_tc_bn<64>(g, nsplit, st);
}
template <class T> int launch_gemm_tc(const GemmArgs<T> &, int, cudaStream_t) { return kErrDevice; }

template <class T> int launch_gemm(GemmArgs<T> g, int nsplit, cudaStream_t st, const char *tag = "gemm") {
    if (g.M <= 0 || g.N <= 0) return kOk;
    if (g.K <= 0 && g.beta_mode == kBetaOne) return kOk;
    if (g.kchunk <= 0) g.kchunk = g.K > 0 ? g.K : 1;
    KScope ks(tag, st);
    if (use_tensor_cores(g)) return launch_gemm_tc(g, nsplit, st);
    // FP64 work: an SM retires an FP64 warp instruction only every ~16
    // cycles, so a grid that leaves SMs idle takes the smaller tiles
    constexpr bool f64 = sizeof(typename Tr<T>::R) == 8;
    const long sms = device_facts().sm_count > 0 ? device_facts().sm_count : 148;
    if (f64 && g.N <= 16 && (long)((g.M + 127) / 128) * nsplit < sms) {
        dim3 grid((g.M + 31) / 32, (g.N + 15) / 16, nsplit);
        k_gemm<T, 32, 16, 16, 2, 1><<<grid, 256, 0, st>>>(g);
    } else if (f64 && g.N > 16 && (long)((g.M + 31) / 32) * ((g.N + 31) / 32) * nsplit < sms / 2) {
        dim3 grid((g.M + 15) / 16, (g.N + 31) / 32, nsplit);
        k_gemm<T, 16, 32, 16, 1, 2><<<grid, 256, 0, st>>>(g);
    } else if (f64 && g.N > 16 && (long)((g.M + 63) / 64) * ((g.N + 63) / 64) * nsplit < sms) {
        dim3 grid((g.M + 31) / 32, (g.N + 31) / 32, nsplit);
        k_gemm<T, 32, 32, 16, 2, 2><<<grid, 256, 0, st>>>(g);
    } else if (g.N <= 16) {
        dim3 grid((g.M + 127) / 128, (g.N + 15) / 16, nsplit);
        k_gemm<T, 128, 16, 16, 8, 1><<<grid, 256, 0, st>>>(g);
    } else if (g.N <= 32) {
        dim3 grid((g.M + 63) / 64, (g.N + 31) / 32, nsplit);
        k_gemm<T, 64, 32, 16, 4, 2><<<grid, 256, 0, st>>>(g);
    } else {
        dim3 grid((g.M + 63) / 64, (g.N + 63) / 64, nsplit);
        k_gemm<T, 64, 64, 16, 4, 4><<<grid, 256, 0, st>>>(g);
    }
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// Cooperative launch; on failure the message names the kernel, its grid and
// how many of its blocks an SM holds.
inline int coop_launch(const char *name, const void *kern, int grid, int threads, void **args, size_t smem, cudaStream_t st) {
    const cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(threads), args, smem, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        int per_sm = -1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess) {
            cudaGetLastError();
            per_sm = -1;
        }
        int per_sm0 = -1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm0, kern, threads, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm0 = -1;
        }
        cudaFuncAttributes fa{};
        if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) cudaGetLastError();
        char msg[400];
        snprintf(msg, sizeof msg, "%s: %s (grid %d x %d threads, %zu B dynamic shared memory; %d blocks per SM fit, %d without dynamic shared memory; %d SMs; %d registers, %zu B static shared memory, max %d threads, max dynamic %d B)",
                 name, cudaGetErrorString(e), grid, threads, smem, per_sm, per_sm0, device_facts().sm_count, fa.numRegs, (size_t)fa.sharedSizeBytes, fa.maxThreadsPerBlock,
                 fa.maxDynamicSharedSizeBytes);
        set_last_error(msg);
        return kErrCuda;
    }
    note_launch();
    return kOk;
}

// one thread-block cluster of `grid` blocks
inline int cluster_launch(const char *name, const void *kern, int grid, int threads, void **args, size_t smem, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = grid;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelExC(&cfg, kern, args);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char msg[200];
        snprintf(msg, sizeof msg, "%s: %s (cluster of %d x %d threads, %zu B dynamic shared memory)", name, cudaGetErrorString(e), grid, threads, smem);
        set_last_error(msg);
        return kErrCuda;
    }
    note_launch();
    return kOk;
}

template <class T> GemmArgs<T> gemm_args(const T *A, size_t lda, int opA, int vunitA, const T *B, size_t ldb, int opB, int vunitB, T *D, size_t ldd, int M, int N, int K, T alpha, int beta_mode) {
    GemmArgs<T> g;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.D = D; g.ldd = ldd;
    g.M = M; g.N = N; g.K = K;
    g.opA = opA; g.opB = opB; g.vunitA = vunitA; g.vunitB = vunitB;
    g.alpha = alpha; g.beta_mode = beta_mode;
    g.kchunk = K; g.dstride = 0;
    return g;
}

// split-K plan for a reduction of length K producing 'tiles' output tiles
// Fewest rows a split-K partial may cover: FP64 arithmetic runs at 1/64 of
// the FP32 rate on this GPU, so FP64 contractions with few output tiles need
// many short splits to occupy the SMs.
template <class T> constexpr int split_min_rows() { return sizeof(typename Tr<T>::R) == 8 ? 32 : 256; }

inline int choose_splits(int K, int tiles, int smax, int min_rows = 256) {
    const int sm = device_facts().sm_count > 0 ? device_facts().sm_count : 148;
    int s = (2 * sm + tiles - 1) / std::max(tiles, 1);
    s = std::min(s, std::max(1, K / min_rows));
    s = std::min(s, smax);
    return std::max(s, 1);
}

// W = (sum of nsplit partials) * op(T) in one launch (many partials: four
// split lanes per entry)
template <class T> int sum_times_t(const T *P, size_t ldp, size_t pstride, int nsplit, int rows, int k, const T *Tm, int ldt, int opT, T *W, size_t ldw, cudaStream_t st) {
    if (nsplit > 8) {
        k_reduce_times_t<T><<<rows, 256, 0, st>>>(P, ldp, pstride, nsplit, rows, k, Tm, ldt, opT, W, ldw);
        RNPGPU_CHECK_LAUNCH();
        return kOk;
    }
    k_sum_times_t<T><<<(rows + 7) / 8, 256, 0, st>>>(P, ldp, pstride, nsplit, rows, k, Tm, ldt, opT, W, ldw);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// ---------------------------------------------------------------------------
// Block reflector application (ApplyBlock, storev "C", dir "F",
// RNP/LA/Reflector.hpp:725-815).  V is the ib-column reflector block in its
// stored form (unit diagonal implicit), T its upper triangular factor.
//   left : C(M x N) <- H C or H^H C :  W = C^H V op(T), C -= V W^H
//   right: C(M x N) <- C H or C H^H :  W = C V op(T),   C -= W V^H
// P holds the split-K partials (smax * rows_of_W * ib), W the result.
// ---------------------------------------------------------------------------
template <class T> struct BlockWs {
    T *P;
    T *W;
    int smax;
};

template <class T> int apply_block(bool left, bool notran, int M, int N, int ib, const T *V, size_t ldv, const T *Tm, int ldt, T *C, size_t ldc, const BlockWs<T> &ws, cudaStream_t st) {
    if (M <= 0 || N <= 0 || ib <= 0) return kOk;
    int rc;
    if (left) {
        if (std::is_same<T, float>::value && w_partials_ok(M, N, ib)) {
            // FP32: W partials per split of the rows (update_f32.cuh), their
            // sum times op(T), then the rank-ib update
            int nsplit = 1;
            {
                KScope ks("larfb_w", st);
                if ((rc = launch_w_partials(C, ldc, V, ldv, ws.P, M, N, ib, ws.smax, nsplit, st))) return rc;
            }
            if ((rc = sum_times_t<T>(ws.P, (size_t)N, (size_t)N * ib, nsplit, N, ib, Tm, ldt, notran ? kOpC : kOpN, ws.W, (size_t)N, st))) return rc;
            GemmArgs<T> u = gemm_args<T>(V, ldv, kOpN, 1, ws.W, (size_t)N, kOpC, 0, C, ldc, M, N, ib, T(-1), kBetaOne);
            return launch_gemm(u, 1, st, "larfb_update");
        }
        // W = C^H V  (N x ib), reduction over the M rows
        const int tiles = (N + 63) / 64;
        const int S = choose_splits(M, tiles, ws.smax, split_min_rows<T>());
        int kchunk = ((M + S - 1) / S + 15) / 16 * 16;
        if (std::is_same<T, float>::value) {
            // tensor-core path: at most ~1024 rows per accumulator, within
            // the partial buffer's smax slots
            const int floor_chunk = ((M + ws.smax - 1) / ws.smax + 15) / 16 * 16;
            kchunk = std::max(floor_chunk, std::min(kchunk, 1024));
        }
        const int nsplit = (M + kchunk - 1) / kchunk;
        GemmArgs<T> g = gemm_args<T>(C, ldc, kOpC, 0, V, ldv, kOpN, 1, ws.P, (size_t)N, N, ib, M, T(1), kBetaZero);
        g.kchunk = kchunk;
        g.dstride = (size_t)N * ib;
        if ((rc = launch_gemm(g, nsplit, st, "larfb_w"))) return rc;
        // W := W T (H^H) or W T^H (H)
        if ((rc = sum_times_t<T>(ws.P, (size_t)N, (size_t)N * ib, nsplit, N, ib, Tm, ldt, notran ? kOpC : kOpN, ws.W, (size_t)N, st))) return rc;
        // C -= V W^H
        GemmArgs<T> u = gemm_args<T>(V, ldv, kOpN, 1, ws.W, (size_t)N, kOpC, 0, C, ldc, M, N, ib, T(-1), kBetaOne);
        return launch_gemm(u, 1, st, "larfb_update");
    } else {
        // W = C V  (M x ib), reduction over the N columns
        const int tiles = (M + 63) / 64;
        const int S = choose_splits(N, tiles, ws.smax, split_min_rows<T>());
        const int kchunk = ((N + S - 1) / S + 15) / 16 * 16;
        const int nsplit = (N + kchunk - 1) / kchunk;
        GemmArgs<T> g = gemm_args<T>(C, ldc, kOpN, 0, V, ldv, kOpN, 1, ws.P, (size_t)M, M, ib, N, T(1), kBetaZero);
        g.kchunk = kchunk;
        g.dstride = (size_t)M * ib;
        if ((rc = launch_gemm(g, nsplit, st, "larfb_w"))) return rc;
        if ((rc = sum_times_t<T>(ws.P, (size_t)M, (size_t)M * ib, nsplit, M, ib, Tm, ldt, notran ? kOpN : kOpC, ws.W, (size_t)M, st))) return rc;
        // C -= W V^H
        GemmArgs<T> u = gemm_args<T>(ws.W, (size_t)M, kOpN, 0, V, ldv, kOpC, 1, C, ldc, M, N, ib, T(-1), kBetaOne);
        return launch_gemm(u, 1, st, "larfb_update");
    }
}

// T factor of one reflector block from V and tau (GenerateBlockTr "F","C"):
// Gram matrix V^H V by a split-K contraction, then the recurrence.
template <class T> int block_t(int rows, int ib, const T *V, size_t ldv, const T *tau, T *Tout, int ldt, T *Pg, int smax, cudaStream_t st) {
    const int S = choose_splits(rows, 1, smax, split_min_rows<T>());
    const int kchunk = ((rows + S - 1) / S + 15) / 16 * 16;
    const int nsplit = (rows + kchunk - 1) / kchunk;
    GemmArgs<T> g = gemm_args<T>(V, ldv, kOpC, 1, V, ldv, kOpN, 1, Pg, (size_t)kPanelMaxCols, ib, ib, rows, T(1), kBetaZero);
    g.kchunk = kchunk;
    g.dstride = (size_t)kPanelMaxCols * kPanelMaxCols;
    int rc = launch_gemm(g, nsplit, st, "larft_gram");
    if (rc) return rc;
    k_build_t<T><<<1, kBuildTThreads, 0, st>>>(Pg, (size_t)kPanelMaxCols * kPanelMaxCols, 0, nsplit, tau, ib, ib, Tout, 0, ldt);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// ---------------------------------------------------------------------------
// Panel factorization launcher (cooperative grid)
// ---------------------------------------------------------------------------
template <class T> struct PanelWs {
    PanelRec<T> *rec;  // [2][gmax]
    unsigned *sync;    // [0] counter, [1] error word
    int gmax;
};

inline int panel_grid(int M, int gmax) {
    int g = (M + 31) / 32;
    g = std::min(g, gmax);
    return std::max(g, 1);
}

// shared-memory budget for a block's rows of the panel
constexpr size_t kPanelSmemMax = 180 * 1024;

// Panels of at most this many rows (default 4096; the environment variable
// RNPGPU_PANEL_CLUSTER_ROWS overrides it, 0 turns the form off) run as one
// thread-block cluster of up to 16 blocks of about 64 rows or more.
inline int panel_cluster_rows() {
    static const int rows = []() {
        const char *e = getenv("RNPGPU_PANEL_CLUSTER_ROWS");
        return e ? atoi(e) : 4096;
    }();
    return rows;
}
constexpr int kPanelClusterRowsPerBlock = 64;
// the short panels' blocks hold few rows: four warps, so that the per-column
// reductions (FP64, whose one pipe per SM takes a warp instruction every 16
// cycles) run in few warps
constexpr int kPanelClusterThreads = 128;

template <class T> int panel_factor(int M, int N, T *A, size_t lda, T *tau, T *Tm, int ldt, const PanelWs<T> &ws, cudaStream_t st) {
    if (M <= panel_cluster_rows() && M > kPanelClusterRowsPerBlock) {
        // short panel: one cluster, records in distributed shared memory
        const void *kc = (const void *)k_panel<T, true, true, kPanelClusterThreads>;
        if (int rc = kernel_attr(kc, (int)kPanelSmemMax)) return rc;
        // the largest cluster (<= 16 blocks) that fits with its rows' shared
        // memory; g falls strictly until the query agrees
        int g = std::min(16, (M + kPanelClusterRowsPerBlock - 1) / kPanelClusterRowsPerBlock);
        while (g >= 2) {
            const size_t smem = (size_t)(((M + g - 1) / g) | 1) * N * sizeof(T);
            if (smem > kPanelSmemMax) {
                g = 0;
                break;
            }
            const int c = kernel_max_cluster(kc, kPanelClusterThreads, smem, g);
            if (c == g) break;
            g = c;
        }
        if (g >= 2 && (M + g - 1) / g <= 1024) {
            PanelArgs<T> p;
            p.A = A; p.lda = lda; p.M = M; p.N = N; p.tau = tau; p.Tm = Tm; p.ldt = ldt;
            p.rec = nullptr;
            p.counter = nullptr; p.err = nullptr;
            p.status = device_status_ptr();
            p.rows_per_cta = (M + g - 1) / g;
            void *args[] = {&p};
            KScope ks("panel", st);
            return cluster_launch("k_panel(cluster)", kc, g, kPanelClusterThreads, args, (size_t)(p.rows_per_cta | 1) * N * sizeof(T), st);
        }
    }
    const int G = panel_grid(M, ws.gmax);
    if (int rc = kernel_attr((const void *)k_panel<T, true>, (int)kPanelSmemMax)) return rc;
    PanelArgs<T> p;
    p.A = A; p.lda = lda; p.M = M; p.N = N; p.tau = tau; p.Tm = Tm; p.ldt = ldt;
    p.rec = ws.rec;
    p.counter = ws.sync; p.err = (int *)(ws.sync + 1);
    p.status = device_status_ptr();
    p.rows_per_cta = (M + G - 1) / G;
    RNPGPU_CHECK(cudaMemsetAsync(ws.sync, 0, 2 * sizeof(unsigned), st));
    void *args[] = {&p};
    KScope ks("panel", st);
    const size_t smem = (size_t)p.rows_per_cta * N * sizeof(T);
    if (smem <= kPanelSmemMax && G <= device_facts().sm_count) return coop_launch("k_panel", (const void *)k_panel<T, true>, G, kPanelThreads, args, smem, st);
    return coop_launch("k_panel", (const void *)k_panel<T, false>, G, kPanelThreads, args, 0, st);
}

template <class T> int panel_gmax() {
    const DeviceFacts &f = device_facts();
    int g = f.panel_max_blocks[TypeIndex<T>::v];
    return std::max(1, std::min(g, f.sm_count));
}

// ---------------------------------------------------------------------------
// Workspace plans (bytes), shared by the query and the run
// ---------------------------------------------------------------------------
template <class T> size_t panel_ws_bytes(int gmax) {
    return ((size_t)2 * gmax * sizeof(PanelRec<T>) + 255) / 256 * 256 + 256;
}
template <class T> PanelWs<T> carve_panel(Carver &cv, int gmax) {
    PanelWs<T> w;
    w.rec = cv.take<PanelRec<T> >((size_t)2 * gmax);
    w.sync = cv.take<unsigned>(2);
    w.gmax = gmax;
    return w;
}
template <class T> size_t block_ws_bytes(int rows_w, int smax) {
    return ((size_t)smax * rows_w * kPanelMaxCols * sizeof(T) + 255) / 256 * 256 + ((size_t)rows_w * kPanelMaxCols * sizeof(T) + 255) / 256 * 256;
}
template <class T> BlockWs<T> carve_block(Carver &cv, int rows_w, int smax) {
    BlockWs<T> w;
    w.P = cv.take<T>((size_t)smax * rows_w * kPanelMaxCols);
    w.W = cv.take<T>((size_t)rows_w * kPanelMaxCols);
    w.smax = smax;
    return w;
}
// split-K slots of the W partials: up to one per SM (the tensor-core W
// reduction writes one partial per persistent block)
template <class T> inline int smax_for(size_t K) {
    return (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(64, device_facts().sm_count), K / (size_t)split_min_rows<T>()));
}
template <class T> size_t t_bytes() { return ((size_t)kPanelMaxCols * kPanelMaxCols * sizeof(T) + 255) / 256 * 256; }

// ---------------------------------------------------------------------------
// Factor (geqrf): RNP/LA/QR.hpp:129-197
// ---------------------------------------------------------------------------
template <class T> int geqr2(size_t m, size_t n, T *a, size_t lda, T *tau, T *work);

}  // namespace rnpgpu
#include "wide_f32.cuh"
namespace rnpgpu {

// CholeskyQR2 panels of the mixed solver's FP32 factor (panel_cqr.cuh):
// Gram partials, the top rows of Q1, the failure flag; optionally the
// workspace of the 128-column tensor-core trailing update (wide_f32.cuh)
struct CqrWs {
    float2 *gpart = nullptr;
    float2 *gfin = nullptr;
    float *qtop = nullptr;
    int *fail = nullptr;
    wide::WideWs wide;
    bool use_wide = false;
    // when set, the matrix may still be arriving (host staging), 128 columns
    // at a time: range r (columns 128 r ..) is ready once range_ready[r] has
    // completed.  The mixed factor then runs left-looking by 128-column
    // blocks (each range is brought up to date by the blocks left of it when
    // it is reached), so that it works on the ranges that have landed while
    // the rest is still copied.
    const cudaEvent_t *range_ready = nullptr;
    int nranges = 0;
    // left-looking only: block b's V slice images at vcache + b * vcache_stride
    // (made by its first application, reused by the later ones)
    unsigned char *vcache = nullptr;
    size_t vcache_stride = 0;
    // when set, the 128 x 128 T of every wide block is kept here (block b at
    // t128 + b * 128 * 128, row-major); geqrf reports in nwide how many
    // leading 128-column blocks have one
    float *t128 = nullptr;
    mutable int nwide = 0;
};
inline size_t cqr_ws_bytes() {
    const auto r = [](size_t b) { return (b + 255) / 256 * 256; };
    return r((size_t)kPanelMaxBlocksCqr * kCqrEntries * sizeof(float2)) + r(kCqrEntries * sizeof(float2)) +
           r((size_t)kPanelMaxCols * kPanelMaxCols * sizeof(float)) + 256;
}
inline CqrWs carve_cqr(Carver &cv) {
    CqrWs w;
    w.gpart = cv.take<float2>((size_t)kPanelMaxBlocksCqr * kCqrEntries);
    w.gfin = cv.take<float2>(kCqrEntries);
    w.qtop = cv.take<float>((size_t)kPanelMaxCols * kPanelMaxCols);
    w.fail = cv.take<int>(1);
    return w;
}
// rows of a CholeskyQR2 panel per block: block 0 holds the top 32 rows, the
// other blocks share the rest (one block: all rows)
inline int cqr_rows_per_block(int M, int g) { return g == 1 ? M : (M - kPanelMaxCols + g - 2) / (g - 1); }
inline int cqr_rows_held(int M, int g) { return std::max(kPanelMaxCols, cqr_rows_per_block(M, g)); }
// grid of a CholeskyQR2 panel: M / 32 blocks at most (every block at least
// 32 rows), all of a block's rows in shared memory; 0 when the panel does not
// qualify
inline int cqr_grid(int M, int N) {
    if (N < 1 || N > kPanelMaxCols) return 0;
    const int g = std::min({M / kPanelMaxCols, device_facts().sm_count, kPanelMaxBlocksCqr});
    if (g < 1) return 0;
    if ((size_t)cqr_rows_held(M, g) * kCqrLd * sizeof(float) > (size_t)kCqrMaxDynSmem) return 0;
    return g;
}
inline int panel_factor_cqr(int M, int N, float *A, size_t lda, float *tau, float *Tm, int ldt, const PanelWs<float> &pw, const CqrWs &cw, cudaStream_t st) {
    const int G = cqr_grid(M, N);
    if (G == 0) return kErrDevice;
    if (int rc = kernel_attr((const void *)k_panel_cqr<0>, kCqrMaxDynSmem)) return rc;
    CqrArgs p;
    p.A = A; p.lda = lda; p.M = M; p.N = N; p.tau = tau; p.Tm = Tm; p.ldt = ldt;
    p.gpart = cw.gpart; p.gfin = cw.gfin; p.qtop = cw.qtop; p.fail = cw.fail;
    p.counter = pw.sync; p.err = (int *)(pw.sync + 1); p.status = device_status_ptr();
    p.rows_per_cta = cqr_rows_per_block(M, G);
    RNPGPU_CHECK(cudaMemsetAsync(pw.sync, 0, 2 * sizeof(unsigned), st));
    void *args[] = {&p};
    KScope ks("panel_cqr", st);
    const size_t smem = (size_t)cqr_rows_held(M, G) * kCqrLd * sizeof(float);
    return coop_launch("k_panel_cqr", (const void *)k_panel_cqr<0>, G, kCqrThreads, args, smem, st);
}

// serial blocked form: panel workspace, one T, one update workspace
template <class T> size_t geqrf_serial_bytes(size_t m, size_t n, int smax) {
    return panel_ws_bytes<T>(panel_gmax<T>()) + t_bytes<T>() + block_ws_bytes<T>((int)n, smax);
}
// Look-ahead (below) pays for FP64 and complex data, whose trailing updates
// are FMA-bound and long against the panel (square 4096 complex: 513 -> 451
// ms); FP32 trailing updates on the tensor cores are short and latency bound,
// and running the next panel beside them made the 65536 x 512 FP32 factor
// slower (8.8 -> 9.6 ms per mixed solve), so FP32 keeps the serial order.
template <class T> constexpr bool geqrf_lookahead() { return !std::is_same<T, float>::value; }
// look-ahead form: a second T and a second update workspace
template <class T> size_t geqrf_bytes(size_t m, size_t n, int smax) {
    return geqrf_serial_bytes<T>(m, n, smax) + (geqrf_lookahead<T>() ? t_bytes<T>() + block_ws_bytes<T>((int)n, smax) : 0);
}

// Per host thread and device: the side stream and two events of the
// look-ahead factorization (created on first use, outside stream capture).
struct LookAhead {
    cudaStream_t side = nullptr;
    cudaEvent_t ev_panel = nullptr, ev_big = nullptr;
};
inline LookAhead *lookahead_ctx() {
    constexpr int kMaxDev = 16;
    static thread_local LookAhead la[kMaxDev];
    static thread_local int state[kMaxDev] = {};  // 0 untried, 1 ready, 2 failed
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
    if (state[dev] == 0) {
        LookAhead &l = la[dev];
        const bool ok = cudaStreamCreateWithFlags(&l.side, cudaStreamNonBlocking) == cudaSuccess &&
                        cudaEventCreateWithFlags(&l.ev_panel, cudaEventDisableTiming) == cudaSuccess &&
                        cudaEventCreateWithFlags(&l.ev_big, cudaEventDisableTiming) == cudaSuccess;
        state[dev] = ok ? 1 : 2;
        if (!ok) cudaGetLastError();
    }
    return state[dev] == 1 ? &la[dev] : nullptr;
}

// Tstore (optional): receives the 32 x 32 T factor of every column block
// (block b at Tstore + b*32*32, leading dimension 32) for later MultQ calls.
//
// Look-ahead: after panel i only the next panel's columns are updated on the
// caller's stream; the rest of the trailing matrix is updated on a side
// stream while panel i + 1 (latency bound: one grid barrier per column) is
// factored, and the caller's stream waits for that update before it touches
// those columns again.  The results are the same as in the serial order (the
// same operations on the same data).  Without the larger workspace, inside
// stream capture, or for a single trailing block the serial order is used.
//
// lookahead_ok = false keeps the serial order (no side stream or events are
// created, nothing beyond the serial plan is asked of the work block).
inline bool a32_usable(int M, int N, int K, const float *V, size_t ldv, const float *C, size_t ldc, const BlockWs<float> &ws, size_t p_floats, size_t w_floats);
inline int apply32(int M, int N, int K, const float *V, size_t ldv, const float *Tm, float *C, size_t ldc, const BlockWs<float> &ws, cudaStream_t st);
template <class T> int geqrf(size_t m, size_t n, T *a, size_t lda, T *tau, size_t *lwork, T *work, T *Tstore = nullptr, const CqrWs *cqr = nullptr, bool lookahead_ok = true) {
    if (lwork == nullptr) return -6;
    const size_t k = std::min(m, n);
    if (k == 0) return kOk;
    if (lda < std::max<size_t>(1, m)) return -4;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -1;
    int smax = smax_for<T>(m);
    if (work == nullptr || *lwork == 0) {
        *lwork = elems_for<T>(geqrf_bytes<T>(m, n, smax));
        return kOk;
    }
    if (a == nullptr) return -3;
    if (tau == nullptr) return -5;
    const size_t nb = GpuTuning::nb;
    cudaStream_t st = current_stream();
    bool ahead = lookahead_ok && geqrf_lookahead<T>() && n > 2 * nb && k > nb && elems_for<T>(geqrf_bytes<T>(m, n, smax)) <= *lwork;
    if (ahead) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) ahead = false;
    }
    LookAhead *la = ahead ? lookahead_ctx() : nullptr;
    if (la == nullptr) {
        ahead = false;
        while (smax > 1 && elems_for<T>(geqrf_serial_bytes<T>(m, n, smax)) > *lwork) smax /= 2;
        if (elems_for<T>(geqrf_serial_bytes<T>(m, n, smax)) > *lwork) {
            // not enough workspace for the blocked code: level-2 code needs n
            if (*lwork < n) return -6;
            return geqr2<T>(m, n, a, lda, tau, work);
        }
    }
    Carver cv(work);
    const int gmax = panel_gmax<T>();
    PanelWs<T> pw = carve_panel<T>(cv, gmax);
    T *Tm[2];
    Tm[0] = cv.take<T>((size_t)kPanelMaxCols * kPanelMaxCols);
    BlockWs<T> bw = carve_block<T>(cv, (int)n, smax);
    BlockWs<T> bw2 = bw;
    Tm[1] = Tm[0];
    if (ahead) {
        Tm[1] = cv.take<T>((size_t)kPanelMaxCols * kPanelMaxCols);
        bw2 = carve_block<T>(cv, (int)n, smax);
    }
    // the mixed solver's FP32 factor: 128-column blocks of four panels,
    // updated among themselves by the rank-32 passes, the rest of the matrix
    // by one tensor-core update per block (wide_f32.cuh)
    bool wide_mode = false;
    if constexpr (std::is_same<T, float>::value) {
        wide_mode = !ahead && cqr != nullptr && cqr->use_wide && Tstore != nullptr && wide::usable(m, n, a, lda);
    }
    if (cqr != nullptr) cqr->nwide = 0;
    bool big_pending = false;
    // staged input: left-looking 128-column blocks in wide mode, else wait
    // for every range up front
    const bool staged = cqr != nullptr && cqr->range_ready != nullptr && cqr->nranges > 0;
    const bool left_looking = staged && wide_mode;
    if (staged && !left_looking) {
        for (int r = 0; r < cqr->nranges; ++r) {
            RNPGPU_CHECK(cudaStreamWaitEvent(st, cqr->range_ready[r], 0));
            if (la) RNPGPU_CHECK(cudaStreamWaitEvent(la->side, cqr->range_ready[r], 0));
        }
    }
    for (size_t i = 0; i < k; i += nb) {
        const int ib = (int)std::min(nb, k - i);
        T *Ai = a + i + i * lda;
        T *Tb = Tstore ? Tstore + (i / nb) * kPanelMaxCols * kPanelMaxCols : Tm[(i / nb) & 1];
        int rc;
        if constexpr (std::is_same<T, float>::value) {
            if (left_looking && i % wide::kNb == 0) {
                // block jb's columns: once landed, updated by every block left of it
                const int jb = (int)(i / wide::kNb);
                if (jb < cqr->nranges) RNPGPU_CHECK(cudaStreamWaitEvent(st, cqr->range_ready[jb], 0));
                const size_t cend = std::min(n, (size_t)(jb + 1) * wide::kNb);
                for (int b0 = 0; b0 < jb; ++b0) {
                    const size_t j0 = (size_t)b0 * wide::kNb;
                    float *tsave = cqr->t128 ? cqr->t128 + (size_t)b0 * wide::kNb * wide::kNb : nullptr;
                    unsigned char *vc = (cqr->vcache && tsave) ? cqr->vcache + (size_t)b0 * cqr->vcache_stride : nullptr;
                    rc = wide::apply(a, lda, (int)m, (int)cend, (int)j0, Tstore + (j0 / nb) * kPanelMaxCols * kPanelMaxCols, (size_t)kPanelMaxCols * kPanelMaxCols, cqr->wide, st, tsave,
                                     (int)i, vc, vc != nullptr && jb > b0 + 1);
                    if (rc) return rc;
                    if (tsave && cqr->nwide == b0) cqr->nwide = b0 + 1;
                }
            }
        }
        if constexpr (std::is_same<T, float>::value) {
            if (cqr != nullptr && cqr_grid((int)(m - i), ib) > 0)
                rc = panel_factor_cqr((int)(m - i), ib, Ai, lda, tau + i, Tb, kPanelMaxCols, pw, *cqr, st);
            else
                rc = panel_factor<T>((int)(m - i), ib, Ai, lda, tau + i, Tb, kPanelMaxCols, pw, st);
        } else {
            rc = panel_factor<T>((int)(m - i), ib, Ai, lda, tau + i, Tb, kPanelMaxCols, pw, st);
        }
        if (rc) return rc;
        const size_t c1 = i + ib;  // first trailing column
        if (c1 >= n) continue;
        if constexpr (std::is_same<T, float>::value) {
            if (wide_mode) {
                const size_t j0 = i / wide::kNb * wide::kNb, jend = std::min(j0 + wide::kNb, n);
                if (c1 < jend) {
                    // the rest of the block: one launch when it is at most 64
                    // columns (k_apply32), else the three launches of the
                    // rank-32 passes
                    const int Mr = (int)(m - i), Nr = (int)(jend - c1);
                    float *Cr = a + i + c1 * lda;
                    // (two launches of 48 columns for the 96-column case measured
                    // slower than the three-launch path)
                    if (a32_usable(Mr, Nr, ib, Ai, lda, Cr, lda, bw, (size_t)bw.smax * n * kPanelMaxCols, n * kPanelMaxCols))
                        rc = apply32(Mr, Nr, ib, Ai, lda, Tb, Cr, lda, bw, st);
                    else
                        rc = apply_block<T>(true, false, Mr, Nr, ib, Ai, lda, Tb, kPanelMaxCols, Cr, lda, bw, st);
                    if (rc) return rc;
                }
                const bool block_done = (c1 == j0 + wide::kNb) || (c1 == k);
                if (block_done && jend < n && !left_looking) {
                    if (c1 == j0 + wide::kNb && m - j0 >= 128) {
                        const int wb = (int)(j0 / wide::kNb);
                        float *tsave = cqr->t128 ? cqr->t128 + (size_t)wb * wide::kNb * wide::kNb : nullptr;
                        rc = wide::apply(a, lda, (int)m, (int)n, (int)j0, Tstore + (j0 / nb) * kPanelMaxCols * kPanelMaxCols, (size_t)kPanelMaxCols * kPanelMaxCols, cqr->wide, st, tsave);
                        if (rc) return rc;
                        if (tsave && cqr->nwide == wb) cqr->nwide = wb + 1;
                    } else {
                        for (size_t p = j0; p < c1; p += nb) {
                            const int pb = (int)std::min(nb, k - p);
                            rc = apply_block<T>(true, false, (int)(m - p), (int)(n - jend), pb, a + p + p * lda, lda, Tstore + (p / nb) * kPanelMaxCols * kPanelMaxCols,
                                                kPanelMaxCols, a + p + jend * lda, lda, bw, st);
                            if (rc) return rc;
                        }
                    }
                }
                continue;
            }
        }
        if (!ahead) {
            rc = apply_block<T>(true, false, (int)(m - i), (int)(n - c1), ib, Ai, lda, Tb, kPanelMaxCols, a + i + c1 * lda, lda, bw, st);
            if (rc) return rc;
            continue;
        }
        const size_t w1 = std::min(nb, n - c1);  // the next panel's columns
        if (c1 + w1 < n) {
            // the rest of the trailing matrix, on the side stream (after the
            // previous side update, in stream order)
            RNPGPU_CHECK(cudaEventRecord(la->ev_panel, st));
            RNPGPU_CHECK(cudaStreamWaitEvent(la->side, la->ev_panel, 0));
        }
        // the next panel's columns were last written by the previous side update
        if (big_pending) RNPGPU_CHECK(cudaStreamWaitEvent(st, la->ev_big, 0));
        big_pending = false;
        rc = apply_block<T>(true, false, (int)(m - i), (int)w1, ib, Ai, lda, Tb, kPanelMaxCols, a + i + c1 * lda, lda, bw, st);
        if (rc) return rc;
        if (c1 + w1 < n) {
            rc = apply_block<T>(true, false, (int)(m - i), (int)(n - c1 - w1), ib, Ai, lda, Tb, kPanelMaxCols, a + i + (c1 + w1) * lda, lda, bw2, la->side);
            if (rc) return rc;
            RNPGPU_CHECK(cudaEventRecord(la->ev_big, la->side));
            big_pending = true;
        }
    }
    if (big_pending) RNPGPU_CHECK(cudaStreamWaitEvent(st, la->ev_big, 0));
    return kOk;
}

// ---------------------------------------------------------------------------
// Factor_unblocked (geqr2): RNP/LA/QR.hpp:78-102.  Level-2 kernels, work of
// length n holds w = v^H C, as in the reference.
// ---------------------------------------------------------------------------
template <class T> int larf_launch(bool left, int mc, int nc, const T *v, const T *taup, bool conj_tau, T *C, size_t ldc, T *w, cudaStream_t st) {
    if (mc <= 0 || nc <= 0) return kOk;
    if (left) k_larf_w<T><<<(nc + 7) / 8, 256, 0, st>>>(1, mc, nc, v, C, ldc, w);
    else k_larf_w<T><<<(mc + 255) / 256, 256, 0, st>>>(0, mc, nc, v, C, ldc, w);
    RNPGPU_CHECK_LAUNCH();
    dim3 grid((mc + 255) / 256, std::min(nc, 65535));
    k_larf_update<T><<<grid, 256, 0, st>>>(left ? 1 : 0, mc, nc, v, w, taup, conj_tau ? 1 : 0, C, ldc);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> int geqr2(size_t m, size_t n, T *a, size_t lda, T *tau, T *work) {
    const size_t k = std::min(m, n);
    if (k == 0) return kOk;
    if (lda < std::max<size_t>(1, m)) return -4;
    if (a == nullptr) return -3;
    if (tau == nullptr) return -5;
    if (work == nullptr && n > 1) return -6;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -1;
    cudaStream_t st = current_stream();
    for (size_t i = 0; i < k; ++i) {
        const size_t row = std::min(i + 1, m - 1);
        k_larfg<T><<<1, 256, 0, st>>>((int)(m - i), a + i + i * lda, a + row + i * lda, tau + i);
        RNPGPU_CHECK_LAUNCH();
        if (i + 1 < n) {
            int rc = larf_launch<T>(true, (int)(m - i), (int)(n - i - 1), a + i + i * lda, tau + i, true, a + i + (i + 1) * lda, lda, work, st);
            if (rc) return rc;
        }
    }
    return kOk;
}

// ---------------------------------------------------------------------------
// T factors of all reflector blocks of a call (GenerateBlockTr "F","C" for
// every block, RNP/LA/Reflector.hpp:580-626): the Gram matrices of all blocks
// in one launch (row chunks of every block in parallel), then the
// recurrence for all blocks in one launch.
// ---------------------------------------------------------------------------
inline int gram_splits(size_t rows, size_t nblk, int scap, int min_rows) {
    size_t s = std::min<size_t>((size_t)std::max(scap, 1), std::max<size_t>(1, (rows + min_rows - 1) / (size_t)min_rows));
    s = std::min<size_t>(s, std::max<size_t>(1, 4096 / std::max<size_t>(nblk, 1)));
    return (int)std::max<size_t>(s, 1);
}
template <class T> size_t gram_bytes(size_t rows, size_t nblk, int scap) {
    return (nblk * (size_t)gram_splits(rows, nblk, scap, 2 * split_min_rows<T>()) * kPanelMaxCols * kPanelMaxCols * sizeof(T) + 255) / 256 * 256;
}
template <class T> int build_all_t(size_t rows, size_t k, const T *a, size_t lda, const T *tau, T *Tout, T *Pg, int scap, cudaStream_t st) {
    const size_t nblk = (k + kPanelMaxCols - 1) / kPanelMaxCols;
    if (nblk == 0) return kOk;
    const int S = gram_splits(rows, nblk, scap, 2 * split_min_rows<T>());
    const int chunk = (int)((rows + S - 1) / S);
    KScope ks("larft_all", st);
    k_gram_blocks<T><<<dim3((unsigned)S, (unsigned)nblk), 256, 0, st>>>(a, lda, (int)rows, (int)k, chunk, Pg);
    RNPGPU_CHECK_LAUNCH();
    k_build_t<T><<<(unsigned)nblk, kBuildTThreads, 0, st>>>(Pg, (size_t)kPanelMaxCols * kPanelMaxCols, (size_t)S * kPanelMaxCols * kPanelMaxCols, S, tau, kPanelMaxCols, (int)k,
                                                           Tout, (size_t)kPanelMaxCols * kPanelMaxCols, kPanelMaxCols);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

// ---------------------------------------------------------------------------
// Thin left MultQ in one cooperative launch (multq_thin.cuh)
// ---------------------------------------------------------------------------
struct ThinPlan {
    bool dyn;
    bool csmem;
    int vbuf;
    int grid, rows;
    size_t smem;
};
constexpr size_t kThinSmemMax = 200 * 1024;

template <class T> size_t thin_ws_bytes(size_t n) {
    const int G = std::max(1, device_facts().sm_count);
    return ((size_t)(G + 1) * kPanelMaxCols * n * sizeof(T) + 255) / 256 * 256 + 1024;
}
// C's rows and two V staging buffers in shared memory when they fit, then one
// buffer, then C alone, then neither
template <class T> ThinPlan thin_plan(size_t m, size_t n, size_t k) {
    ThinPlan tp;
    const int sms = std::max(1, device_facts().sm_count);
    // reflectors covering a quarter of the rows or more: re-split the active
    // rows over all blocks for every reflector block (k_multq_thin_dyn)
    tp.dyn = false;
    if (k * 4 >= m && k > (size_t)kPanelMaxCols) {
        const int grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)sms, m / 4));
        const int rows = (int)((m + grid - 1) / grid);
        const size_t smem = thin_dyn_smem_bytes<T>(rows, (int)n);
        if (smem <= kThinSmemMax) {
            tp.dyn = true;
            tp.grid = grid;
            tp.rows = rows;
            tp.csmem = false;
            tp.vbuf = 0;
            tp.smem = smem;
            return tp;
        }
    }
    tp.grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)sms, (m + 31) / 32));
    tp.rows = (int)((m + tp.grid - 1) / tp.grid);
    static const int modes[4][2] = {{1, 2}, {1, 1}, {1, 0}, {0, 0}};
    for (int q = 0; q < 4; ++q) {
        tp.csmem = modes[q][0] != 0;
        tp.vbuf = modes[q][1];
        tp.smem = thin_smem_bytes<T>(tp.rows, (int)n, tp.csmem, tp.vbuf);
        if (tp.smem <= kThinSmemMax) break;
    }
    return tp;
}
template <class T, bool CS, int VB> const void *thin_kernel() { return (const void *)k_multq_thin<T, CS, VB>; }
template <class T> int multq_thin(bool notran, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *Tf, T *c, size_t ldc, void *ws, cudaStream_t st) {
    const ThinPlan tp = thin_plan<T>(m, n, k);
    const void *kern = tp.dyn ? (const void *)k_multq_thin_dyn<T>
                              : tp.csmem ? (tp.vbuf == 2 ? thin_kernel<T, true, 2>() : tp.vbuf == 1 ? thin_kernel<T, true, 1>() : thin_kernel<T, true, 0>()) : thin_kernel<T, false, 0>();
    if (int rc = kernel_attr(kern, (int)kThinSmemMax)) return rc;
    Carver cv(ws);
    ThinArgs<T> p;
    p.A = a; p.lda = lda; p.Tf = Tf; p.C = c; p.ldc = ldc;
    p.m = (int)m; p.n = (int)n; p.k = (int)k;
    p.nblk = (int)((k + kPanelMaxCols - 1) / kPanelMaxCols);
    p.forward = notran ? 0 : 1;
    p.part = cv.take<T>((size_t)tp.grid * kPanelMaxCols * n);
    p.wred = cv.take<T>((size_t)kPanelMaxCols * n);
    unsigned *sync = cv.take<unsigned>(2);
    p.counter = sync;
    p.err = (int *)(sync + 1);
    p.status = device_status_ptr();
    p.rows_per_cta = tp.rows;
    RNPGPU_CHECK(cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), st));
    void *args[] = {&p};
    KScope ks("multq_thin", st);
    return coop_launch("k_multq_thin", kern, tp.grid, kThinThreads, args, tp.smem, st);
}

// Q^T C with wide reflector blocks (k_qtc_blocks): C is m x n FP32 with n at
// most kQtcMaxCols, the first nwide 128-column blocks of the reflectors have
// their T in t128, the rest are 32-column panels with their T in Tf.
inline size_t qtc_ws_bytes(size_t n) {
    const int G = std::max(1, device_facts().sm_count);
    const size_t nq = (n + 3) / 4 * 4;
    return ((size_t)(G + 1) * kQtcMaxW * nq * sizeof(float) + 255) / 256 * 256 + 1024;
}
inline int qtc_rows(size_t m) {
    const int G = std::max(1, device_facts().sm_count);
    return (int)(((m + G - 1) / G + 3) / 4 * 4);
}
inline bool qtc_usable(size_t m, size_t n, size_t k, const float *a, size_t lda, int nwide) {
    if (nwide <= 0 || n == 0 || n > (size_t)kQtcMaxCols || k > m || m > (size_t)INT32_MAX / 2) return false;
    if (device_facts().sm_count > 256) return false;  // the cross-block sum keeps 8 partials per lane
    if (((uintptr_t)a % 16) != 0 || lda % 4 != 0 || m % 4 != 0) return false;
    if ((size_t)nwide * kQtcMaxW > k) return false;
    return qtc_smem_bytes(qtc_rows(m), (int)((n + 3) / 4 * 4)) <= kQtcSmemMax;
}
inline int qtc_blocks(size_t m, size_t n, size_t k, const float *a, size_t lda, const float *Tf, const float *t128, int nwide, float *c, size_t ldc, void *ws, cudaStream_t st) {
    const int G = std::max(1, device_facts().sm_count);
    const int R = qtc_rows(m), nq = (int)((n + 3) / 4 * 4);
    const size_t smem = qtc_smem_bytes(R, nq);
    const void *kern = (const void *)k_qtc_blocks<0>;
    if (int rc = kernel_attr(kern, (int)kQtcSmemMax)) return rc;
    Carver cv(ws);
    QtcArgs p;
    p.A = a; p.lda = lda; p.Tf = Tf; p.T128 = t128; p.C = c; p.ldc = ldc;
    p.m = (int)m; p.n = (int)n; p.k = (int)k; p.nwide = nwide;
    p.part = cv.take<float>((size_t)G * kQtcMaxW * nq);
    p.wred = cv.take<float>((size_t)kQtcMaxW * nq);
    unsigned *sync = cv.take<unsigned>(2);
    p.counter = sync;
    p.err = (int *)(sync + 1);
    p.status = device_status_ptr();
    p.rows_per_cta = R;
    RNPGPU_CHECK(cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), st));
    void *args[] = {&p};
    KScope ks("multq_thin", st);
    return coop_launch("k_qtc_blocks", kern, G, kThinThreads, args, smem, st);
}

// C -= V (T^T (V^T C)) for a K <= 32 column block reflector and an FP32 C of
// at most kA32MaxCols columns in one launch (k_apply32); false when the shapes
// or the workspace do not suit it.  ws: the block-apply workspace (its
// partial buffer and W buffer hold the partials, the sum and the barrier).
inline bool a32_usable(int M, int N, int K, const float *V, size_t ldv, const float *C, size_t ldc, const BlockWs<float> &ws, size_t p_floats, size_t w_floats) {
    const int G = std::max(1, device_facts().sm_count);
    if (N <= 0 || N > kA32MaxCols || N % 4 != 0 || K <= 0 || K > kPanelMaxCols || M % 4 != 0 || M < 4096 || G > 256) return false;
    if (((uintptr_t)V % 16) != 0 || ((uintptr_t)C % 16) != 0 || ldv % 4 != 0 || ldc % 4 != 0) return false;
    if ((size_t)G * kPanelMaxCols * N > p_floats || (size_t)kPanelMaxCols * N + 64 > w_floats || ws.P == nullptr || ws.W == nullptr) return false;
    return a32_smem_bytes(qtc_rows((size_t)M), N) <= kQtcSmemMax;
}
inline int apply32(int M, int N, int K, const float *V, size_t ldv, const float *Tm, float *C, size_t ldc, const BlockWs<float> &ws, cudaStream_t st) {
    const int G = std::max(1, device_facts().sm_count);
    const int R = qtc_rows((size_t)M);
    const void *kern = (const void *)k_apply32<0>;
    if (int rc = kernel_attr(kern, (int)kQtcSmemMax)) return rc;
    A32Args p;
    p.V = V; p.ldv = ldv; p.T = Tm; p.C = C; p.ldc = ldc;
    p.M = M; p.N = N; p.K = K;
    p.part = ws.P;
    p.wred = ws.W;
    unsigned *sync = reinterpret_cast<unsigned *>(ws.W + (size_t)kPanelMaxCols * N + 32);
    p.counter = sync;
    p.err = (int *)(sync + 1);
    p.status = device_status_ptr();
    p.rows_per_cta = R;
    RNPGPU_CHECK(cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), st));
    void *args[] = {&p};
    KScope ks("larfb_update", st);
    return coop_launch("k_apply32", kern, G, kThinThreads, args, a32_smem_bytes(R, N), st);
}

// ---------------------------------------------------------------------------
// MultQ (unmqr): RNP/LA/QR.hpp:337-429.  The T factors of all blocks are
// built once per call (or taken from the factorization) and kept in the
// workspace.  A thin C on the left (at most kThinMaxCols columns) goes
// through the one-launch kernel; otherwise every block is one ApplyBlock.
// ---------------------------------------------------------------------------
template <class T> int unm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, T *work);

template <class T> size_t unmqr_bytes(size_t nq, size_t nw, size_t k, int smax, int sgram) {
    const size_t nblk = (k + GpuTuning::nb - 1) / GpuTuning::nb;
    size_t uni = std::max(block_ws_bytes<T>((int)nw, smax), gram_bytes<T>(nq, nblk, sgram));
    if (nw <= (size_t)kThinMaxCols) uni = std::max(uni, thin_ws_bytes<T>(nw));
    return nblk * t_bytes<T>() + uni;
}

// Tcache (optional): the T factors of the reflector blocks as stored by
// geqrf(..., Tstore); when given they are not rebuilt.
template <class T> int unmqr(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, size_t *lwork, T *work, const T *Tcache = nullptr) {
    if (side == nullptr) return -1;
    if (trans == nullptr) return -2;
    if (lwork == nullptr) return -11;
    if (m == 0 || n == 0 || k == 0) return kOk;
    const bool left = (side[0] == 'L'), notran = (trans[0] == 'N');
    const size_t nq = left ? m : n, nw = left ? n : m;
    if (k > nq) return -5;
    if (lda < std::max<size_t>(1, nq)) return -7;
    if (ldc < std::max<size_t>(1, m)) return -10;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -3;
    int smax = smax_for<T>(nq);
    int sgram = smax_for<T>(nq);
    if (work == nullptr || *lwork == 0) {
        *lwork = elems_for<T>(unmqr_bytes<T>(nq, nw, k, smax, sgram));
        return kOk;
    }
    if (a == nullptr) return -6;
    if (tau == nullptr) return -8;
    if (c == nullptr) return -9;
    while ((smax > 1 || sgram > 1) && elems_for<T>(unmqr_bytes<T>(nq, nw, k, smax, sgram)) > *lwork) {
        smax = std::max(1, smax / 2);
        sgram = std::max(1, sgram / 2);
    }
    const bool thin = left && n <= (size_t)kThinMaxCols;
    if (elems_for<T>(unmqr_bytes<T>(nq, nw, k, smax, sgram)) > *lwork) {
        if (*lwork < nw) return -11;
        return unm2r<T>(side, trans, m, n, k, a, lda, tau, c, ldc, work);
    }
    cudaStream_t st = current_stream();
    Carver cv(work);
    const size_t nb = GpuTuning::nb;
    const size_t nblk = (k + nb - 1) / nb;
    T *Tc = cv.take<T>(nblk * kPanelMaxCols * kPanelMaxCols);
    // one region shared by the Gram partials (used first) and the apply workspace
    const size_t mark = cv.off;
    T *Pg = cv.take<T>(gram_bytes<T>(nq, nblk, sgram) / sizeof(T));
    cv.off = mark;
    int rc;
    if (Tcache == nullptr && (rc = build_all_t<T>(nq, k, a, lda, tau, Tc, Pg, sgram, st))) return rc;
    const T *Tuse = Tcache ? Tcache : Tc;
    if (thin) return multq_thin<T>(notran, m, n, k, a, lda, Tuse, c, ldc, cv.take<T>(0), st);
    BlockWs<T> bw = carve_block<T>(cv, (int)nw, smax);
    const bool forward = (left && !notran) || (!left && notran);
    for (size_t s = 0; s < nblk; ++s) {
        const size_t b = forward ? s : nblk - 1 - s;
        const size_t i = b * nb;
        const int ib = (int)std::min(nb, k - i);
        const T *V = a + i + i * lda;
        const T *Tb = Tuse + b * kPanelMaxCols * kPanelMaxCols;
        if (left) rc = apply_block<T>(true, notran, (int)(m - i), (int)n, ib, V, lda, Tb, kPanelMaxCols, c + i, ldc, bw, st);
        else rc = apply_block<T>(false, notran, (int)m, (int)(n - i), ib, V, lda, Tb, kPanelMaxCols, c + i * ldc, ldc, bw, st);
        if (rc) return rc;
    }
    return kOk;
}

// MultQ_unblocked (unm2r): RNP/LA/QR.hpp:234-298
template <class T> int unm2r(const char *side, const char *trans, size_t m, size_t n, size_t k, const T *a, size_t lda, const T *tau, T *c, size_t ldc, T *work) {
    if (side == nullptr) return -1;
    if (trans == nullptr) return -2;
    if (m < 1 || n < 1 || k < 1) return kOk;
    const bool left = (side[0] == 'L'), notran = (trans[0] == 'N');
    const size_t nq = left ? m : n;
    if (k > nq) return -5;
    if (lda < std::max<size_t>(1, nq)) return -7;
    if (ldc < std::max<size_t>(1, m)) return -10;
    if (a == nullptr) return -6;
    if (tau == nullptr) return -8;
    if (c == nullptr) return -9;
    if (work == nullptr) return -11;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -3;
    cudaStream_t st = current_stream();
    const bool forward = (left && !notran) || (!left && notran);
    for (size_t s = 0; s < k; ++s) {
        const size_t i = forward ? s : k - 1 - s;
        int rc;
        if (left) rc = larf_launch<T>(true, (int)(m - i), (int)n, a + i + i * lda, tau + i, !notran, c + i, ldc, work, st);
        else rc = larf_launch<T>(false, (int)m, (int)(n - i), a + i + i * lda, tau + i, !notran, c + i * ldc, ldc, work, st);
        if (rc) return rc;
    }
    return kOk;
}

// ---------------------------------------------------------------------------
// GenerateQ (ungqr): RNP/LA/QR.hpp:509-570.  Blocks are processed backwards;
// block i is applied to the columns to its right (ApplyBlock "L","N") and
// its own columns become  I - V (T V1^H).
// ---------------------------------------------------------------------------
template <class T> int ung2r(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work);

template <class T> size_t ungqr_bytes(size_t m, size_t n, size_t k, int smax, int sgram) {
    const size_t nblk = (k + GpuTuning::nb - 1) / GpuTuning::nb;
    return (nblk + 1) * t_bytes<T>() + std::max(gram_bytes<T>(m, nblk, sgram), block_ws_bytes<T>((int)n, smax));
}

template <class T> int ungqr(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, size_t *lwork, T *work) {
    if (lwork == nullptr) return -7;
    if (n == 0) return kOk;
    if (k > n) return -3;
    if (n > m) return -2;
    if (lda < std::max<size_t>(1, m)) return -5;
    if (m > (size_t)INT32_MAX) return -1;
    int smax = smax_for<T>(m), sgram = smax_for<T>(m);
    if (work == nullptr || *lwork == 0) {
        *lwork = elems_for<T>(ungqr_bytes<T>(m, n, k, smax, sgram));
        return kOk;
    }
    if (a == nullptr) return -4;
    if (tau == nullptr && k > 0) return -6;
    while ((smax > 1 || sgram > 1) && elems_for<T>(ungqr_bytes<T>(m, n, k, smax, sgram)) > *lwork) {
        smax = std::max(1, smax / 2);
        sgram = std::max(1, sgram / 2);
    }
    if (elems_for<T>(ungqr_bytes<T>(m, n, k, smax, sgram)) > *lwork) {
        if (*lwork < n) return -7;
        return ung2r<T>(m, n, k, a, lda, tau, work);
    }
    cudaStream_t st = current_stream();
    Carver cv(work);
    const size_t nb = GpuTuning::nb;
    const size_t nblk = (k + nb - 1) / nb;
    T *Tall = cv.take<T>(nblk * kPanelMaxCols * kPanelMaxCols);
    T *Y = cv.take<T>((size_t)kPanelMaxCols * kPanelMaxCols);
    // the Gram partials (used first) and the block workspace share one region
    const size_t mark = cv.off;
    T *Pg = cv.take<T>(gram_bytes<T>(m, nblk, sgram) / sizeof(T));
    cv.off = mark;
    BlockWs<T> bw = carve_block<T>(cv, (int)n, smax);
    if (k < n) {
        dim3 grid((unsigned)std::min<size_t>((m + 255) / 256, 1024), (unsigned)std::min<size_t>(n - k, 65535));
        k_identity_cols<T><<<grid, 256, 0, st>>>((int)m, (int)k, (int)n, a, lda);
        RNPGPU_CHECK_LAUNCH();
    }
    // T of every block from the untouched reflectors, before any is overwritten
    int rc = build_all_t<T>(m, k, a, lda, tau, Tall, Pg, sgram, st);
    if (rc) return rc;
    for (size_t s = 0; s < nblk; ++s) {
        const size_t b = nblk - 1 - s;
        const size_t i = b * nb;
        const int ib = (int)std::min(nb, k - i);
        T *V = a + i + i * lda;
        const T *Tm = Tall + b * kPanelMaxCols * kPanelMaxCols;
        if (i + ib < n) {
            rc = apply_block<T>(true, true, (int)(m - i), (int)(n - i - ib), ib, V, lda, Tm, kPanelMaxCols, a + i + (i + ib) * lda, lda, bw, st);
            if (rc) return rc;
        }
        k_t_v1h<T><<<(unsigned)ib, kPanelMaxCols, 0, st>>>(Tm, kPanelMaxCols, V, lda, ib, Y, kPanelMaxCols);
        RNPGPU_CHECK_LAUNCH();
        // V block columns <- I - V Y  (in place: each thread block owns whole rows)
        GemmArgs<T> g = gemm_args<T>(V, lda, kOpN, 1, Y, (size_t)kPanelMaxCols, kOpN, 0, V, lda, (int)(m - i), ib, ib, T(-1), kBetaIdentity);
        if ((rc = launch_gemm(g, 1, st))) return rc;
        if (i > 0) {
            dim3 grid((unsigned)std::min<size_t>((i + 255) / 256, 1024), (unsigned)ib);
            k_zero_rows<T><<<grid, 256, 0, st>>>((int)i, (int)i, (int)i + ib, a, lda);
            RNPGPU_CHECK_LAUNCH();
        }
    }
    return kOk;
}

// GenerateQ_unblocked (ung2r): RNP/LA/QR.hpp:451-485
template <class T> int ung2r(size_t m, size_t n, size_t k, T *a, size_t lda, const T *tau, T *work) {
    if (n < 1) return kOk;
    if (k > n) return -3;
    if (n > m) return -2;
    if (lda < std::max<size_t>(1, m)) return -5;
    if (a == nullptr) return -4;
    if (tau == nullptr && k > 0) return -6;
    if (work == nullptr && n > 1) return -7;
    if (m > (size_t)INT32_MAX) return -1;
    cudaStream_t st = current_stream();
    if (k < n) {
        dim3 grid((unsigned)std::min<size_t>((m + 255) / 256, 1024), (unsigned)std::min<size_t>(n - k, 65535));
        k_identity_cols<T><<<grid, 256, 0, st>>>((int)m, (int)k, (int)n, a, lda);
        RNPGPU_CHECK_LAUNCH();
    }
    for (size_t s = 0; s < k; ++s) {
        const size_t i = k - 1 - s;
        if (i + 1 < n) {
            int rc = larf_launch<T>(true, (int)(m - i), (int)(n - i - 1), a + i + i * lda, tau + i, false, a + i + (i + 1) * lda, lda, work, st);
            if (rc) return rc;
        }
        k_ung2r_col<T><<<(unsigned)std::min<size_t>((m + 255) / 256, 1024), 256, 0, st>>>((int)m, (int)i, a, lda, tau);
        RNPGPU_CHECK_LAUNCH();
    }
    return kOk;
}

} // namespace rnpgpu
