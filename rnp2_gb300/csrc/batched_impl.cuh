// batched_impl.cuh — batched QR and least-squares plans: size-class launch
// helpers and the per-type run, tune and solve templates shared by the
// per-type translation units (batched_s/d/c/z.cu).
#pragma once
#include "batched_ls.cuh"
#include "qr_driver.cuh"
#include "../../include/rnp_gpu/batched_gb300.h"

#include <algorithm>
#include <vector>

namespace rnpgpu {

// size classes: class 0 holds matrices with m, n <= 32 (a warp per matrix,
// or a small block), classes 1..3 those with m <= 64, 256, 512 (a block per
// matrix staging kClassMR[c] rows)
constexpr int kClasses = 4;
constexpr int kClassRows[kClasses] = {32, 64, 256, 512};
constexpr int kClassMR[kClasses] = {64, 64, 256, 512};
inline int class_of(int m, int n) {
    if (m <= kWarpRows && n <= kWarpRows) return 0;
    if (m <= 64) return 1;
    return m <= 256 ? 2 : 3;
}

struct BatchConfig {
    int threads, nb;  // threads == 32: one warp per matrix (k_geqrf_warp)
};
// candidate block shapes (threads, panel width) per class
static const BatchConfig kCandidates[kClasses][4] = {
    {{32, 0}, {64, 8}, {0, 0}, {0, 0}},
    {{64, 8}, {128, 8}, {128, 16}, {0, 0}},
    {{128, 8}, {128, 16}, {256, 16}, {256, 32}},
    {{256, 8}, {256, 16}, {512, 16}, {0, 0}},
};
static const BatchConfig kDefaults[kClasses] = {{32, 0}, {64, 8}, {256, 16}, {256, 8}};
constexpr int kWarpsPerBlock = 4;

template <int MR> constexpr int tile_for() { return MR >= 512 ? 16 : 32; }

template <class T, int NT, int NB, int MR> int launch_batched_cfg(const BatchDesc *desc, int count, T *A, T *tau, unsigned *queue, cudaStream_t st) {
    typedef BatchSmem<T, NB, MR, tile_for<MR>()> L;
    const void *kern = (const void *)k_geqrf_batched<T, NT, NB, MR, tile_for<MR>()>;
    if (int rc = kernel_attr(kern, (int)L::kBytes)) return rc;
    const int per_sm = kernel_blocks_per_sm(kern, NT, L::kBytes);
    const int grid = std::max(1, std::min(count, device_facts().sm_count * per_sm));
    KScope ks("geqrf_batched", st);
    k_geqrf_batched<T, NT, NB, MR, tile_for<MR>()><<<grid, NT, L::kBytes, st>>>(desc, count, A, tau, queue);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> int launch_batched_warp(const BatchDesc *desc, int count, T *A, T *tau, unsigned *queue, cudaStream_t st) {
    constexpr size_t smem = (size_t)kWarpsPerBlock * kWarpRows * kWarpLd * sizeof(T);
    const void *kern = (const void *)k_geqrf_warp<T, kWarpsPerBlock>;
    if (int rc = kernel_attr(kern, (int)smem)) return rc;
    const int per_sm = kernel_blocks_per_sm(kern, kWarpsPerBlock * 32, smem);
    const int blocks = (count + kWarpsPerBlock - 1) / kWarpsPerBlock;
    const int grid = std::max(1, std::min(blocks, device_facts().sm_count * per_sm));
    KScope ks("geqrf_batched", st);
    k_geqrf_warp<T, kWarpsPerBlock><<<grid, kWarpsPerBlock * 32, smem, st>>>(desc, count, A, tau, queue);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> size_t batched_smem(int cls, BatchConfig cfg) {
    if (cfg.threads == 32) return (size_t)kWarpsPerBlock * kWarpRows * kWarpLd * sizeof(T);
    const int mr = kClassMR[cls], tile = mr >= 512 ? 16 : 32;
    return ((size_t)mr * cfg.nb + (size_t)mr * tile + (size_t)tile * cfg.nb + (size_t)cfg.nb * cfg.nb + 2 * (size_t)cfg.nb + (size_t)mr) * sizeof(T);
}
inline bool fits_smem(size_t bytes) {
    static int optin = 0;
    if (optin == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || optin <= 0) optin = 48 * 1024;
    }
    return bytes + 2048 <= (size_t)optin;
}

template <class T> int launch_batched(int cls, BatchConfig cfg, const BatchDesc *desc, int count, T *A, T *tau, unsigned *queue, cudaStream_t st) {
    if (count <= 0) return kOk;
    if (cls == 0 && cfg.threads == 32) return launch_batched_warp<T>(desc, count, A, tau, queue, st);
    if (!fits_smem(batched_smem<T>(cls, cfg))) cfg = BatchConfig{cfg.threads, 8};
    const int t = cfg.threads, nb = cfg.nb;
    if (cls <= 1) {
        if (t == 128 && nb == 8) return launch_batched_cfg<T, 128, 8, 64>(desc, count, A, tau, queue, st);
        if (t == 128 && nb == 16) return launch_batched_cfg<T, 128, 16, 64>(desc, count, A, tau, queue, st);
        return launch_batched_cfg<T, 64, 8, 64>(desc, count, A, tau, queue, st);
    }
    if (cls == 2) {
        if (t == 128 && nb == 8) return launch_batched_cfg<T, 128, 8, 256>(desc, count, A, tau, queue, st);
        if (t == 128 && nb == 16) return launch_batched_cfg<T, 128, 16, 256>(desc, count, A, tau, queue, st);
        if (t == 256 && nb == 32) return launch_batched_cfg<T, 256, 32, 256>(desc, count, A, tau, queue, st);
        if (t == 256 && nb == 8) return launch_batched_cfg<T, 256, 8, 256>(desc, count, A, tau, queue, st);
        return launch_batched_cfg<T, 256, 16, 256>(desc, count, A, tau, queue, st);
    }
    if (t == 256 && nb == 16) return launch_batched_cfg<T, 256, 16, 512>(desc, count, A, tau, queue, st);
    if (t == 512 && nb == 16) return launch_batched_cfg<T, 512, 16, 512>(desc, count, A, tau, queue, st);
    return launch_batched_cfg<T, 256, 8, 512>(desc, count, A, tau, queue, st);
}

// one warp per problem for the least-squares solves; MT = rows / 32 per lane
template <class TH, class TL, int MT> int launch_ls_cls(LsBatchArgs<TH, TL> q, cudaStream_t st) {
    const int per_sm = kernel_blocks_per_sm((const void *)k_ls_batched<TH, TL, MT>, 256, 0);
    const int warps = device_facts().sm_count * per_sm * 8;
    const int grid = std::max(1, (std::min(q.count, warps) + 7) / 8);
    KScope ks(q.refine ? "ls_refine_batched" : "ls_solve_batched", st);
    k_ls_batched<TH, TL, MT><<<grid, 256, 0, st>>>(q);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}
template <class TH, class TL> int launch_ls(int cls, const LsBatchArgs<TH, TL> &q, cudaStream_t st) {
    if (q.count <= 0) return kOk;
    if (cls == 0) return launch_ls_cls<TH, TL, 1>(q, st);
    if (cls == 1) return launch_ls_cls<TH, TL, 2>(q, st);
    if (cls == 2) return launch_ls_cls<TH, TL, 8>(q, st);
    return launch_ls_cls<TH, TL, 16>(q, st);
}

} // namespace rnpgpu

struct rnpgpu_batch_plan {
    int type;                                   // 0 s, 1 d, 2 c, 3 z
    int batch;
    int nclass[rnpgpu::kClasses];               // matrices per class
    int first[rnpgpu::kClasses];                // first descriptor of each class
    rnpgpu::BatchConfig cfg[rnpgpu::kClasses];
    long long a_extent, tau_extent;             // elements spanned by the packed a and tau
    rnpgpu::BatchDesc *d_desc;                  // device, sorted by class, then by cost
    unsigned *d_queue;                          // 2 * kClasses work-queue counters
    std::vector<rnpgpu::BatchDesc> host;        // same order as d_desc
    cudaStream_t side[rnpgpu::kClasses - 1];    // streams of classes 0 .. kClasses-2
    cudaEvent_t fork, join[rnpgpu::kClasses - 1];
};

namespace rnpgpu {

// Runs body(cls, stream) for every non-empty class: the largest class on the
// caller's stream, the others on the plan's side streams, joined back.
template <class F> int for_classes(const rnpgpu_batch_plan *p, F body) {
    using namespace rnpgpu;
    cudaStream_t st = current_stream();
    RNPGPU_CHECK(cudaEventRecord(p->fork, st));
    for (int c = 0; c < kClasses - 1; ++c) {
        if (p->nclass[c] == 0) continue;
        RNPGPU_CHECK(cudaStreamWaitEvent(p->side[c], p->fork, 0));
        int rc = body(c, p->side[c]);
        if (rc) return rc;
        RNPGPU_CHECK(cudaEventRecord(p->join[c], p->side[c]));
    }
    if (p->nclass[kClasses - 1] > 0) {
        int rc = body(kClasses - 1, st);
        if (rc) return rc;
    }
    for (int c = 0; c < kClasses - 1; ++c)
        if (p->nclass[c] > 0) RNPGPU_CHECK(cudaStreamWaitEvent(st, p->join[c], 0));
    return kOk;
}

template <class T> int plan_run(const rnpgpu_batch_plan *p, T *a, T *tau) {
    using namespace rnpgpu;
    if (p == nullptr) return -1;
    if (p->batch == 0) return kOk;
    if (a == nullptr) return -2;
    if (tau == nullptr) return -3;
    RNPGPU_CHECK(cudaMemsetAsync(p->d_queue, 0, kClasses * sizeof(unsigned), current_stream()));
    return for_classes(p, [&](int c, cudaStream_t s) { return launch_batched<T>(c, p->cfg[c], p->d_desc + p->first[c], p->nclass[c], a, tau, p->d_queue + c, s); });
}

// Autotuner: every candidate block shape is timed on each class (on the
// caller's scratch copy of the batch, which it overwrites) and the fastest
// is kept in the plan.
template <class T> int plan_tune(rnpgpu_batch_plan *p, T *a, T *tau, double *ms_out) {
    using namespace rnpgpu;
    if (p == nullptr) return -1;
    if (a == nullptr) return -2;
    if (tau == nullptr) return -3;
    cudaStream_t st = current_stream();
    cudaEvent_t e0, e1;
    RNPGPU_CHECK(cudaEventCreate(&e0));
    RNPGPU_CHECK(cudaEventCreate(&e1));
    double total = 0.0;
    for (int cls = 0; cls < kClasses; ++cls) {
        const int cnt = p->nclass[cls];
        if (cnt == 0) continue;
        const BatchDesc *dd = p->d_desc + p->first[cls];
        float best = 1e30f;
        BatchConfig bestc = p->cfg[cls];
        for (const BatchConfig &c : kCandidates[cls]) {
            if (c.threads == 0) continue;
            if (!fits_smem(batched_smem<T>(cls, c))) continue;
            float tmin = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {
                RNPGPU_CHECK(cudaMemsetAsync(p->d_queue + cls, 0, sizeof(unsigned), st));
                RNPGPU_CHECK(cudaEventRecord(e0, st));
                int rc = launch_batched<T>(cls, c, dd, cnt, a, tau, p->d_queue + cls, st);
                if (rc) return rc;
                RNPGPU_CHECK(cudaEventRecord(e1, st));
                RNPGPU_CHECK(cudaEventSynchronize(e1));
                float ms = 0.f;
                RNPGPU_CHECK(cudaEventElapsedTime(&ms, e0, e1));
                tmin = std::min(tmin, ms);
            }
            if (tmin < best) {
                best = tmin;
                bestc = c;
            }
        }
        p->cfg[cls] = bestc;
        total += best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_out) *ms_out = total;
    return kOk;
}

// plain batched least squares in the plan's precision: factor in place, then
// one warp per problem forms x = R^{-1} (Q^H b)(0:n)
template <class T> int plan_gels(const rnpgpu_batch_plan *p, T *a, T *tau, const T *b, T *x) {
    using namespace rnpgpu;
    if (p == nullptr) return -1;
    if (p->batch == 0) return kOk;
    if (b == nullptr) return -4;
    if (x == nullptr) return -5;
    for (const BatchDesc &d : p->host)
        if (d.m < d.n) return -1;
    int rc = plan_run<T>(p, a, tau);
    if (rc) return rc;
    RNPGPU_CHECK(cudaMemsetAsync(p->d_queue + kClasses, 0, kClasses * sizeof(unsigned), current_stream()));
    return for_classes(p, [&](int c, cudaStream_t s) {
        LsBatchArgs<T, T> q;
        q.desc = p->d_desc + p->first[c];
        q.count = p->nclass[c];
        q.A = nullptr;
        q.F = a;
        q.tau = tau;
        q.B = b;
        q.X = x;
        q.refine = 0;
        q.max_iter = 0;
        q.iters = nullptr;
        q.berr = nullptr;
        q.eta = nullptr;
        q.queue = p->d_queue + kClasses + c;
        return launch_ls<T, T>(c, q, s);
    });
}

// mixed batched least squares: the low-precision copy of every problem is
// factored in the workspace, then one warp per problem refines x in FP64
template <class TL> size_t mixed_ws_bytes(const rnpgpu_batch_plan *p) {
    return ((size_t)p->a_extent * sizeof(TL) + 255) / 256 * 256 + ((size_t)p->tau_extent * sizeof(TL) + 255) / 256 * 256 + 512;
}
template <class TH, class TL>
int plan_gels_mixed(const rnpgpu_batch_plan *p, const TH *a, const TH *b, TH *x, int max_iter, int *iters, double *berr, double *eta, void *work, size_t *lwork_bytes, bool tune, double *tune_ms) {
    using namespace rnpgpu;
    if (p == nullptr) return -1;
    if (lwork_bytes == nullptr) return -11;
    if (work == nullptr || *lwork_bytes == 0) {
        *lwork_bytes = mixed_ws_bytes<TL>(p);
        return kOk;
    }
    if (*lwork_bytes < mixed_ws_bytes<TL>(p)) return -11;
    if (p->batch == 0) return kOk;
    if (a == nullptr) return -2;
    for (const BatchDesc &d : p->host)
        if (d.m < d.n) return -1;
    Carver cv(work);
    TL *af = cv.take<TL>((size_t)p->a_extent);
    TL *tauf = cv.take<TL>((size_t)std::max<long long>(p->tau_extent, 1));
    cudaStream_t st = current_stream();
    const size_t ne = (size_t)p->a_extent;
    const unsigned cgrid = (unsigned)std::max<size_t>(1, std::min<size_t>((ne + 255) / 256, 4096));
    k_convert_flat<TH, TL><<<cgrid, 256, 0, st>>>(ne, a, af);
    RNPGPU_CHECK_LAUNCH();
    if (tune) {
        int rc = plan_tune<TL>(const_cast<rnpgpu_batch_plan *>(p), af, tauf, tune_ms);
        if (rc) return rc;
        k_convert_flat<TH, TL><<<cgrid, 256, 0, st>>>(ne, a, af);
        RNPGPU_CHECK_LAUNCH();
        return kOk;
    }
    if (b == nullptr) return -3;
    if (x == nullptr) return -4;
    int rc = plan_run<TL>(p, af, tauf);
    if (rc) return rc;
    RNPGPU_CHECK(cudaMemsetAsync(p->d_queue + kClasses, 0, kClasses * sizeof(unsigned), st));
    return for_classes(p, [&](int c, cudaStream_t s) {
        LsBatchArgs<TH, TL> q;
        q.desc = p->d_desc + p->first[c];
        q.count = p->nclass[c];
        q.A = a;
        q.F = af;
        q.tau = tauf;
        q.B = b;
        q.X = x;
        q.refine = 1;
        q.max_iter = max_iter > 0 ? max_iter : 10;
        q.iters = iters;
        q.berr = berr;
        q.eta = eta;
        q.queue = p->d_queue + kClasses + c;
        return launch_ls<TH, TL>(c, q, s);
    });
}

} // namespace rnpgpu
