// batched.cu — batched Householder QR: plans, size classes, autotuning and
// the C ABI (include/rnp_gpu/batched_gb300.h).
//
// A plan is built once per batch shape: the host sorts the matrices by
// decreasing cost (2mn^2 - 2n^3/3), splits them into size classes (rows
// <= kSmallRows: small blocks; larger: wide blocks), uploads the sorted
// descriptors into the caller's workspace and keeps, per class, the block
// shape (threads, panel width) chosen by the autotuner.  A run resets the
// classes' work-queue counters and launches one persistent kernel per class,
// the classes on two streams joined by events, so a run can be captured into
// a CUDA graph and replayed.
#include "batched.cuh"
#include "qr_driver.cuh"
#include "../../include/rnp_gpu/batched_gb300.h"

#include <algorithm>
#include <cstdio>
#include <numeric>
#include <vector>

namespace rnpgpu {

constexpr int kSmallRows = 64;

struct BatchConfig {
    int threads, nb;
};
// candidate block shapes, per class
static const BatchConfig kCandidates[] = {{64, 8}, {128, 8}, {128, 16}, {256, 16}, {256, 32}};

template <class T, int NT, int NB> int launch_batched_cfg(const BatchDesc *desc, int count, T *A, T *tau, unsigned *queue, cudaStream_t st) {
    typedef BatchSmem<T, NB> L;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    static int per_sm = 1;
    std::call_once(once, []() {
        attr = cudaFuncSetAttribute((const void *)k_geqrf_batched<T, NT, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kBytes);
        if (attr == cudaSuccess) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_geqrf_batched<T, NT, NB>, NT, L::kBytes);
        if (per_sm < 1) per_sm = 1;
    });
    RNPGPU_CHECK(attr);
    const int grid = std::max(1, std::min(count, device_facts().sm_count * per_sm));
    KScope ks("geqrf_batched", st);
    k_geqrf_batched<T, NT, NB><<<grid, NT, L::kBytes, st>>>(desc, count, A, tau, queue);
    RNPGPU_CHECK_LAUNCH();
    return kOk;
}

template <class T> size_t batched_smem(BatchConfig cfg) {
    if (cfg.nb == 8) return BatchSmem<T, 8>::kBytes;
    if (cfg.nb == 32) return BatchSmem<T, 32>::kBytes;
    return BatchSmem<T, 16>::kBytes;
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

template <class T> int launch_batched(BatchConfig cfg, const BatchDesc *desc, int count, T *A, T *tau, unsigned *queue, cudaStream_t st) {
    if (count <= 0) return kOk;
    if (!fits_smem(batched_smem<T>(cfg))) cfg = BatchConfig{cfg.threads >= 256 ? 256 : 128, cfg.nb == 32 ? 16 : 8};
    if (cfg.threads == 64 && cfg.nb == 8) return launch_batched_cfg<T, 64, 8>(desc, count, A, tau, queue, st);
    if (cfg.threads == 128 && cfg.nb == 8) return launch_batched_cfg<T, 128, 8>(desc, count, A, tau, queue, st);
    if (cfg.threads == 128 && cfg.nb == 16) return launch_batched_cfg<T, 128, 16>(desc, count, A, tau, queue, st);
    if (cfg.threads == 256 && cfg.nb == 32) return launch_batched_cfg<T, 256, 32>(desc, count, A, tau, queue, st);
    return launch_batched_cfg<T, 256, 16>(desc, count, A, tau, queue, st);
}

} // namespace rnpgpu

struct rnpgpu_batch_plan {
    int type;                              // 0 s, 1 d, 2 c, 3 z
    int batch;
    int nclass[2];                         // matrices per class (0 small, 1 large)
    rnpgpu::BatchConfig cfg[2];
    rnpgpu::BatchDesc *d_desc;             // device, sorted: class 0 then class 1
    unsigned *d_queue;                     // two counters
    std::vector<rnpgpu::BatchDesc> host;   // same order as d_desc
    cudaStream_t side;                     // second stream for the small class
    cudaEvent_t fork, join;
};

namespace {

size_t plan_bytes(int batch) { return ((size_t)batch * sizeof(rnpgpu::BatchDesc) + 255) / 256 * 256 + 256 + 256; }

int plan_create(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_off, const long long *tau_off, void *work, size_t *lwork_bytes, rnpgpu_batch_plan **out) {
    using namespace rnpgpu;
    if (batch < 0) return -2;
    if (lwork_bytes == nullptr) return -9;
    if (work == nullptr || *lwork_bytes == 0) {
        *lwork_bytes = plan_bytes(batch);
        return kOk;
    }
    if (out == nullptr) return -10;
    if (m == nullptr || n == nullptr || lda == nullptr || a_off == nullptr || tau_off == nullptr) return -3;
    if (*lwork_bytes < plan_bytes(batch)) return -9;
    std::vector<BatchDesc> small, large;
    for (int i = 0; i < batch; ++i) {
        if (m[i] < 0 || n[i] < 0) return -3;
        if (m[i] > kBatchMaxRows) return -3;
        if (lda[i] < std::max(1, m[i])) return -5;
        BatchDesc d;
        d.a_off = a_off[i];
        d.tau_off = tau_off[i];
        d.m = m[i];
        d.n = n[i];
        d.lda = lda[i];
        d.index = i;
        (m[i] <= kSmallRows ? small : large).push_back(d);
    }
    auto cost = [](const BatchDesc &d) {
        const double mm = d.m, nn = std::min(d.m, d.n), nc = d.n;
        return 2.0 * mm * nn * nc - nn * nn * (mm + nc) + 2.0 * nn * nn * nn / 3.0;
    };
    auto by_cost = [&](const BatchDesc &x, const BatchDesc &y) { return cost(x) > cost(y); };
    std::stable_sort(small.begin(), small.end(), by_cost);
    std::stable_sort(large.begin(), large.end(), by_cost);
    rnpgpu_batch_plan *p = new rnpgpu_batch_plan();
    p->type = type;
    p->batch = batch;
    p->nclass[0] = (int)small.size();
    p->nclass[1] = (int)large.size();
    p->cfg[0] = BatchConfig{64, 8};
    p->cfg[1] = BatchConfig{256, 16};
    p->host = small;
    p->host.insert(p->host.end(), large.begin(), large.end());
    Carver cv(work);
    p->d_desc = cv.take<BatchDesc>((size_t)std::max(batch, 1));
    p->d_queue = cv.take<unsigned>(2);
    cudaStream_t st = current_stream();
    p->side = nullptr;
    p->fork = p->join = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming);
    if (e == cudaSuccess && batch > 0) e = cudaMemcpyAsync(p->d_desc, p->host.data(), (size_t)batch * sizeof(BatchDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        if (p->side) cudaStreamDestroy(p->side);
        if (p->fork) cudaEventDestroy(p->fork);
        if (p->join) cudaEventDestroy(p->join);
        delete p;
        return kErrCuda;
    }
    *out = p;
    return kOk;
}

template <class T> int plan_run(const rnpgpu_batch_plan *p, T *a, T *tau) {
    using namespace rnpgpu;
    if (p == nullptr) return -1;
    if (p->batch == 0) return kOk;
    if (a == nullptr) return -2;
    if (tau == nullptr) return -3;
    cudaStream_t st = current_stream();
    RNPGPU_CHECK(cudaMemsetAsync(p->d_queue, 0, 2 * sizeof(unsigned), st));
    // small class on the side stream, large class on the caller's stream
    RNPGPU_CHECK(cudaEventRecord(p->fork, st));
    RNPGPU_CHECK(cudaStreamWaitEvent(p->side, p->fork, 0));
    int rc = launch_batched<T>(p->cfg[0], p->d_desc, p->nclass[0], a, tau, p->d_queue, p->side);
    if (rc) return rc;
    rc = launch_batched<T>(p->cfg[1], p->d_desc + p->nclass[0], p->nclass[1], a, tau, p->d_queue + 1, st);
    if (rc) return rc;
    RNPGPU_CHECK(cudaEventRecord(p->join, p->side));
    RNPGPU_CHECK(cudaStreamWaitEvent(st, p->join, 0));
    return kOk;
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
    for (int cls = 0; cls < 2; ++cls) {
        const int cnt = p->nclass[cls];
        if (cnt == 0) continue;
        const BatchDesc *dd = p->d_desc + (cls == 0 ? 0 : p->nclass[0]);
        float best = 1e30f;
        BatchConfig bestc = p->cfg[cls];
        for (const BatchConfig &c : kCandidates) {
            if (cls == 0 && c.threads > 128) continue;
            if (!fits_smem(batched_smem<T>(c))) continue;
            float tmin = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {
                RNPGPU_CHECK(cudaMemsetAsync(p->d_queue + cls, 0, sizeof(unsigned), st));
                RNPGPU_CHECK(cudaEventRecord(e0, st));
                int rc = launch_batched<T>(c, dd, cnt, a, tau, p->d_queue + cls, st);
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

} // namespace

extern "C" {

int rnpgpu_geqrf_batched_plan(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_offset, const long long *tau_offset, void *work, size_t *lwork_bytes, rnpgpu_batch_plan **plan) {
    if (type < 0 || type > 3) return -1;
    return plan_create(type, batch, m, n, lda, a_offset, tau_offset, work, lwork_bytes, plan);
}

int rnpgpu_batch_plan_destroy(rnpgpu_batch_plan *plan) {
    if (plan == nullptr) return 0;
    if (plan->side) cudaStreamDestroy(plan->side);
    if (plan->fork) cudaEventDestroy(plan->fork);
    if (plan->join) cudaEventDestroy(plan->join);
    delete plan;
    return 0;
}

int rnpgpu_batch_plan_config(const rnpgpu_batch_plan *plan, int cls, int *threads, int *nb, int *count) {
    if (plan == nullptr || cls < 0 || cls > 1) return -1;
    if (threads) *threads = plan->cfg[cls].threads;
    if (nb) *nb = plan->cfg[cls].nb;
    if (count) *count = plan->nclass[cls];
    return 0;
}

#define RNPGPU_BATCHED(P, T, CT, TI)                                                                        \
    int rnpgpu_##P##geqrf_batched(const rnpgpu_batch_plan *plan, CT *a, CT *tau) {                          \
        if (plan != nullptr && plan->type != TI) return -1;                                                 \
        return plan_run<T>(plan, reinterpret_cast<T *>(a), reinterpret_cast<T *>(tau));                    \
    }                                                                                                       \
    int rnpgpu_##P##geqrf_batched_tune(rnpgpu_batch_plan *plan, CT *a, CT *tau, double *ms) {               \
        if (plan != nullptr && plan->type != TI) return -1;                                                 \
        return plan_tune<T>(plan, reinterpret_cast<T *>(a), reinterpret_cast<T *>(tau), ms);                \
    }
RNPGPU_BATCHED(s, float, float, 0)
RNPGPU_BATCHED(d, double, double, 1)
RNPGPU_BATCHED(c, rnpgpu::cf32, rnpgpu_complex_float, 2)
RNPGPU_BATCHED(z, rnpgpu::cf64, rnpgpu_complex_double, 3)

} // extern "C"
