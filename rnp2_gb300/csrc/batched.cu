// batched.cu — batched Householder QR: plans, size classes, autotuning and
// the C ABI (include/rnp_gpu/batched_gb300.h).
//
// A plan is built once per batch shape: the host splits the matrices into
// size classes (m, n <= 32: a warp per matrix; m <= 64, <= 256, <= 512: a
// block per matrix staging that many rows),
// sorts each class by decreasing cost (2mn^2 - 2n^3/3), uploads the sorted
// descriptors into the caller's workspace and keeps, per class, the block
// shape (threads, panel width) chosen by the autotuner.  A run resets the
// classes' work-queue counters and launches one persistent kernel per class,
// the classes on their own streams joined by events, so a run can be
// captured into a CUDA graph and replayed.  The least-squares entry points
// add one warp-per-problem launch per class (batched_ls.cuh).
#include "batched_impl.cuh"

namespace rnpgpu {

size_t plan_bytes(int batch) { return ((size_t)batch * sizeof(rnpgpu::BatchDesc) + 255) / 256 * 256 + 256 + 256; }

void plan_free(rnpgpu_batch_plan *p) {
    if (p == nullptr) return;
    for (int c = 0; c < rnpgpu::kClasses - 1; ++c) {
        if (p->side[c]) cudaStreamDestroy(p->side[c]);
        if (p->join[c]) cudaEventDestroy(p->join[c]);
    }
    if (p->fork) cudaEventDestroy(p->fork);
    delete p;
}

int plan_create(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_off, const long long *tau_off, const long long *b_off, const long long *x_off, void *work, size_t *lwork_bytes,
                rnpgpu_batch_plan **out) {
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
    std::vector<BatchDesc> cls[kClasses];
    long long aext = 0, text = 0;
    for (int i = 0; i < batch; ++i) {
        if (m[i] < 0 || n[i] < 0) return -3;
        if (m[i] > kBatchMaxRows) return -3;
        if (lda[i] < std::max(1, m[i])) return -5;
        if (a_off[i] < 0 || tau_off[i] < 0) return -6;
        BatchDesc d;
        d.a_off = a_off[i];
        d.tau_off = tau_off[i];
        d.b_off = b_off ? b_off[i] : 0;
        d.x_off = x_off ? x_off[i] : 0;
        d.m = m[i];
        d.n = n[i];
        d.lda = lda[i];
        d.index = i;
        aext = std::max(aext, d.a_off + (long long)d.lda * d.n);
        text = std::max(text, d.tau_off + (long long)std::min(d.m, d.n));
        const int c = class_of(m[i], n[i]);
        cls[c].push_back(d);
    }
    auto cost = [](const BatchDesc &d) {
        const double mm = d.m, nn = std::min(d.m, d.n), nc = d.n;
        return 2.0 * mm * nn * nc - nn * nn * (mm + nc) + 2.0 * nn * nn * nn / 3.0;
    };
    auto by_cost = [&](const BatchDesc &x, const BatchDesc &y) { return cost(x) > cost(y); };
    rnpgpu_batch_plan *p = new rnpgpu_batch_plan();
    p->type = type;
    p->batch = batch;
    p->a_extent = aext;
    p->tau_extent = text;
    for (int c = 0; c < kClasses; ++c) {
        std::stable_sort(cls[c].begin(), cls[c].end(), by_cost);
        p->nclass[c] = (int)cls[c].size();
        p->first[c] = (int)p->host.size();
        p->cfg[c] = kDefaults[c];
        p->host.insert(p->host.end(), cls[c].begin(), cls[c].end());
    }
    Carver cv(work);
    p->d_desc = cv.take<BatchDesc>((size_t)std::max(batch, 1));
    p->d_queue = cv.take<unsigned>(2 * kClasses);
    cudaStream_t st = current_stream();
    p->fork = nullptr;
    for (int c = 0; c < kClasses - 1; ++c) {
        p->side[c] = nullptr;
        p->join[c] = nullptr;
    }
    cudaError_t e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    for (int c = 0; c < kClasses - 1 && e == cudaSuccess; ++c) {
        e = cudaStreamCreateWithFlags(&p->side[c], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join[c], cudaEventDisableTiming);
    }
    if (e == cudaSuccess && batch > 0) e = cudaMemcpyAsync(p->d_desc, p->host.data(), (size_t)batch * sizeof(BatchDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        plan_free(p);
        return kErrCuda;
    }
    *out = p;
    return kOk;
}

} // namespace rnpgpu

using namespace rnpgpu;

extern "C" {

int rnpgpu_geqrf_batched_plan(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_offset, const long long *tau_offset, void *work, size_t *lwork_bytes, rnpgpu_batch_plan **plan) {
    if (type < 0 || type > 3) return -1;
    return plan_create(type, batch, m, n, lda, a_offset, tau_offset, nullptr, nullptr, work, lwork_bytes, plan);
}

int rnpgpu_gels_batched_plan(int type, int batch, const int *m, const int *n, const int *lda, const long long *a_offset, const long long *tau_offset, const long long *b_offset, const long long *x_offset, void *work,
                             size_t *lwork_bytes, rnpgpu_batch_plan **plan) {
    if (type < 0 || type > 3) return -1;
    if (work != nullptr && lwork_bytes != nullptr && *lwork_bytes != 0 && (b_offset == nullptr || x_offset == nullptr)) return -8;
    return plan_create(type, batch, m, n, lda, a_offset, tau_offset, b_offset, x_offset, work, lwork_bytes, plan);
}

int rnpgpu_batch_plan_destroy(rnpgpu_batch_plan *plan) {
    plan_free(plan);
    return 0;
}

int rnpgpu_batch_plan_set_config(rnpgpu_batch_plan *plan, int cls, int threads, int nb) {
    if (plan == nullptr || cls < 0 || cls >= rnpgpu::kClasses) return -1;
    for (const rnpgpu::BatchConfig &c : rnpgpu::kCandidates[cls])
        if (c.threads != 0 && c.threads == threads && c.nb == nb) {
            plan->cfg[cls] = c;
            return 0;
        }
    return -3;
}

int rnpgpu_batch_plan_config(const rnpgpu_batch_plan *plan, int cls, int *threads, int *nb, int *count) {
    if (plan == nullptr || cls < 0 || cls >= rnpgpu::kClasses) return -1;
    if (threads) *threads = plan->cfg[cls].threads;
    if (nb) *nb = plan->cfg[cls].nb;
    if (count) *count = plan->nclass[cls];
    return 0;
}

} // extern "C"
