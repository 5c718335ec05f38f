// batched_s.cu — batched QR and least squares in float precision: the C ABI entry
// points of include/rnp_gpu/batched_gb300.h for this type and the mixed
// form whose low-precision factorization runs in this type.
#include "batched_impl.cuh"

using namespace rnpgpu;

extern "C" {

#define RNPGPU_BATCHED(P, T, CT, TI)                                                                        \
    int rnpgpu_##P##geqrf_batched(const rnpgpu_batch_plan *plan, CT *a, CT *tau) {                          \
        if (plan != nullptr && plan->type != TI) return -1;                                                 \
        return plan_run<T>(plan, reinterpret_cast<T *>(a), reinterpret_cast<T *>(tau));                    \
    }                                                                                                       \
    int rnpgpu_##P##geqrf_batched_tune(rnpgpu_batch_plan *plan, CT *a, CT *tau, double *ms) {               \
        if (plan != nullptr && plan->type != TI) return -1;                                                 \
        return plan_tune<T>(plan, reinterpret_cast<T *>(a), reinterpret_cast<T *>(tau), ms);                \
    }                                                                                                       \
    int rnpgpu_##P##gels_batched(const rnpgpu_batch_plan *plan, CT *a, CT *tau, const CT *b, CT *x) {       \
        if (plan != nullptr && plan->type != TI) return -1;                                                 \
        return plan_gels<T>(plan, reinterpret_cast<T *>(a), reinterpret_cast<T *>(tau),                    \
                            reinterpret_cast<const T *>(b), reinterpret_cast<T *>(x));                      \
    }
RNPGPU_BATCHED(s, float, float, 0)

#define RNPGPU_BATCHED_MIXED(NAME, TH, TL, CT, TI)                                                                                       \
    int NAME(const rnpgpu_batch_plan *plan, const CT *a, const CT *b, CT *x, int max_iter, int *iters, double *berr, double *eta,         \
             void *work, size_t *lwork_bytes) {                                                                                          \
        if (plan != nullptr && plan->type != TI) return -1;                                                                              \
        return plan_gels_mixed<TH, TL>(plan, reinterpret_cast<const TH *>(a), reinterpret_cast<const TH *>(b), reinterpret_cast<TH *>(x), \
                                       max_iter, iters, berr, eta, work, lwork_bytes, false, nullptr);                                   \
    }                                                                                                                                    \
    int NAME##_tune(rnpgpu_batch_plan *plan, const CT *a, void *work, size_t *lwork_bytes, double *ms) {                                 \
        if (plan != nullptr && plan->type != TI) return -1;                                                                              \
        return plan_gels_mixed<TH, TL>(plan, reinterpret_cast<const TH *>(a), nullptr, nullptr, 0, nullptr, nullptr, nullptr, work,      \
                                       lwork_bytes, true, ms);                                                                           \
    }
RNPGPU_BATCHED_MIXED(rnpgpu_dsgels_batched, double, float, double, 1)

} // extern "C"
