// batched_z.cu — batched QR and least squares in complex double precision: the C ABI entry
// points of include/rnp_gpu/batched_gb300.h for this type.
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
RNPGPU_BATCHED(z, rnpgpu::cf64, rnpgpu_complex_double, 3)

} // extern "C"
