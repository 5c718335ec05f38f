// qr_noalloc.cu — Factor (double) for callers that cannot allocate device memory.
//
// The regular rnpgpu_dgeqrf takes a caller-owned work block, which the caller
// must obtain with cudaMalloc (or from an allocator that calls it).  Some
// callers cannot do that: host frameworks and plugin hosts that own and
// pre-budget all device memory, or fixed-budget real-time loops where a
// cudaMalloc/cudaFree would synchronize the device or fail.  For them this
// file provides rnpgpu_dgeqrf_noalloc, which uses a fixed scratch array built
// into the library instead of a work block.
//
//  * The scratch is one file-scope __device__ array of kFactorScratchBytes
//    (8 MiB).  Every GPU that loads the library holds it until the process
//    exits.
//  * Host code cannot pass the array's name to a kernel (in host code it is a
//    host-side stand-in, not a device address).  The device address is looked
//    up with cudaGetSymbolAddress once per device, with that device current,
//    by the first call made on that device; make that first call before any
//    stream capture.
//  * Size limit: this entry point always factors in the serial order (the
//    look-ahead order of rnpgpu_dgeqrf would need a second update workspace,
//    and a side stream and two events created on first use).  Its plan needs
//    the panel records (about 120 KB on a 152-SM GPU), one 32 x 32 T factor
//    and 512 * n bytes for W, so n up to 16,000 columns (any m) always fits;
//    past about 16,100 columns the call is rejected with status -2 and a
//    message in rnpgpu_get_last_error().
//  * Every call uses the same array and leaves its contents behind.  The
//    grid-barrier counter and error word that must start at zero are cleared
//    before each panel launch; every other region is written before it is
//    read.  Calls whose work overlaps on the GPU (different streams, or
//    different host threads, without ordering between them) race on the
//    array: order them on one stream.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include "qr_driver.cuh"
#include "../../include/rnp_gpu/qr_gb300.h"

// the FP64 factorization (and every kernel it launches) is instantiated once,
// by the double unit
namespace rnpgpu {
extern template int geqrf<double>(size_t, size_t, double *, size_t, double *, size_t *, double *, double *, const CqrWs *, bool);
}

#include <cstdio>
#include <mutex>

namespace {

constexpr size_t kFactorScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_factor_scratch[kFactorScratchBytes];

constexpr int kMaxDevices = 64;
struct ScratchAddress {
    void *ptr = nullptr;
    cudaError_t err = cudaErrorUnknown;
};
static ScratchAddress g_scratch[kMaxDevices];
static std::once_flag g_scratch_once[kMaxDevices];

// Device address of g_factor_scratch on the current device (set up on the
// first call per device).
int factor_scratch(void **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        rnpgpu::set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "rnpgpu_dgeqrf_noalloc: device index out of range");
        return rnpgpu::kErrCuda;
    }
    std::call_once(g_scratch_once[dev], [dev]() {
        void *p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_factor_scratch);
        g_scratch[dev].ptr = p;
        g_scratch[dev].err = err;
    });
    if (g_scratch[dev].err != cudaSuccess || g_scratch[dev].ptr == nullptr) {
        rnpgpu::set_last_error(cudaGetErrorString(g_scratch[dev].err));
        return rnpgpu::kErrCuda;
    }
    *out = g_scratch[dev].ptr;
    return rnpgpu::kOk;
}

} // namespace

extern "C" int rnpgpu_dgeqrf_noalloc(size_t m, size_t n, double *a, size_t lda, double *tau) {
    const size_t k = m < n ? m : n;
    if (k == 0) return rnpgpu::kOk;
    if (lda < (m > 1 ? m : 1)) return -4;
    if (m > (size_t)INT32_MAX || n > (size_t)INT32_MAX) return -1;
    // the smallest serial plan (one split of W) must fit in the built-in scratch
    const size_t need = rnpgpu::elems_for<double>(rnpgpu::geqrf_serial_bytes<double>(m, n, 1)) * sizeof(double);
    if (need > kFactorScratchBytes) {
        char msg[200];
        snprintf(msg, sizeof(msg), "rnpgpu_dgeqrf_noalloc: a %zu x %zu factorization needs %zu bytes of scratch; the built-in scratch holds %zu", m, n, need, kFactorScratchBytes);
        rnpgpu::set_last_error(msg);
        return -2;
    }
    if (a == nullptr) return -3;
    if (tau == nullptr) return -5;
    void *scratch = nullptr;
    int rc = factor_scratch(&scratch);
    if (rc) return rc;
    size_t lwork = kFactorScratchBytes / sizeof(double);
    return rnpgpu::geqrf<double>(m, n, a, lda, tau, &lwork, static_cast<double *>(scratch), nullptr, nullptr, false);
}
