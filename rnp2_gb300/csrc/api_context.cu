// api_context.cu — per-thread stream and error state, device facts, and the
// library-level C ABI entry points (rnpgpu_set_stream & co.).
#include "qr_driver.cuh"
#include "../../include/rnp_gpu/qr_gb300.h"
#include <algorithm>
#include <atomic>
#include <cstring>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace rnpgpu {

static thread_local cudaStream_t t_stream = nullptr;
static thread_local std::string t_last_error;

cudaStream_t current_stream() { return t_stream; }
void set_last_error(const char *msg) { t_last_error = msg ? msg : ""; }

// ---------------------------------------------------------------------------
// launch accounting and per-kernel-class event timing
// ---------------------------------------------------------------------------
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

struct TimedLaunch {
    const char *name;
    cudaEvent_t start, stop;
};
struct KTimer {
    bool on = false;
    std::vector<TimedLaunch> done;
    std::vector<TimedLaunch> open;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
};
static thread_local KTimer t_timer;

void ktimer_begin(const char *name, cudaStream_t st) {
    if (!t_timer.on) return;
    TimedLaunch t{name, t_timer.get(), t_timer.get()};
    cudaEventRecord(t.start, st);
    t_timer.open.push_back(t);
}
void ktimer_end(cudaStream_t st) {
    if (!t_timer.on || t_timer.open.empty()) return;
    TimedLaunch t = t_timer.open.back();
    t_timer.open.pop_back();
    cudaEventRecord(t.stop, st);
    t_timer.done.push_back(t);
}

// ---------------------------------------------------------------------------
// Kernel attributes, set once per (kernel host stub, device).  nvcc gives a
// kernel's host stub internal linkage, so a kernel template that several
// units instantiate has one stub and one device copy per unit; keying on the
// stub a launch site actually uses keeps the attribute on the copy that runs.
// ---------------------------------------------------------------------------
struct AttrKey {
    const void *kern;
    int dev;
    bool operator<(const AttrKey &o) const { return kern != o.kern ? kern < o.kern : dev < o.dev; }
};
struct AttrState {
    int smem = -1;
    bool carveout = false;
    bool cluster16 = false;
};
static std::mutex g_attr_mu;
static std::map<AttrKey, AttrState> g_attr;
static std::map<std::pair<AttrKey, std::pair<int, size_t> >, int> g_occ;

int kernel_attr(const void *kern, int dyn_smem, bool max_carveout) {
    int dev = 0;
    RNPGPU_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_attr_mu);
    AttrState &a = g_attr[AttrKey{kern, dev}];
    if (dyn_smem > a.smem) {
        RNPGPU_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem));
        a.smem = dyn_smem;
    }
    if (max_carveout && !a.carveout) {
        RNPGPU_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared));
        a.carveout = true;
    }
    return kOk;
}

int kernel_blocks_per_sm(const void *kern, int threads, size_t dyn_smem) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    std::lock_guard<std::mutex> lk(g_attr_mu);
    auto key = std::make_pair(AttrKey{kern, dev}, std::make_pair(threads, dyn_smem));
    auto it = g_occ.find(key);
    if (it != g_occ.end()) return it->second;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, dyn_smem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    per_sm = std::max(per_sm, 1);
    g_occ[key] = per_sm;
    return per_sm;
}

// Largest cluster (<= 16 blocks, non-portable sizes above 8 allowed) of
// `threads` threads and `dyn_smem` bytes that the device can co-schedule for
// this kernel; 0 when none of 2 .. 16 blocks fits.  Cached per size.
static std::map<std::pair<AttrKey, std::pair<int, size_t> >, int> g_cluster;
int kernel_max_cluster(const void *kern, int threads, size_t dyn_smem, int want) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_attr_mu);
    AttrState &a = g_attr[AttrKey{kern, dev}];
    if (!a.cluster16) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        a.cluster16 = true;
    }
    auto key = std::make_pair(AttrKey{kern, dev}, std::make_pair(threads * 64 + want, dyn_smem));
    auto it = g_cluster.find(key);
    if (it != g_cluster.end()) return it->second;
    int best = 0;
    for (int c = want; c >= 2; --c) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(c);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = dyn_smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = c;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        if (n > 0) {
            best = c;
            break;
        }
    }
    g_cluster[key] = best;
    return best;
}

// ---------------------------------------------------------------------------
// TMA tensor maps (cuTensorMapEncodeTiled through the runtime's driver entry
// point: no link against the driver library)
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *, const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, []() {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// swizzle128: the box's 128-byte rows (box_rows == 32) land in shared memory
// with their 16-byte chunks XOR-permuted by the row index mod 8
int encode_map_f32(CUtensorMap *map, const float *base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols, bool swizzle128) {
    EncodeTiledFn fn = encode_tiled_fn();
    if (fn == nullptr) {
        set_last_error("cuTensorMapEncodeTiled is not available");
        return kErrCuda;
    }
    const cuuint64_t dims[2] = {rows, cols};
    const cuuint64_t strides[1] = {ld * sizeof(float)};
    const cuuint32_t box[2] = {box_rows, box_cols};
    const cuuint32_t estride[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char msg[160];
        snprintf(msg, sizeof msg, "cuTensorMapEncodeTiled failed (%d) for a %llu x %llu FP32 matrix, ld %llu, box %u x %u", (int)r, (unsigned long long)rows,
                 (unsigned long long)cols, (unsigned long long)ld, box_rows, box_cols);
        set_last_error(msg);
        return kErrCuda;
    }
    return kOk;
}

// FP64 / FP32 FMA throughput probe (independent FMA chains, full occupancy)
__global__ void k_probe_dfma(double *out, int iters, double b, double c) {
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void k_probe_ffma(float *out, int iters, float b, float c) {
    float a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
        a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// FP64 tensor-core (DMMA) throughput probe: eight independent m8n8k4 FP64
// MMA chains per warp (512 flops each per step)
__global__ void k_probe_dmma(double *out, int iters) {
    const double a = 1.0 + threadIdx.x * 1e-3, b = 0.999;
    double c[8][2];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = 0.0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};" : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 latency probes (one block, SM clock cycles from clock64):
// kind 3: one thread, a dependent chain of DFMA (cycles per DFMA);
// kind 4: one warp, eight independent DFMA chains (cycles per warp
//         instruction: how often one warp can issue FP64 work);
// kind 5: one thread, a dependent chain of FP64 divisions (cycles each)
__global__ void k_probe_fp64_lat(int kind, double *out, long long *cyc, int n, double b, double c) {
    double a0 = threadIdx.x + 1.5, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const long long t0 = clock64();
    if (kind == 3) {
        for (int i = 0; i < n; ++i) a0 = fma(a0, b, c);
    } else if (kind == 4) {
        for (int i = 0; i < n; ++i) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
    } else {
        for (int i = 0; i < n; ++i) a0 = b / a0;
    }
    const long long t1 = clock64();
    if (threadIdx.x == 0) cyc[0] = t1 - t0;
    out[threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// per-type occupancy of the panel kernel (defined in the per-type units)
int panel_blocks_per_sm_s();
int panel_blocks_per_sm_d();
int panel_blocks_per_sm_c();
int panel_blocks_per_sm_z();

static constexpr int kMaxDevices = 64;
static DeviceFacts g_facts[kMaxDevices];
static std::once_flag g_facts_once[kMaxDevices];

// Library-wide device status word: set by any kernel whose bounded wait
// expired (tensor-core pipelines, grid barriers); read by
// rnpgpu_device_status.  One file-scope variable, so no allocation.
static __device__ int g_device_status;
int *device_status_ptr() {
    static int *ptr[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    if (ptr[dev] == nullptr) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_status) == cudaSuccess) ptr[dev] = (int *)p;
    }
    return ptr[dev];
}

const DeviceFacts &device_facts() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    std::call_once(g_facts_once[dev], [dev]() {
        DeviceFacts f;
        cudaDeviceGetAttribute(&f.sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (f.sm_count <= 0) f.sm_count = 1;
        f.panel_max_blocks[0] = panel_blocks_per_sm_s() * f.sm_count;
        f.panel_max_blocks[1] = panel_blocks_per_sm_d() * f.sm_count;
        f.panel_max_blocks[2] = panel_blocks_per_sm_c() * f.sm_count;
        f.panel_max_blocks[3] = panel_blocks_per_sm_z() * f.sm_count;
        g_facts[dev] = f;
    });
    return g_facts[dev];
}

} // namespace rnpgpu

extern "C" {

// Device status word (nonzero if a bounded wait of some kernel expired since
// the last reset): returns it and, if reset is nonzero, clears it; synchronous.
int rnpgpu_device_status(int reset) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, rnpgpu::g_device_status, sizeof(int)) != cudaSuccess) return -1;
    if (reset) {
        const int z = 0;
        cudaMemcpyToSymbol(rnpgpu::g_device_status, &z, sizeof(int));
    }
    return v;
}

int rnpgpu_set_stream(void *stream) {
    rnpgpu::t_stream = (cudaStream_t)stream;
    return 0;
}
void *rnpgpu_get_stream(void) { return (void *)rnpgpu::t_stream; }
const char *rnpgpu_get_last_error(void) { return rnpgpu::t_last_error.c_str(); }
const char *rnpgpu_version(void) { return "rnp2_gb300 0.1 (sm_103a)"; }

unsigned long long rnpgpu_launch_count(void) { return rnpgpu::g_launches.load(); }

int rnpgpu_timing_enable(int on) {
    rnpgpu::t_timer.on = (on != 0);
    return 0;
}

// "name count total_ms\n" per kernel class since the last report; resets.
int rnpgpu_timing_report(char *buf, size_t len) {
    using namespace rnpgpu;
    std::map<std::string, std::pair<long, double> > acc;
    for (auto &t : t_timer.done) {
        cudaEventSynchronize(t.stop);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t.start, t.stop);
        auto &a = acc[t.name];
        a.first += 1;
        a.second += ms;
        t_timer.pool.push_back(t.start);
        t_timer.pool.push_back(t.stop);
    }
    t_timer.done.clear();
    std::string out;
    char line[256];
    for (auto &kv : acc) {
        snprintf(line, sizeof(line), "%s %ld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
        out += line;
    }
    if (buf && len) {
        size_t n = std::min(len - 1, out.size());
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return (int)out.size();
}

// Measured FMA throughput of the current device in TFLOP/s
// (kind 0: FP64 DFMA, kind 1: FP32 FFMA); synchronous.
int rnpgpu_probe_peak(int kind, void *scratch, size_t scratch_bytes, double *tflops) {
    using namespace rnpgpu;
    const DeviceFacts &f = device_facts();
    const int blocks = f.sm_count * 8, threads = 256;
    if (scratch_bytes < (size_t)blocks * threads * sizeof(double) || tflops == nullptr) return -2;
    if (kind < 0 || kind > 5) return -1;
    cudaStream_t st = current_stream();
    if (kind >= 3) {
        // latencies in cycles: scratch holds 32 doubles of outputs and the count
        const int n = kind == 5 ? 1024 : 4096;
        long long *cyc = reinterpret_cast<long long *>((double *)scratch + 64);
        double best = 1e300;
        for (int rep = 0; rep < 3; ++rep) {
            k_probe_fp64_lat<<<1, kind == 4 ? 32 : 1, 0, st>>>(kind, (double *)scratch, cyc, n, 0.999, 1e-3);
            long long h = 0;
            if (cudaMemcpyAsync(&h, cyc, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) break;
            best = std::min(best, (double)h / (kind == 4 ? 8.0 * n : (double)n));
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_last_error(cudaGetErrorString(e));
            return 1;
        }
        *tflops = best;
        return 0;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = kind == 0 ? 4096 : kind == 2 ? 2048 : 65536;
    double best = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, st);
        if (kind == 0) k_probe_dfma<<<blocks, threads, 0, st>>>((double *)scratch, iters, 0.999, 1e-3);
        else if (kind == 2) k_probe_dmma<<<blocks, threads, 0, st>>>((double *)scratch, iters);
        else k_probe_ffma<<<blocks, threads, 0, st>>>((float *)scratch, iters, 0.999f, 1e-3f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        // FMA kinds: 8 chains x 2 flops per thread per step; DMMA: 8 MMAs x
        // 512 flops per warp per step
        double fl = kind == 2 ? 8.0 * 512.0 * (double)iters * blocks * (threads / 32) : 2.0 * 8 * (double)iters * blocks * threads;
        if (ms > 0) best = std::max(best, fl / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return 1;
    }
    *tflops = best;
    return 0;
}

} // extern "C"
