// api_context.cu — per-thread stream and error state, device facts, and the
// library-level C ABI entry points (rnpgpu_set_stream & co.).
#include "qr_driver.cuh"
#include "../../include/rnp_gpu/qr_gb300.h"
#include <cstdio>
#include <string>

namespace rnpgpu {

static thread_local cudaStream_t t_stream = nullptr;
static thread_local std::string t_last_error;

cudaStream_t current_stream() { return t_stream; }
void set_last_error(const char *msg) { t_last_error = msg ? msg : ""; }

// per-type occupancy of the panel kernel (defined in the per-type units)
int panel_blocks_per_sm_s();
int panel_blocks_per_sm_d();
int panel_blocks_per_sm_c();
int panel_blocks_per_sm_z();

static constexpr int kMaxDevices = 64;
static DeviceFacts g_facts[kMaxDevices];
static std::once_flag g_facts_once[kMaxDevices];

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

int rnpgpu_set_stream(void *stream) {
    rnpgpu::t_stream = (cudaStream_t)stream;
    return 0;
}
void *rnpgpu_get_stream(void) { return (void *)rnpgpu::t_stream; }
const char *rnpgpu_get_last_error(void) { return rnpgpu::t_last_error.c_str(); }
const char *rnpgpu_version(void) { return "rnp2_gb300 0.1 (sm_103a)"; }

} // extern "C"
