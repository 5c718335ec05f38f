// qr_z.cu — rnpgpu::cf64 instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T rnpgpu::cf64
#define RNPGPU_CT rnpgpu_complex_double
#define RNPGPU_P z
#define RNPGPU_LOW_T rnpgpu::cf32
#define RNPGPU_MIXED_FN rnpgpu_zcgels
#include "qr_type.inc"
