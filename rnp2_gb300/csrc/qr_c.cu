// qr_c.cu — rnpgpu::cf32 instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T rnpgpu::cf32
#define RNPGPU_CT rnpgpu_complex_float
#define RNPGPU_P c
#include "qr_type.inc"
