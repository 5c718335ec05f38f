// qr_d.cu — double instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T double
#define RNPGPU_CT double
#define RNPGPU_P d
#define RNPGPU_LOW_T float
#define RNPGPU_MIXED_FN rnpgpu_dsgels
#include "qr_type.inc"
