// qr_d.cu — double instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T double
#define RNPGPU_CT double
#define RNPGPU_P d
#include "qr_type.inc"
