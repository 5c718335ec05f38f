// qr_s.cu — float instantiation of the QR path and its C ABI entry points.
#define RNPGPU_T float
#define RNPGPU_CT float
#define RNPGPU_P s
#include "qr_type.inc"
