// FP32-mixed kernels.
#define REAL float
#define CRV_REAL_IS_FLOAT 1
#include "crv_kernels_prec.inc"
