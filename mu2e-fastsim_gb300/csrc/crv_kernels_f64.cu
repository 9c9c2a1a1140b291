// FP64 plain kernels (built with -fmad=false: bit-exact with the CPU oracle).
#define REAL double
#define CRV_REAL_IS_FLOAT 0
#include "crv_kernels_prec.inc"
