// ks_f64.cu -- FP64 (KS_PREC_FP64) unit of the kernels; compiled with
// --fmad=false so products and sums round separately, as in the reference.
#include "ks_kernels.cuh"
#define KS_R double
#define KS_SUF f64
#include "ks_unit.inc"
