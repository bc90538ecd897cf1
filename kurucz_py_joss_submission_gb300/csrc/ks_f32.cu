// ks_f32.cu -- single-precision (KS_PREC_MIXED) unit of the kernels.
#include "ks_kernels.cuh"
#define KS_R float
#define KS_SUF f32
#include "ks_unit.inc"
