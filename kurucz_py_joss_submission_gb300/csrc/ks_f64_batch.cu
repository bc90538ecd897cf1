// ks_f64_batch.cu -- batched kernels of the FP64 unit (compiled, like
// ks_f64.cu, with --fmad=false).
#include "ks_kernels.cuh"
#define KS_R double
#define KS_SUF f64
#define KS_BATCH_UNIT
#include "ks_unit.inc"
