// ks_f32_batch.cu -- batched (one launch per stage over a job table) kernels
// of the single-precision unit; a unit of its own so that it compiles in
// parallel with ks_f32.cu.
#include "ks_kernels.cuh"
#define KS_R float
#define KS_SUF f32
#define KS_BATCH_UNIT
#include "ks_unit.inc"
