// ks_launch.h -- host-side launchers of the per-precision kernel units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "kurucz_gb300.h"
#include "ks_internal.h"

namespace ks {

// JOSH constants in single precision -- the mean-intensity operator, the
// flux weights and the optical-depth grid -- passed to the transfer kernels
// by value so they live in the kernel's constant bank.
struct CoefJ32 {
    float c[51 * 51];
    float ch[51];
    float xtau[51];
};

#define KS_DECLARE_LAUNCHERS(R, SUF)                                                              \
    cudaError_t launch_prep_##SUF(const PrepArgs& a, cudaStream_t s);                             \
    cudaError_t launch_continuum_##SUF(const ContArgs& a, R* ca, R* cs, cudaStream_t s);         \
    cudaError_t launch_pair_setup_##SUF(const PairArgs& a, bool fused, const R* kap_a,           \
                                        const R* kap_b, PairDesc<R>* desc, uint8_t* cls,         \
                                        cudaStream_t s);                                          \
    cudaError_t launch_accumulate_##SUF(const AccArgs& a, int warps, const PairDesc<R>* desc,    \
                                        R* out, cudaStream_t s);                                  \
    cudaError_t launch_transfer_##SUF(const TransferArgs& a, const CoefJ32* cj, const R* ca,     \
                                      const R* cs, const R* lo, const R* lsc, const R* src,      \
                                      cudaStream_t s);                                            \
    cudaError_t launch_transfer_stream_##SUF(const TransferArgs& a, const CoefJ32* cj,           \
                                             const R* ca, const R* cs, const R* lo,               \
                                             int32_t* list, unsigned long long* count,            \
                                             cudaStream_t s);                                     \
    size_t accumulate_smem_bytes_##SUF(int tile_bins, int warps);                                \
    cudaError_t batch_grids_##SUF(int warps_per_tile, int tile_bins, bool stream_pass,            \
                                  const int64_t* totals, int* grids);                             \
    cudaError_t launch_prep_batch_##SUF(const PrepArgs* jobs, BatchGrid g, int grid, cudaStream_t s); \
    cudaError_t launch_continuum_batch_##SUF(const void* jobs, BatchGrid g, int grid, cudaStream_t s); \
    cudaError_t launch_pair_setup_batch_##SUF(const void* jobs, BatchGrid g, int grid, cudaStream_t s); \
    cudaError_t launch_accumulate_batch_##SUF(const void* jobs, BatchGrid g, int grid, int warps,    \
                                             int tile_bins, cudaStream_t s);                         \
    cudaError_t launch_transfer_batch_##SUF(const void* jobs, BatchGrid g, BatchGrid g_list,         \
                                           const CoefJ32* cj, int grid, int grid_list,               \
                                           bool stream_pass, cudaStream_t s);

KS_DECLARE_LAUNCHERS(float, f32)
KS_DECLARE_LAUNCHERS(double, f64)

// records `msg` as the calling thread's last error (ks_last_error) and returns `code`
ks_status set_error(ks_status code, const std::string& msg);

// adjoint kernels (FP64 unit)
cudaError_t launch_transfer_adjoint(const AdjArgs& a, cudaStream_t s);
cudaError_t launch_line_adjoint(const LineAdjArgs& a, cudaStream_t s);
cudaError_t launch_line_grad(const LineGradArgs& a, cudaStream_t s);
cudaError_t launch_atm_grad(const AtmGradArgs& a, cudaStream_t s);

// hydrogen lines (ks_hydrogen.cu), added onto the line-opacity cube
cudaError_t launch_hydrogen_f32(const HydArgs& a, float* cube, cudaStream_t s);
cudaError_t launch_hydrogen_f64(const HydArgs& a, double* cube, cudaStream_t s);
cudaError_t launch_helium_f32(const HeArgs& a, float* cube, cudaStream_t s);
cudaError_t launch_helium_f64(const HeArgs& a, double* cube, cudaStream_t s);
cudaError_t launch_f19_f32(const F19Args& a, float* cube, cudaStream_t s);
cudaError_t launch_f19_f64(const F19Args& a, double* cube, cudaStream_t s);
// device copy of the hydrogen profile tables (uploaded on first use per device)
ks_status hydrogen_device_tables(const HydTables** out);

}  // namespace ks
