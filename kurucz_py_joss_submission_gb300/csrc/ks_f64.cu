// ks_f64.cu -- FP64 (KS_PREC_FP64) unit of the kernels; compiled with
// --fmad=false so products and sums round separately, as in the reference.
#include "ks_kernels.cuh"
#define KS_R double
#define KS_SUF f64
#include "ks_unit.inc"

// adjoint kernels of the differentiable form (FP64 only)
#include "ks_adjoint.cuh"

namespace ks {

cudaError_t launch_transfer_adjoint(const AdjArgs& a, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    transfer_adjoint_kernel<<<(unsigned)((a.n + 63) / 64), 64, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_line_adjoint(const LineAdjArgs& a, cudaStream_t s) {
    if (a.n_lines == 0) return cudaSuccess;
    line_adjoint_kernel<<<152 * 16, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_line_grad(const LineGradArgs& a, cudaStream_t s) {
    if (a.n_lines == 0) return cudaSuccess;
    line_grad_kernel<<<(unsigned)((a.n_lines + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_atm_grad(const AtmGradArgs& a, cudaStream_t s) {
    if (a.n_layers == 0) return cudaSuccess;
    if (a.n_groups > 0) {
        atm_grad_group_kernel<<<dim3((unsigned)a.n_groups, (unsigned)a.n_layers), 128, 0, s>>>(a);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    atm_grad_depth_kernel<<<(unsigned)((a.n_layers + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace ks
