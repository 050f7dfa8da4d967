// FP32 instantiation of the step kernels (the production path): FP32 state,
// reconstruction and fluxes; FP64 metric (cell widths), FP64 CFL reduction
// and FP64 diagnostics.  FMA contraction on.
#include "mhd_kernels.cuh"

namespace mhd {
template struct Launch<float>;
template struct Batch<float>;
}
