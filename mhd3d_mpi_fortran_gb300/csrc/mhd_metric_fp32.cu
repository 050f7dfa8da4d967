// FP32 instantiation of the metric-mode (curvilinear) step kernels: FP32
// state, reconstruction and fluxes; FP64 metric terms, converted per load.
// FMA contraction on.
#include "mhd_kernels.cuh"

namespace mhd {
template struct Launch<float, true>;
}
