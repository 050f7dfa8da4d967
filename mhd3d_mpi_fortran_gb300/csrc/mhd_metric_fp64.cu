// FP64 instantiation of the metric-mode (curvilinear) step kernels, built
// with -fmad=false like mhd_fp64.cu, so that results round as the oracle's
// metric mode writes them.
#include "mhd_kernels.cuh"

namespace mhd {
template struct Launch<double, true>;
}
