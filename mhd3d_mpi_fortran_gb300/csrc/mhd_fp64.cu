// FP64 instantiation of the step kernels.  Built with -fmad=false so that no
// multiply-add is contracted: every FP64 result is rounded as the reference's
// Fortran expression is written (the all-FP64 parity mode).
#include "mhd_kernels.cuh"

namespace mhd {
template struct Launch<double>;
template struct Batch<double>;
}
