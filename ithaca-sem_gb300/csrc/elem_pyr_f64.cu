// Pyramid element kernels instantiated for double.
#include "elem_pyr.cuh"

namespace ithaca {
ITHACA_PYR_INSTANTIATE(double)
}  // namespace ithaca
