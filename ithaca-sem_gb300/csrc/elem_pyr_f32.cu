// Pyramid element kernels instantiated for float.
#include "elem_pyr.cuh"

namespace ithaca {
ITHACA_PYR_INSTANTIATE(float)
}  // namespace ithaca
