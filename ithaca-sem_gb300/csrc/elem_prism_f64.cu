// Prism element kernels instantiated for double.
#include "elem_prism.cuh"

namespace ithaca {
ITHACA_PRISM_INSTANTIATE(double)
}  // namespace ithaca
