// Prism element kernels instantiated for float.
#include "elem_prism.cuh"

namespace ithaca {
ITHACA_PRISM_INSTANTIATE(float)
}  // namespace ithaca
