// Triangle element kernels instantiated for float.
#include "elem_tri.cuh"

namespace ithaca {
ITHACA_TRI_INSTANTIATE(float)
}  // namespace ithaca
