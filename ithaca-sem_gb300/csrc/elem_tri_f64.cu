// Triangle element kernels instantiated for double.
#include "elem_tri.cuh"

namespace ithaca {
ITHACA_TRI_INSTANTIATE(double)
}  // namespace ithaca
