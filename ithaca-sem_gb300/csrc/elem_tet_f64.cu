// Tetrahedron element kernels instantiated for double.
#include "elem_tet.cuh"

namespace ithaca {
ITHACA_TET_INSTANTIATE(double)
}  // namespace ithaca
