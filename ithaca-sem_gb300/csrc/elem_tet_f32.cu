// Tetrahedron element kernels instantiated for float.
#include "elem_tet.cuh"

namespace ithaca {
ITHACA_TET_INSTANTIATE(float)
}  // namespace ithaca
