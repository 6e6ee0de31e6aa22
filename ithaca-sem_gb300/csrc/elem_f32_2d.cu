// Element kernels instantiated for float, dimension 2.
#include "elem_launch.cuh"
ITHACA_ELEM_INSTANTIATE(float, 2)
