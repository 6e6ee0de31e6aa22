// Element kernels instantiated for float, dimension 3.
#include "elem_launch.cuh"
ITHACA_ELEM_INSTANTIATE(float, 3)
