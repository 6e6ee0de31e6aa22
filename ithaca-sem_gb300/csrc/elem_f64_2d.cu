// Element kernels instantiated for double, dimension 2.
#include "elem_launch.cuh"
ITHACA_ELEM_INSTANTIATE(double, 2)
