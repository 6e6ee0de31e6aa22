// Element kernels instantiated for double, dimension 3.
#include "elem_launch.cuh"
ITHACA_ELEM_INSTANTIATE(double, 3)
