// FP32 pencil / pipelined hexahedral Helmholtz kernels for orders 9 and 10 (P = 8, 9), in
// their own unit so that they compile alongside the other orders.
#include "elem_pencil_launch.cuh"

namespace ithaca {

bool launch_helm_pencil_f32_top(int n, int Q, int E, int variant, const double* hB, const double* hD, const float* jg,
                                float lambda, const float* in, float* out, const int* l2g, int ndir, const int* skip,
                                const float* lam_ptr, int* err, cudaStream_t s, OwnedRows* own) {
  using T = float;
#define X(NN, QQ) ITHACA_PENCIL_F32_ORDER(NN, QQ)
  X(9, 10) X(10, 11)
#undef X
  return false;
}

}  // namespace ithaca
