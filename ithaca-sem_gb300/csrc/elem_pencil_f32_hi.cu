// FP32 pencil / pipelined hexahedral Helmholtz kernels for orders 7 and 8 (P = 6, 7), in
// their own unit so that they compile alongside the other orders.
#include "elem_pencil_launch.cuh"

namespace ithaca {

// orders 9 and 10 (elem_pencil_f32_top.cu)
bool launch_helm_pencil_f32_top(int n, int Q, int E, int variant, const double* hB, const double* hD, const float* jg,
                                float lambda, const float* in, float* out, const int* l2g, int ndir, const int* skip,
                                const float* lam_ptr, int* err, cudaStream_t s, OwnedRows* own);

bool launch_helm_pencil_f32_hi(int n, int Q, int E, int variant, const double* hB, const double* hD, const float* jg,
                               float lambda, const float* in, float* out, const int* l2g, int ndir, const int* skip,
                               const float* lam_ptr, int* err, cudaStream_t s, OwnedRows* own) {
  using T = float;
#define X(NN, QQ) ITHACA_PENCIL_F32_ORDER(NN, QQ)
  X(7, 8) X(8, 9)
#undef X
  return launch_helm_pencil_f32_top(n, Q, E, variant, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s,
                                    own);
}

}  // namespace ithaca
