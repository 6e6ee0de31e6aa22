// FP32 pipelined hexahedral Helmholtz kernel on half-precision geometry (the 16-bit
// geometry mode of the mixed solver).
#include "elem_pencil_launch.cuh"

namespace ithaca {

// Pipelined kernel on half-precision geometry with per-element, per-field FP32 scales (8
// floats per element). At (n, Q) = (7, 8) variants 43 and 47 run the vector-pencil kernel
// (two elements per group, conflict-free shared-memory layout; 47 with the even-odd 1-D
// operators) on that geometry; every other case runs one element per group with packed
// FP32 pairs.
bool launch_helm_pipe_geo16(int n, int Q, int E, int variant, const double* hB, const double* hD, const void* jg16,
                            const float* gscale, float lambda, const float* in, float* out, const int* l2g, int ndir,
                            const int* skip, const float* lam_ptr, int* err, cudaStream_t s, OwnedRows* own) {
  const __half* jg = static_cast<const __half*>(jg16);
  if (n == 7 && Q == 8 && variant == 47) {
    dev::pipe_nq<float, 7, 8, 2, 1, __half, true, true, false, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip,
                                                                     lam_ptr, err, s, gscale, own);
    return true;
  }
  if (n == 7 && Q == 8 && variant == 43) {
    dev::pipe_nq<float, 7, 8, 2, 1, __half, true, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err,
                                                        s, gscale, own);
    return true;
  }
#define X(NN, QQ)                                                                                          \
  if (n == NN && Q == QQ) {                                                                                \
    dev::pipe_nq<float, NN, QQ, 1, 1, __half, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr,   \
                                                    err, s, gscale, own);                                  \
    return true;                                                                                           \
  }
  X(2, 3) X(3, 4) X(4, 5) X(5, 6) X(6, 7) X(7, 8) X(8, 9) X(9, 10) X(10, 11)
#undef X
  return false;
}

}  // namespace ithaca
