// FP64 instantiations of the persistent pipelined hexahedral Helmholtz kernel: scalar FP64
// pencils with every 1-D operator in its even-odd form (the GLL points' symmetry and the
// ModifiedA modes' parity halve the multiply-adds of the contractions), the geometry
// slab staged by TMA as in the FP32 kernel. Built for Q even (P = 2, 4, 6, 8).
#include "elem_pencil_launch.cuh"

namespace ithaca {

// variant 1 / 2: one / two elements per group (64 / 128 threads per CTA).
bool launch_helm_pencil64(int n, int Q, int E, int variant, const double* hB, const double* hD, const double* jg,
                          double lambda, const double* in, double* out, const int* l2g, int ndir, const int* skip,
                          const double* lam_ptr, int* err, cudaStream_t s) {
  if (variant != 1 && variant != 2) return false;
#define X(NN, QQ)                                                                                              \
  if (n == NN && Q == QQ) {                                                                                    \
    if (variant == 1)                                                                                          \
      dev::pipe_nq<double, NN, QQ, 1, 1, double, false, false, false, true>(E, hB, hD, jg, lambda, in, out, l2g, \
                                                                            ndir, skip, lam_ptr, err, s);      \
    else                                                                                                       \
      dev::pipe_nq<double, NN, QQ, 2, 1, double, false, false, false, true>(E, hB, hD, jg, lambda, in, out, l2g, \
                                                                            ndir, skip, lam_ptr, err, s);      \
    return true;                                                                                               \
  }
  X(3, 4) X(5, 6) X(7, 8) X(9, 10)
#undef X
  return false;
}

}  // namespace ithaca
