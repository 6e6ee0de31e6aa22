// FP32 instantiations and launcher of the pencil hexahedral Helmholtz kernels.
#include <algorithm>
#include <type_traits>

#include "elem_pencil_launch.cuh"

namespace ithaca {

// variant: 2 or 4 = one pass per CTA with a TMA-staged geometry slab and that many
// elements per CTA; 21 or 22 = the persistent pipelined kernel with 1 or 2 elements per
// group and a double geometry buffer; 31 or 32 = the same with a single buffer; 41 or 42 =
// the single-buffer kernel with its contractions on packed FP32 pairs (fma.rn.f32x2); 43 or
// 44 = 42 or 41 with vector pencils in shared memory, 46 = 43 with the contractions along i
// and j on the tensor cores (TF32 MMAs in three-term split precision), 47 = 43 with every
// 1-D operator in its even-odd form (half the multiply-adds; Q = 8; other orders run 42 or
// 41).

// orders 7..10 of the variants below (elem_pencil_f32_hi.cu and _top.cu, compiled in parallel)
bool launch_helm_pencil_f32_hi(int n, int Q, int E, int variant, const double* hB, const double* hD, const float* jg,
                               float lambda, const float* in, float* out, const int* l2g, int ndir, const int* skip,
                               const float* lam_ptr, int* err, cudaStream_t s, OwnedRows* own);

template <typename T>
bool launch_helm_pencil(int n, int Q, int E, int variant, const double* hB, const double* hD, const T* jg, T lambda,
                        const T* in, T* out, const int* l2g, int ndir, const int* skip, const T* lam_ptr, int* err,
                        cudaStream_t s, OwnedRows* own) {
  if (own != nullptr) own->ctas = -1;  // set by the pipelined kernels only
  if (variant == 43 || variant == 44 || variant == 46 || variant == 47) {
    // vector pencils are built for Q = 8; elsewhere the scalar-pencil kernel with the same
    // arithmetic (and so the same results) runs
    if (n == 7 && Q == 8 && std::is_same<T, float>::value) {
      if (variant == 47)
        dev::pipe_nq<T, 7, 8, 2, 1, T, true, true, false, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip,
                                                                lam_ptr, err, s, nullptr, own);
      else if (variant == 46)
        dev::pipe_nq<T, 7, 8, 2, 1, T, true, true, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err,
                                                         s, nullptr, own);
      else if (variant == 43)
        dev::pipe_nq<T, 7, 8, 2, 1, T, true, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s,
                                                   nullptr, own);
      else
        dev::pipe_nq<T, 7, 8, 1, 1, T, true, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s,
                                                   nullptr, own);
      return true;
    }
    variant = variant == 44 ? 41 : 42;
  }
#define X(NN, QQ) ITHACA_PENCIL_F32_ORDER(NN, QQ)
  X(2, 3) X(3, 4) X(4, 5) X(5, 6) X(6, 7)
#undef X
  return launch_helm_pencil_f32_hi(n, Q, E, variant, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s,
                                   own);
}

template bool launch_helm_pencil<float>(int, int, int, int, const double*, const double*, const float*, float,
                                        const float*, float*, const int*, int, const int*, const float*, int*,
                                        cudaStream_t, OwnedRows*);

}  // namespace ithaca
