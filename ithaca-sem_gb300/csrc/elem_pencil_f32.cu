// FP32 instantiations and launcher of the pencil hexahedral Helmholtz kernel.
#include "elem_pencil.cuh"

namespace ithaca {
namespace dev {

template <typename T, int N, int Q, int EB>
static void pencil_nq(int E, const double* hB, const double* hD, const T* jg, T lambda, const T* in, T* out,
                      const int* l2g, int ndir, const int* skip, const T* lam_ptr, int* err, cudaStream_t s) {
  PTabs<T, N, Q> tab;
  for (int i = 0; i < N * Q; ++i) tab.B[i] = (T)hB[i];
  for (int i = 0; i < Q * Q; ++i) tab.D[i] = (T)hD[i];
  using L = PencilLayout<T, N, Q, EB>;
  auto k = l2g ? helm3_pencil_kernel<T, N, Q, EB, true> : helm3_pencil_kernel<T, N, Q, EB, false>;
  static bool prepared[2] = {false, false};
  if (!prepared[l2g ? 1 : 0]) {
    ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes()));
    prepared[l2g ? 1 : 0] = true;
  }
  const dim3 block(Q * Q, EB), grid((E + EB - 1) / EB);
  k<<<grid, block, L::bytes(), s>>>(in, out, tab, jg, lambda, E, l2g, ndir, skip, lam_ptr, err);
}

}  // namespace dev

template <typename T>
bool launch_helm_pencil(int n, int Q, int E, int eb, const double* hB, const double* hD, const T* jg, T lambda,
                        const T* in, T* out, const int* l2g, int ndir, const int* skip, const T* lam_ptr, int* err,
                        cudaStream_t s) {
#define X(NN, QQ)                                                                                        \
  if (n == NN && Q == QQ) {                                                                              \
    if (eb >= 4)                                                                                         \
      dev::pencil_nq<T, NN, QQ, 4>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s);    \
    else                                                                                                 \
      dev::pencil_nq<T, NN, QQ, 2>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s);    \
    return true;                                                                                         \
  }
  X(2, 3) X(3, 4) X(4, 5) X(5, 6) X(6, 7) X(7, 8) X(8, 9) X(9, 10) X(10, 11)
#undef X
  return false;
}

template bool launch_helm_pencil<float>(int, int, int, int, const double*, const double*, const float*, float,
                                        const float*, float*, const int*, int, const int*, const float*, int*,
                                        cudaStream_t);

}  // namespace ithaca
