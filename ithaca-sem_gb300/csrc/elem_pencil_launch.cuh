// Host launcher of the persistent pipelined hexahedral Helmholtz kernel
// (elem_pencil_pipe.cuh), shared by its FP32 and FP64 instantiation units.
#pragma once

#include <algorithm>
#include <type_traits>

#include "elem_pencil_pipe.cuh"

namespace ithaca {
namespace dev {

template <typename T, int N, int Q, int EB>
inline void pencil_nq(int E, const double* hB, const double* hD, const T* jg, T lambda, const T* in, T* out,
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

template <typename T, int N, int Q>
inline PTabs3<T, N, Q> eo_tables(const double* hB, const double* hD) {
  PTabs3<T, N, Q> t{};
  if constexpr (Q % 2 == 0) {
    constexpr int H = Q / 2, NE = (N + 1) / 2;
    for (int i = 0; i < H; ++i) {
      for (int j = 0; j < NE; ++j) {
        double x, y;
        if (j == 0) {
          x = 0.5 * (hB[i] + hB[Q + i]);
          y = 0.5 * (hB[i] - hB[Q + i]);
        } else {
          x = 2 * j < N ? hB[2 * j * Q + i] : 0.0;
          y = 2 * j + 1 < N ? hB[(2 * j + 1) * Q + i] : 0.0;
        }
        t.bw[i][j] = TPair<T>{(T)x, (T)y};
      }
      for (int k = 0; k < H; ++k) {
        const double a = hD[k * Q + i], b = hD[(Q - 1 - k) * Q + i];            // l'_k(z_i), l'_{Q-1-k}(z_i)
        const double c = hD[i * Q + k], d = hD[i * Q + Q - 1 - k];              // l'_i(z_k), l'_i(z_{Q-1-k})
        t.d[i][k] = TPair<T>{(T)(0.5 * (a + b)), (T)(0.5 * (a - b))};
        t.dt[i][k] = TPair<T>{(T)(0.5 * (c + d)), (T)(0.5 * (c - d))};
      }
    }
  }
  return t;
}

// Persistent pipelined kernel: one CTA per resident slot (SMs x CTAs per SM, from the
// occupancy calculator), never more CTAs than element groups.
template <typename T, int N, int Q, int EB, int NB, typename TG = T, bool PACK = false, bool V4 = false,
          bool TC = false, bool EO = false>
inline void pipe_nq(int E, const double* hB, const double* hD, const TG* jg, T lambda, const T* in, T* out,
                    const int* l2g, int ndir, const int* skip, const T* lam_ptr, int* err, cudaStream_t s,
                    const float* gscale = nullptr, OwnedRows* own = nullptr) {
  PTabs<T, N, Q> tab;
  for (int i = 0; i < N * Q; ++i) tab.B[i] = (T)hB[i];
  for (int i = 0; i < Q * Q; ++i) tab.D[i] = (T)hD[i];
  PTabs2<N, Q> tab2{};
  constexpr int QP = PTabs2<N, Q>::QP, NP = PTabs2<N, Q>::NP;
  for (int p = 0; p < N; ++p)
    for (int i = 0; i < Q; ++i) {
      tab2.BF[p * QP + i] = (float)hB[p * Q + i];
      tab2.BT[i * NP + p] = (float)hB[p * Q + i];
    }
  for (int k = 0; k < Q; ++k)
    for (int i = 0; i < Q; ++i) {
      tab2.DF[k * QP + i] = (float)hD[k * Q + i];  // l_k'(z_i)
      tab2.DT[i * QP + k] = (float)hD[k * Q + i];
    }
  using L = PipeLayout<T, N, Q, EB, NB, TG, V4>;
  const PTabs3<T, N, Q> tab3 = eo_tables<T, N, Q>(hB, hD);
  auto k = l2g ? helm3_pipe_kernel<T, N, Q, EB, true, NB, TG, PACK, V4, TC, EO>
               : helm3_pipe_kernel<T, N, Q, EB, false, NB, TG, PACK, V4, TC, EO>;
  static int slots[2] = {0, 0};  // resident CTAs on the whole GPU
  const int gi = l2g ? 1 : 0;
  if (slots[gi] == 0) {
    ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes()));
    int dev = 0, sms = 0, per_sm = 0;
    ITHACA_CUDA(cudaGetDevice(&dev));
    ITHACA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ITHACA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, Q * Q * EB, L::bytes()));
    slots[gi] = std::max(1, sms * std::max(1, per_sm));
  }
  const int ngroups = (E + EB - 1) / EB;
  const dim3 block(Q * Q, EB), grid(std::min(ngroups, slots[gi]));
  T* sown = nullptr;
  double* opart = nullptr;
  const int* ocode = nullptr;
  if constexpr (std::is_same<T, float>::value) {  // the scattered output is FP32 only
    if (own != nullptr && l2g != nullptr && own->ocode != nullptr) {
      sown = own->s;
      opart = own->part;
      ocode = own->ocode;
      own->ctas = (int)grid.x;
    }
  }
  k<<<grid, block, L::bytes(), s>>>(in, out, tab, tab2, tab3, jg, lambda, E, l2g, ndir, skip, lam_ptr, err, gscale,
                                    sown, opart, ocode);
}

}  // namespace dev
}  // namespace ithaca

// One order of the FP32 variants 2..42 (launch_helm_pencil): returns from the enclosing
// launcher when (n, Q) == (NN, QQ).
#define ITHACA_PENCIL_F32_ORDER(NN, QQ)                                                                    \
  if (n == NN && Q == QQ) {                                                                                \
    if (variant == 4)                                                                                      \
      dev::pencil_nq<T, NN, QQ, 4>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s);      \
    else if (variant == 2)                                                                                 \
      dev::pencil_nq<T, NN, QQ, 2>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s);      \
    else if (variant == 21)                                                                                \
      dev::pipe_nq<T, NN, QQ, 1, 2>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own);     \
    else if (variant == 22)                                                                                \
      dev::pipe_nq<T, NN, QQ, 2, 2>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own);     \
    else if (variant == 31)                                                                                \
      dev::pipe_nq<T, NN, QQ, 1, 1>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own);     \
    else if (variant == 32)                                                                                \
      dev::pipe_nq<T, NN, QQ, 2, 1>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own);     \
    else if (variant == 41)                                                                                \
      dev::pipe_nq<T, NN, QQ, 1, 1, T, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own); \
    else if (variant == 42)                                                                                \
      dev::pipe_nq<T, NN, QQ, 2, 1, T, true>(E, hB, hD, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, err, s, nullptr, own); \
    else                                                                                                   \
      return false;                                                                                        \
    return true;                                                                                           \
  }
