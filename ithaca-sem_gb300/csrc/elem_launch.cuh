// Host-side launchers for the element kernels of one precision and dimension.
// Each translation unit that includes this instantiates all (n, Q = n + 1),
// 2 <= n <= 10, for one (T, DIM) pair through ITHACA_ELEM_INSTANTIATE.
#pragma once

#include "elem.cuh"
#include "elem2_pencil.cuh"

namespace ithaca {
namespace dev {

template <typename T, int DIM, int N, int Q>
struct Cfg {
  using S = Shape<DIM, Q>;
  static size_t smem() { return Layout<T, DIM, N, Q>::bytes(S::EB); }
  static dim3 block() { return dim3(S::TPE, S::EB); }
  static dim3 grid(int E) { return dim3((E + S::EB - 1) / S::EB); }
  template <class K>
  static void prep(K k) {
    static bool done = false;  // attribute set once per kernel instantiation
    if (!done) {
      ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()));
      done = true;
    }
  }
};

// 1-D tables of (N, Q) as kernel parameters, computed on the host once per instantiation.
template <typename T, int N, int Q>
const PTabs<T, N, Q>& host_ptabs() {
  static const PTabs<T, N, Q> t = [] {
    const BasisTables b = make_basis(N, Q);
    PTabs<T, N, Q> r{};
    for (int i = 0; i < N * Q; ++i) r.B[i] = (T)b.B[i];
    for (int i = 0; i < Q * Q; ++i) r.D[i] = (T)b.D[i];
    return r;
  }();
  return t;
}

// The register-pencil kernel for deformed quads with CT threads per CTA (CT / Q elements).
template <typename T, int N, int Q, int CT>
void helm2_pencil_launch(int E, const T* jg, T lambda, const T* in, T* out, const int* l2g, int ndir, const int* skip,
                         const T* lam_ptr, const int* esolve, int skip_stride, cudaStream_t s) {
  using P = Pencil2<T, N, Q, CT>;
  auto k = l2g ? helm2_pencil_kernel<T, N, Q, true, CT> : helm2_pencil_kernel<T, N, Q, false, CT>;
  static bool prepared[2] = {false, false};
  if (!prepared[l2g ? 1 : 0]) {
    ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::bytes()));
    prepared[l2g ? 1 : 0] = true;
  }
  k<<<(E + P::EB - 1) / P::EB, dim3(Q, P::EB), P::bytes(), s>>>(in, out, host_ptabs<T, N, Q>(), jg, lambda, E, l2g,
                                                             ndir, skip, lam_ptr, esolve, skip_stride);
}

// variant (deformed quads; ignored elsewhere): -1 the default (FP32: the register-pencil
// kernel with 256 threads per CTA; FP64: the shared-memory kernel, as FP64 arithmetic
// bounds both and its smaller CTAs spread small meshes over more SMs), 0 the
// shared-memory kernel, 1 / 2 the register-pencil kernel with 256 / 128 threads per CTA.
template <typename T, int DIM, int N, int Q>
void helm_nq(int E, int deformed, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g, int ndir,
             const int* skip, const T* lam_ptr, const int* esolve, int skip_stride, cudaStream_t s, int variant) {
  if constexpr (DIM == 2) {
    if (deformed) {
      const int v = variant >= 0 ? variant : (sizeof(T) == 4 ? 1 : 0);
      if (v == 1) {
        helm2_pencil_launch<T, N, Q, 256>(E, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, esolve, skip_stride, s);
        return;
      }
      if (v == 2 && Q <= 128) {
        helm2_pencil_launch<T, N, Q, 128>(E, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, esolve, skip_stride, s);
        return;
      }
    }
  }
  using C = Cfg<T, DIM, N, Q>;
  constexpr int TPE = C::S::TPE;
  auto k = deformed ? (l2g ? helm_kernel<T, DIM, N, Q, TPE, true, true> : helm_kernel<T, DIM, N, Q, TPE, true, false>)
                    : (l2g ? helm_kernel<T, DIM, N, Q, TPE, false, true> : helm_kernel<T, DIM, N, Q, TPE, false, false>);
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, lambda, E, l2g, ndir, skip, lam_ptr, esolve,
                                               skip_stride);
}

template <typename T, int DIM, int N, int Q>
void bwd_nq(int E, const T* tab, const T* in, T* out, cudaStream_t s) {
  using C = Cfg<T, DIM, N, Q>;
  auto k = bwd_kernel<T, DIM, N, Q, C::S::TPE>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, E);
}

template <typename T, int DIM, int N, int Q>
void ipr_nq(int E, int deformed, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s) {
  using C = Cfg<T, DIM, N, Q>;
  auto k = deformed ? ipr_kernel<T, DIM, N, Q, C::S::TPE, true> : ipr_kernel<T, DIM, N, Q, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, E);
}

template <typename T, int DIM, int N, int Q>
void deriv_nq(int E, int deformed, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2, cudaStream_t s) {
  using C = Cfg<T, DIM, N, Q>;
  auto k = deformed ? deriv_kernel<T, DIM, N, Q, C::S::TPE, true> : deriv_kernel<T, DIM, N, Q, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, d0, d1, d2, tab, df, E);
}

template <typename T, int DIM, int N, int Q>
void iprd_nq(int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0, const T* in1, const T* in2,
             T* out, cudaStream_t s) {
  using C = Cfg<T, DIM, N, Q>;
  auto k = deformed ? iprd_kernel<T, DIM, N, Q, C::S::TPE, true> : iprd_kernel<T, DIM, N, Q, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in0, in1, in2, out, tab, jg, df, E);
}

template <typename T, int DIM, int N, int Q>
void diag_nq(int E, int deformed, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s) {
  using C = Cfg<T, DIM, N, Q>;
  auto k = deformed ? diag_kernel<T, DIM, N, Q, C::S::TPE, true> : diag_kernel<T, DIM, N, Q, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(out, tab, jg, lambda, E);
}


}  // namespace dev

#define ITHACA_FOR_EACH_NQ(X) X(2, 3) X(3, 4) X(4, 5) X(5, 6) X(6, 7) X(7, 8) X(8, 9) X(9, 10) X(10, 11)

template <typename T, int DIM>
bool ElemApi<T, DIM>::helm(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, const T* in,
                           T* out, const int* l2g, int ndir, const int* skip, const T* lam_ptr, const int* esolve,
                           int skip_stride, cudaStream_t s, int variant) {
#define X(NN, QQ)                                                                                  \
  if (n == NN && Q == QQ) {                                                                        \
    dev::helm_nq<T, DIM, NN, QQ>(E, deformed, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, esolve,           \
                                 skip_stride, s, variant);                                                         \
    return true;                                                                                   \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}

template <typename T, int DIM>
bool ElemApi<T, DIM>::bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s) {
#define X(NN, QQ)                                          \
  if (n == NN && Q == QQ) {                                \
    dev::bwd_nq<T, DIM, NN, QQ>(E, tab, in, out, s);       \
    return true;                                           \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}

template <typename T, int DIM>
bool ElemApi<T, DIM>::ipr(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* in, T* out,
                          cudaStream_t s) {
#define X(NN, QQ)                                                      \
  if (n == NN && Q == QQ) {                                            \
    dev::ipr_nq<T, DIM, NN, QQ>(E, deformed, tab, jg, in, out, s);     \
    return true;                                                       \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}

template <typename T, int DIM>
bool ElemApi<T, DIM>::deriv(int n, int Q, int E, int deformed, const T* tab, const T* df, const T* in, T* d0, T* d1,
                            T* d2, cudaStream_t s) {
#define X(NN, QQ)                                                                \
  if (n == NN && Q == QQ) {                                                      \
    dev::deriv_nq<T, DIM, NN, QQ>(E, deformed, tab, df, in, d0, d1, d2, s);      \
    return true;                                                                 \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}

template <typename T, int DIM>
bool ElemApi<T, DIM>::iprd(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0,
                           const T* in1, const T* in2, T* out, cudaStream_t s) {
#define X(NN, QQ)                                                                        \
  if (n == NN && Q == QQ) {                                                              \
    dev::iprd_nq<T, DIM, NN, QQ>(E, deformed, tab, jg, df, in0, in1, in2, out, s);      \
    return true;                                                                         \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}

template <typename T, int DIM>
bool ElemApi<T, DIM>::diag(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, T* out,
                           cudaStream_t s) {
#define X(NN, QQ)                                                          \
  if (n == NN && Q == QQ) {                                                \
    dev::diag_nq<T, DIM, NN, QQ>(E, deformed, tab, jg, lambda, out, s);    \
    return true;                                                           \
  }
  ITHACA_FOR_EACH_NQ(X)
#undef X
  return false;
}


}  // namespace ithaca

#define ITHACA_ELEM_INSTANTIATE(T, DIM) template struct ithaca::ElemApi<T, DIM>;
