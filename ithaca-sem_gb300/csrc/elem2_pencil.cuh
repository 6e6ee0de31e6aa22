// Register-pencil Helmholtz kernel for deformed quadrilaterals (used for FP32).
//
// The generic shared-memory kernel (elem.cuh) reads two shared-memory operands per
// multiply-add; on 2-D elements of high order that bounds it at a small fraction of the
// memory bandwidth. Here each element has Q threads. A thread holds one row (a fixed q or
// j) or one column (a fixed i) of the element in registers and contracts it against the
// 1-D tables, which are kernel parameters (constant bank). Shared memory is used only to
// hand rows to columns and back: six transposes of Q x (Q + 1) padded fields.
//
// Stages (collocation form, as elem.cuh; D[a*Q + i] = l_a'(z_i), B[p*Q + i] = B_p(z_i)):
//   rows q:     r(i, q)  = sum_p B(p, i) c(p, q)
//   columns i:  u(i, j)  = sum_q B(q, j) r(i, q);  g1(i, j) = sum_a D(a, j) u(i, a)
//   rows j:     g0(i, j) = sum_a D(a, i) u(a, j)
//   columns i:  f0 = m00 g0 + m01 g1, f1 = m01 g0 + m11 g1, v = lambda Jw u + sum_c D(j, c) f1(i, c)
//   rows j:     d(i, j)  = sum_c D(i, c) f0(c, j)
//   columns i:  v += d;  y(i, q) = sum_j B(q, j) v(i, j)
//   rows q:     out(p, q) = sum_i B(p, i) y(i, q)
#pragma once

#include "elem_pencil.cuh"

namespace ithaca {
namespace dev {

template <typename T, int N, int Q, int CT = 256>
struct Pencil2 {
  static constexpr int EB = CT / Q;         // elements per CTA (threadIdx.y) of CT threads
  static constexpr int PAD = Q + 1;         // row stride of a work field
  static constexpr int FS = Q * PAD;        // one work field
  static constexpr size_t bytes() { return sizeof(T) * (size_t)EB * 2 * FS; }
};

template <typename T, int N, int Q, bool GATHER, int CT = 256>
__global__ void __launch_bounds__(CT) helm2_pencil_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                           const PTabs<T, N, Q> tab, const T* __restrict__ jg,
                                                           T lambda, int E, const int* __restrict__ l2g, int ndir,
                                                           const int* __restrict__ skip,
                                                           const T* __restrict__ lam_ptr,
                                                           const int* __restrict__ esolve, int skip_stride) {
  using L = Pencil2<T, N, Q, CT>;
  constexpr int NM = N * N, NQ = Q * Q, PAD = L::PAD, FS = L::FS;
  if (esolve == nullptr && skip != nullptr && *skip) return;  // a converged solve: the whole CTA leaves
  if (lam_ptr != nullptr) lambda = *lam_ptr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* SA = reinterpret_cast<T*>(smem_raw) + threadIdx.y * 2 * FS;
  T* SB = SA + FS;
  const int t = threadIdx.x;
  const int e = blockIdx.x * L::EB + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const bool active = e < E && !(esolve != nullptr && skip[(size_t)esolve[ee] * skip_stride] != 0);
  if (esolve != nullptr && !__syncthreads_or(active)) return;  // every element's solve has converged

  // ---- rows q: gather and BwdTrans along p ----
  if (t < N) {
    T c[N];
#pragma unroll
    for (int p = 0; p < N; ++p) {
      const int m = t * N + p;
      if constexpr (GATHER) {
        const int code = l2g[(size_t)ee * NM + m];
        const int g = code >= 0 ? code : ~code;
        const T v = g < ndir ? T(0) : in[g];
        c[p] = code >= 0 ? v : -v;
      } else {
        c[p] = in[(size_t)ee * NM + m];
      }
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.B[i] * c[0];
#pragma unroll
      for (int p = 1; p < N; ++p) acc = fma(tab.B[p * Q + i], c[p], acc);
      SA[t * PAD + i] = acc;
    }
  }
  __syncthreads();
  // ---- columns i: BwdTrans along q, derivative along j ----
  T u[Q], g1[Q];
  {
    T a[N];
#pragma unroll
    for (int q = 0; q < N; ++q) a[q] = SA[q * PAD + t];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = tab.B[j] * a[0];
#pragma unroll
      for (int q = 1; q < N; ++q) acc = fma(tab.B[q * Q + j], a[q], acc);
      u[j] = acc;
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = tab.D[j] * u[0];
#pragma unroll
      for (int c = 1; c < Q; ++c) acc = fma(tab.D[c * Q + j], u[c], acc);
      g1[j] = acc;
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) SB[j * PAD + t] = u[j];
  }
  __syncthreads();
  // ---- rows j: derivative along i ----
  {
    T r[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) r[a] = SB[t * PAD + a];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.D[i] * r[0];
#pragma unroll
      for (int c = 1; c < Q; ++c) acc = fma(tab.D[c * Q + i], r[c], acc);
      SA[t * PAD + i] = acc;
    }
  }
  __syncthreads();
  // ---- columns i: metric, mass term, D^T along j ----
  T v[Q];
  {
    const T* G = jg + (size_t)ee * 4 * NQ;
    T f1[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const int pt = t + Q * j;
      const T g0 = SA[j * PAD + t];
      const T jw = G[pt], m00 = G[NQ + pt], m01 = G[2 * NQ + pt], m11 = G[3 * NQ + pt];
      SB[j * PAD + t] = fma(m00, g0, m01 * g1[j]);  // f0, handed to the rows
      f1[j] = fma(m01, g0, m11 * g1[j]);
      v[j] = lambda * jw * u[j];
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = v[j];
#pragma unroll
      for (int c = 0; c < Q; ++c) acc = fma(tab.D[j * Q + c], f1[c], acc);
      v[j] = acc;
    }
  }
  __syncthreads();
  // ---- rows j: D^T along i ----
  {
    T r[Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) r[c] = SB[t * PAD + c];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.D[i * Q] * r[0];
#pragma unroll
      for (int c = 1; c < Q; ++c) acc = fma(tab.D[i * Q + c], r[c], acc);
      SA[t * PAD + i] = acc;
    }
  }
  __syncthreads();
  // ---- columns i: sum, IProduct along j ----
  {
#pragma unroll
    for (int j = 0; j < Q; ++j) v[j] += SA[j * PAD + t];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      T acc = tab.B[q * Q] * v[0];
#pragma unroll
      for (int j = 1; j < Q; ++j) acc = fma(tab.B[q * Q + j], v[j], acc);
      SB[q * PAD + t] = acc;
    }
  }
  __syncthreads();
  // ---- rows q: IProduct along i, store ----
  if (t < N && active) {
    T y[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) y[i] = SB[t * PAD + i];
    T* o = out + (size_t)e * NM + t * N;
#pragma unroll
    for (int p = 0; p < N; ++p) {
      T acc = tab.B[p * Q] * y[0];
#pragma unroll
      for (int i = 1; i < Q; ++i) acc = fma(tab.B[p * Q + i], y[i], acc);
      o[p] = acc;
    }
  }
}

}  // namespace dev
}  // namespace ithaca
