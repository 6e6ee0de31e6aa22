// Sum-factorised element operators for tensor-product quads (DIM 2) and hexes (DIM 3).
//
// One group of TPE threads works on one element; a CTA holds EB such groups
// (blockDim = (TPE, EB)). The 1-D tables and the per-element tensors live in shared
// memory; every stage is a 1-D contraction along one direction
// (sum factorisation, as MatrixFreeOps/*Kernels.hpp do per SIMD lane).
//
// The Helmholtz operator uses the collocation form
//   out = B^T [ lambda Jw (B u) + sum_a D_a^T ( sum_b G_ab D_b (B u) ) ]
// with Jw = J w and G_ab = J w g^{ab} precomputed per quadrature point. It equals the
// reference composition (MatrixFreeOps/Helmholtz.h:137-275,763-993), which applies
// the derivative tables DB = D B inside three separate inner products, because
// IProduct_{DB_a}(f) = IProduct_B(D_a^T f); it needs fewer FP64 operations.
#pragma once

#include "ithaca_internal.h"

namespace ithaca {
namespace dev {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }
__host__ __device__ constexpr int cdiv(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ constexpr int tables_size(int n, int Q) { return 4 * n * Q + 2 * Q * Q + Q; }
__host__ __device__ constexpr int align_up(int x, int a) { return (x + a - 1) / a * a; }

// out[o] = sum_k A[k*M + m] in[...k...] along direction DIR; input extents
// (X0, X1, X2) with X_DIR == K, output extents equal except X_DIR -> M. X0 fastest.
template <typename T, int DIR, int K, int M, int X0, int X1, int X2>
__device__ __forceinline__ void contract(const T* __restrict__ in, T* __restrict__ out, const T* __restrict__ A,
                                         int t, int nt) {
  constexpr int O0 = DIR == 0 ? M : X0;
  constexpr int O1 = DIR == 1 ? M : X1;
  constexpr int O2 = DIR == 2 ? M : X2;
  constexpr int NOUT = O0 * O1 * O2;
  constexpr int S = DIR == 0 ? 1 : (DIR == 1 ? X0 : X0 * X1);
  for (int idx = t; idx < NOUT; idx += nt) {
    const int i0 = idx % O0;
    const int r = idx / O0;
    const int i1 = r % O1;
    const int i2 = r / O1;
    const int m = DIR == 0 ? i0 : (DIR == 1 ? i1 : i2);
    const int base = (DIR == 0 ? 0 : i0) + X0 * ((DIR == 1 ? 0 : i1) + X1 * (DIR == 2 ? 0 : i2));
    T acc = A[m] * in[base];
#pragma unroll
    for (int k = 1; k < K; ++k) acc = fma(A[k * M + m], in[base + k * S], acc);
    out[idx] = acc;
  }
}

// Coefficients (N^DIM, in C) -> values at points (Q^DIM, in U). Uses W0/W1 as scratch.
template <typename T, int DIM, int N, int Q>
__device__ __forceinline__ void bwd_stages(const T* C, T* W0, T* W1, T* U, const T* sB, int t, int nt) {
  if constexpr (DIM == 2) {
    contract<T, 0, N, Q, N, N, 1>(C, W0, sB, t, nt);
    __syncthreads();
    contract<T, 1, N, Q, Q, N, 1>(W0, U, sB, t, nt);
  } else {
    contract<T, 0, N, Q, N, N, N>(C, W0, sB, t, nt);
    __syncthreads();
    contract<T, 1, N, Q, Q, N, N>(W0, W1, sB, t, nt);
    __syncthreads();
    contract<T, 2, N, Q, Q, Q, N>(W1, U, sB, t, nt);
  }
}

// Values at points (Q^DIM, in V) -> inner products with the basis (N^DIM, in C).
template <typename T, int DIM, int N, int Q>
__device__ __forceinline__ void ipr_stages(const T* V, T* W0, T* W1, T* C, const T* sBt, int t, int nt) {
  if constexpr (DIM == 2) {
    contract<T, 0, Q, N, Q, Q, 1>(V, W0, sBt, t, nt);
    __syncthreads();
    contract<T, 1, Q, N, N, Q, 1>(W0, C, sBt, t, nt);
  } else {
    contract<T, 0, Q, N, Q, Q, Q>(V, W0, sBt, t, nt);
    __syncthreads();
    contract<T, 1, Q, N, N, Q, Q>(W0, W1, sBt, t, nt);
    __syncthreads();
    contract<T, 2, Q, N, N, N, Q>(W1, C, sBt, t, nt);
  }
}

template <typename T>
__device__ __forceinline__ void load_tables(T* s, const T* __restrict__ tab, int size) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nth = blockDim.x * blockDim.y;
  for (int i = tid; i < size; i += nth) s[i] = tab[i];
}

// Product of the quadrature weights at point p (regular elements fold them in here).
template <typename T, int DIM, int Q>
__device__ __forceinline__ T wprod(const T* sw, int p) {
  const int i = p % Q, j = (p / Q) % Q;
  T v = sw[i] * sw[j];
  if constexpr (DIM == 3) v *= sw[p / (Q * Q)];
  return v;
}

// Shared-memory layout of every kernel here: tables, then EB per-element slabs of
// (DIM + 1) * Q^DIM values (U, F0, F1[, F2]).
template <typename T, int DIM, int N, int Q>
struct Layout {
  static constexpr int NM = ipow(N, DIM);
  static constexpr int NQ = ipow(Q, DIM);
  static constexpr int TS = align_up(tables_size(N, Q), 4);
  static constexpr int SLAB = (DIM + 1) * NQ;
  static constexpr size_t bytes(int eb) { return sizeof(T) * ((size_t)TS + (size_t)eb * SLAB); }
};

// ---------------------------------------------------------------------------
// Helmholtz: out = lambda M u + L u on each element (optionally gathering u from a
// global vector through the signed local-to-global map, as AssemblyMapCG::GlobalToLocal).
template <typename T, int DIM, int N, int Q, int TPE, bool DEF, bool GATHER>
__global__ void __launch_bounds__(256) helm_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                    const T* __restrict__ tab, const T* __restrict__ jg, T lambda,
                                                    int E, const int* __restrict__ l2g, int ndir,
                                                    const int* __restrict__ skip, const T* __restrict__ lam_ptr,
                                                    const int* __restrict__ esolve, int skip_stride) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NM = L::NM, NQ = L::NQ, NG = n_jg(DIM);
  constexpr int PPT = cdiv(NQ, TPE);
  if (esolve == nullptr && skip != nullptr && *skip) return;  // a converged solve: the whole CTA leaves together
  if (lam_ptr != nullptr) lambda = *lam_ptr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  const T* sB = s + off_B(N, Q);
  const T* sBt = s + off_Bt(N, Q);
  const T* sD = s + off_D(N, Q);
  const T* sw = s + off_w(N, Q);
  load_tables(s, tab, tables_size(N, Q));
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* F2 = F1 + NQ;  // DIM 3 only
  T* C = DIM == 2 ? F1 : F2;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  // batched solves: elements of converged solves (skip[esolve[e] * skip_stride] != 0) do no I/O
  const bool active = e < E && !(esolve != nullptr && skip[(size_t)esolve[ee] * skip_stride] != 0);
  // a CTA whose elements all belong to converged solves leaves at once (as the batched
  // vector kernels skip converged chunks), so late iterations cost little
  if (esolve != nullptr && !__syncthreads_or(active)) return;

  const int t = threadIdx.x;

  for (int m = t; m < NM; m += TPE) {
    T v;
    if constexpr (GATHER) {
      const int code = l2g[(size_t)ee * NM + m];
      const int g = code >= 0 ? code : ~code;
      v = g < ndir ? T(0) : in[g];
      v = code >= 0 ? v : -v;
    } else {
      v = in[(size_t)ee * NM + m];
    }
    C[m] = v;
  }
  __syncthreads();
  bwd_stages<T, DIM, N, Q>(C, F0, F1, U, sB, t, TPE);
  __syncthreads();

  T mreg[PPT];
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
#pragma unroll
  for (int r = 0; r < PPT; ++r) {
    const int p = t + r * TPE;
    if (p < NQ) {
      const int i = p % Q, j = (p / Q) % Q;
      T g0 = 0, g1 = 0, g2 = 0;
#pragma unroll
      for (int a = 0; a < Q; ++a) {
        g0 = fma(sD[a * Q + i], U[p + (a - i)], g0);
        g1 = fma(sD[a * Q + j], U[p + (a - j) * Q], g1);
      }
      if constexpr (DIM == 3) {
        const int k = p / (Q * Q);
#pragma unroll
        for (int a = 0; a < Q; ++a) g2 = fma(sD[a * Q + k], U[p + (a - k) * Q * Q], g2);
      }
      T jw, m[6];
      if constexpr (DEF) {
        jw = gbase[p];
#pragma unroll
        for (int c = 1; c < NG; ++c) m[c - 1] = gbase[c * NQ + p];
      } else {
        const T wp = wprod<T, DIM, Q>(sw, p);
        jw = gbase[0] * wp;
#pragma unroll
        for (int c = 1; c < NG; ++c) m[c - 1] = gbase[c] * wp;
      }
      if constexpr (DIM == 2) {
        F0[p] = fma(m[0], g0, m[1] * g1);
        F1[p] = fma(m[1], g0, m[2] * g1);
      } else {
        F0[p] = fma(m[0], g0, fma(m[1], g1, m[2] * g2));
        F1[p] = fma(m[1], g0, fma(m[3], g1, m[4] * g2));
        F2[p] = fma(m[2], g0, fma(m[4], g1, m[5] * g2));
      }
      mreg[r] = lambda * jw * U[p];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PPT; ++r) {
    const int p = t + r * TPE;
    if (p < NQ) {
      const int i = p % Q, j = (p / Q) % Q;
      T v = mreg[r];
#pragma unroll
      for (int a = 0; a < Q; ++a) {
        v = fma(sD[i * Q + a], F0[p + (a - i)], v);
        v = fma(sD[j * Q + a], F1[p + (a - j) * Q], v);
      }
      if constexpr (DIM == 3) {
        const int k = p / (Q * Q);
#pragma unroll
        for (int a = 0; a < Q; ++a) v = fma(sD[k * Q + a], F2[p + (a - k) * Q * Q], v);
      }
      U[p] = v;
    }
  }
  __syncthreads();
  ipr_stages<T, DIM, N, Q>(U, F0, F1, C, sBt, t, TPE);
  __syncthreads();
  if (active)
    for (int m = t; m < NM; m += TPE) out[(size_t)e * NM + m] = C[m];
}

// ---------------------------------------------------------------------------
template <typename T, int DIM, int N, int Q, int TPE>
__global__ void __launch_bounds__(256) bwd_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                   const T* __restrict__ tab, int E) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NM = L::NM, NQ = L::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, tables_size(N, Q));
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* C = F1 + (DIM == 3 ? NQ : 0);
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool active = e < E;
  const int ee = active ? e : E - 1;
  const int t = threadIdx.x;
  for (int m = t; m < NM; m += TPE) C[m] = in[(size_t)ee * NM + m];
  __syncthreads();
  bwd_stages<T, DIM, N, Q>(C, F0, F1, U, s + off_B(N, Q), t, TPE);
  __syncthreads();
  if (active)
    for (int p = t; p < NQ; p += TPE) out[(size_t)e * NQ + p] = U[p];
}

template <typename T, int DIM, int N, int Q, int TPE, bool DEF>
__global__ void __launch_bounds__(256) ipr_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                   const T* __restrict__ tab, const T* __restrict__ jg, int E) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NM = L::NM, NQ = L::NQ, NG = n_jg(DIM);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, tables_size(N, Q));
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* C = F1 + (DIM == 3 ? NQ : 0);
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool active = e < E;
  const int ee = active ? e : E - 1;
  const int t = threadIdx.x;
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
  __syncthreads();
  for (int p = t; p < NQ; p += TPE) {
    const T jw = DEF ? gbase[p] : gbase[0] * wprod<T, DIM, Q>(s + off_w(N, Q), p);
    U[p] = jw * in[(size_t)ee * NQ + p];
  }
  __syncthreads();
  ipr_stages<T, DIM, N, Q>(U, F0, F1, C, s + off_Bt(N, Q), t, TPE);
  __syncthreads();
  if (active)
    for (int m = t; m < NM; m += TPE) out[(size_t)e * NM + m] = C[m];
}

template <typename T, int DIM, int N, int Q, int TPE, bool DEF>
__global__ void __launch_bounds__(256) deriv_kernel(const T* __restrict__ in, T* __restrict__ d0,
                                                     T* __restrict__ d1, T* __restrict__ d2,
                                                     const T* __restrict__ tab, const T* __restrict__ df, int E) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NQ = L::NQ, ND = DIM * DIM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, tables_size(N, Q));
  const T* sD = s + off_D(N, Q);
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool active = e < E;
  const int ee = active ? e : E - 1;
  const int t = threadIdx.x;
  for (int p = t; p < NQ; p += TPE) U[p] = in[(size_t)ee * NQ + p];
  __syncthreads();
  if (!active) return;
  const T* fbase = df + (size_t)ee * ND * (DEF ? NQ : 1);
  for (int p = t; p < NQ; p += TPE) {
    const int i = p % Q, j = (p / Q) % Q;
    T g[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < Q; ++a) {
      g[0] = fma(sD[a * Q + i], U[p + (a - i)], g[0]);
      g[1] = fma(sD[a * Q + j], U[p + (a - j) * Q], g[1]);
    }
    if constexpr (DIM == 3) {
      const int k = p / (Q * Q);
#pragma unroll
      for (int a = 0; a < Q; ++a) g[2] = fma(sD[a * Q + k], U[p + (a - k) * Q * Q], g[2]);
    }
    T* outs[3] = {d0, d1, d2};
#pragma unroll
    for (int kx = 0; kx < DIM; ++kx) {
      T v = 0;
#pragma unroll
      for (int jx = 0; jx < DIM; ++jx) {
        const T f = DEF ? fbase[(kx * DIM + jx) * NQ + p] : fbase[kx * DIM + jx];
        v = fma(f, g[jx], v);
      }
      outs[kx][(size_t)e * NQ + p] = v;
    }
  }
}

// IProductWRTDerivBase: out = sum_k (d phi / d x_k, in_k) on each element, i.e. with
// F_j = J w sum_k (d xi_j / d x_k) in_k at the points, out = sum_j B^T D_j^T F_j (the
// reference's IProductWRTDerivBase_IterPerExp, Collections/IProductWRTDerivBase.cpp:446-546:
// tmp[j] = sum_k derivFac[j + k d] in[k], times jac, then StdExpansion::IProductWRTDerivBase
// per direction). Geometry: df as deriv_kernel reads it, J w as field 0 of jg.
template <typename T, int DIM, int N, int Q, int TPE, bool DEF>
__global__ void __launch_bounds__(256) iprd_kernel(const T* __restrict__ in0, const T* __restrict__ in1,
                                                    const T* __restrict__ in2, T* __restrict__ out,
                                                    const T* __restrict__ tab, const T* __restrict__ jg,
                                                    const T* __restrict__ df, int E) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NM = L::NM, NQ = L::NQ, NG = n_jg(DIM), ND = DIM * DIM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, tables_size(N, Q));
  const T* sD = s + off_D(N, Q);
  const T* sw = s + off_w(N, Q);
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* F2 = F1 + NQ;  // DIM 3 only
  T* C = DIM == 2 ? F1 : F2;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool active = e < E;
  const int ee = active ? e : E - 1;
  const int t = threadIdx.x;
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
  const T* fbase = df + (size_t)ee * ND * (DEF ? NQ : 1);
  const T* ins[3] = {in0, in1, in2};
  __syncthreads();  // tables
  for (int p = t; p < NQ; p += TPE) {
    const T jw = DEF ? gbase[p] : gbase[0] * wprod<T, DIM, Q>(sw, p);
    T f[3];
#pragma unroll
    for (int kx = 0; kx < DIM; ++kx) f[kx] = ins[kx][(size_t)ee * NQ + p];
    T* Fs[3] = {F0, F1, F2};
#pragma unroll
    for (int jx = 0; jx < DIM; ++jx) {
      T v = 0;
#pragma unroll
      for (int kx = 0; kx < DIM; ++kx) {
        const T d = DEF ? fbase[(kx * DIM + jx) * NQ + p] : fbase[kx * DIM + jx];
        v = fma(d, f[kx], v);
      }
      Fs[jx][p] = jw * v;
    }
  }
  __syncthreads();
  for (int p = t; p < NQ; p += TPE) {
    const int i = p % Q, j = (p / Q) % Q;
    T v = 0;
#pragma unroll
    for (int a = 0; a < Q; ++a) {
      v = fma(sD[i * Q + a], F0[p + (a - i)], v);
      v = fma(sD[j * Q + a], F1[p + (a - j) * Q], v);
    }
    if constexpr (DIM == 3) {
      const int k = p / (Q * Q);
#pragma unroll
      for (int a = 0; a < Q; ++a) v = fma(sD[k * Q + a], F2[p + (a - k) * Q * Q], v);
    }
    U[p] = v;
  }
  __syncthreads();
  ipr_stages<T, DIM, N, Q>(U, F0, F1, C, s + off_Bt(N, Q), t, TPE);
  __syncthreads();
  if (active)
    for (int m = t; m < NM; m += TPE) out[(size_t)e * NM + m] = C[m];
}

// Diagonal of the element Helmholtz matrix: for mode m = (p, q[, r]),
//   lambda sum Jw phi_m^2 + sum_ab sum G_ab (d_a phi_m)(d_b phi_m),
// every term a separable weighted inner product with squared / mixed 1-D tables.
template <typename T, int DIM, int N, int Q, int TPE, bool DEF>
__global__ void __launch_bounds__(256) diag_kernel(T* __restrict__ out, const T* __restrict__ tab,
                                                    const T* __restrict__ jg, T lambda, int E) {
  using L = Layout<T, DIM, N, Q>;
  constexpr int NM = L::NM, NQ = L::NQ, NG = n_jg(DIM);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, tables_size(N, Q));
  // squared tables in the slab area after the per-element buffers
  T* U = s + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* C = F1 + (DIM == 3 ? NQ : 0);
  __shared__ T sq[3][Q * N];  // BB^t, DD^t, BD^t in [i*N + p] order
  {
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const T* Bt = s + off_Bt(N, Q);
    const T* DBt = s + off_DBt(N, Q);
    __syncthreads();
    for (int i = tid; i < Q * N; i += blockDim.x * blockDim.y) {
      sq[0][i] = Bt[i] * Bt[i];
      sq[1][i] = DBt[i] * DBt[i];
      sq[2][i] = Bt[i] * DBt[i];
    }
  }
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool active = e < E;
  const int ee = active ? e : E - 1;
  const int t = threadIdx.x;
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
  T acc[cdiv(NM, TPE)];
#pragma unroll
  for (int r = 0; r < cdiv(NM, TPE); ++r) acc[r] = 0;
  // term list: field index c (0 = Jw, 1.. = G upper triangle), table choice per direction
  constexpr int NT = NG;
  for (int term = 0; term < NT; ++term) {
    int ta[3] = {0, 0, 0};
    T scale = 1;
    if (term == 0) {
      scale = lambda;
    } else {
      // map term -> (a, b) in the upper triangle order (00, 01, [02,] 11, [12,] 22)
      int a = 0, b = 0, cnt = 1;
      for (int x = 0; x < DIM; ++x)
        for (int y = x; y < DIM; ++y) {
          if (cnt == term) { a = x; b = y; }
          ++cnt;
        }
      if (a == b) {
        ta[a] = 1;
      } else {
        ta[a] = 2;
        ta[b] = 2;
        scale = 2;
      }
    }
    __syncthreads();
    for (int p = t; p < NQ; p += TPE) {
      const T wp = DEF ? T(1) : wprod<T, DIM, Q>(s + off_w(N, Q), p);
      U[p] = scale * wp * (DEF ? gbase[term * NQ + p] : gbase[term]);
    }
    __syncthreads();
    if constexpr (DIM == 2) {
      contract<T, 0, Q, N, Q, Q, 1>(U, F0, sq[ta[0]], t, TPE);
      __syncthreads();
      contract<T, 1, Q, N, N, Q, 1>(F0, C, sq[ta[1]], t, TPE);
    } else {
      contract<T, 0, Q, N, Q, Q, Q>(U, F0, sq[ta[0]], t, TPE);
      __syncthreads();
      contract<T, 1, Q, N, N, Q, Q>(F0, F1, sq[ta[1]], t, TPE);
      __syncthreads();
      contract<T, 2, Q, N, N, N, Q>(F1, C, sq[ta[2]], t, TPE);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < cdiv(NM, TPE); ++r) {
      const int m = t + r * TPE;
      if (m < NM) acc[r] += C[m];
    }
  }
  if (active) {
#pragma unroll
    for (int r = 0; r < cdiv(NM, TPE); ++r) {
      const int m = t + r * TPE;
      if (m < NM) out[(size_t)e * NM + m] = acc[r];
    }
  }
}

// Threads per element and elements per CTA for each shape / order.
template <int DIM, int Q>
struct Shape {
  static constexpr int NQ = ipow(Q, DIM);
  static constexpr int TPE = DIM == 3 ? (NQ <= 256 ? 128 : 256) : (NQ <= 64 ? 32 : 64);
  static constexpr int EB = DIM == 3 ? 1 : 256 / TPE;
};

}  // namespace dev
}  // namespace ithaca
