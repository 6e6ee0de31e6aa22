// Sum-factorised element operators for tetrahedra in collapsed coordinates.
//
// Expansion: ModifiedA on Q0 = N + 1 GLL points (eta0), ModifiedB on Q = N Gauss-Radau
// (alpha 1) points (eta1), ModifiedC on Q = N Gauss-Radau (alpha 2) points (eta2);
// NC = N (N+1) (N+2) / 6 modes m(p, q, r), r fastest; pairs pq(p, q), q fastest, index the
// ModifiedB rows. Values at points u[(k Q + j) Q0 + i].
//
// The reference kernels (MatrixFreeOps/BwdTransKernels.hpp:374-480 BwdTransTetKernel,
// IProductKernels.hpp:601-790 IProductTetKernel, PhysDerivKernels.hpp:555-700,
// Helmholtz.h:2266-2448 HelmholtzTetImpl) work per SIMD lane; here a group of TPE threads
// works on one element with its tensors in shared memory:
//   BwdTrans   F[pq][k] = sum_r B2[m][k] c[m];  G[p][j][k] = sum_q B1[pq][j] F[pq][k];
//              u[k][j][i] = sum_p B0[p][i] G[p][j][k]. The CORRECT terms (top vertex m = 1,
//              bottom vertex m = N, singular edge m = N + r) are folded into the p = 0 and
//              p = 1 rows of G: the modes (0, 1, r) also carry B0[1] (their eta0 factor is
//              B0[0] + B0[1] = 1), and the top vertex is B2[1] (B0[0] + B0[1]) (B1[0] + B1[1]).
//              The reference adds them with the rows B2[0] and B2[r + 1], which hold the
//              same functions as B2[m(0, 1, r)] (phi^c_{pqr} = phi^b_{p+q,r}).
//   IProduct   the transpose of those three contractions and of the folded terms.
//   Helmholtz  the collocation form: out = IProduct(lambda Jw u + sum_a D_a^T G_a),
//              G_a = sum_b Jw m^{ab} d_b with the collapsed derivatives d_b and the metric
//              of HelmholtzTetImpl (built per point by build_jg_tet_kernel).
// Shared memory per element: four tensors of NQ = Q0 Q^2 values (U, F0, F1, F2); the
// BwdTrans / IProduct work arrays (G of N Q^2, F of NPQ Q, C of NC) reuse F0, F1, F2.
#pragma once

#include <type_traits>

#include "elem.cuh"

namespace ithaca {
namespace dev {

template <int N>
struct TetShape {
  static constexpr int Q0 = N + 1, Q = N, NC = N * (N + 1) * (N + 2) / 6, NPQ = N * (N + 1) / 2;
  static constexpr int NQ = Q0 * Q * Q;
  static constexpr TetOff O = tet_off(N);
  static constexpr int TS = align_up(O.core, 4);  // tables the operators read
  static constexpr int TSD = align_up(O.size, 4);  // with DB0, DB1, DB2 (diagonal)
  static constexpr int SLAB = 4 * NQ;
  static constexpr int TPE = NQ <= 32 ? 32 : (NQ <= 64 ? 64 : 128);  // larger elements: two per CTA
  static constexpr int EB = 256 / TPE;
  template <typename T>
  static constexpr size_t bytes() {
    return sizeof(T) * ((size_t)TS + (size_t)EB * SLAB);
  }
};

// Pair index of (p, 0) and mode index of (p, 0, 0).
template <int N>
__device__ __forceinline__ int tet_pq0(int p) {
  return p * N - p * (p - 1) / 2;
}
template <int N>
__device__ __forceinline__ int tet_m0(int p) {
  int m = 0;
#pragma unroll 1
  for (int pp = 0; pp < p; ++pp) m += (N - pp) * (N - pp + 1) / 2;
  return m;
}
// (p, q) of pair pq.
template <int N>
__device__ __forceinline__ void tet_pair(int pq, int& p, int& q) {
  p = 0;
#pragma unroll 1
  while (p < N - 1 && pq >= tet_pq0<N>(p + 1)) ++p;
  q = pq - tet_pq0<N>(p);
}
// (p, q, r) and pair of mode m.
template <int N>
__device__ __forceinline__ void tet_mode(int m, int& p, int& q, int& r, int& pq) {
  p = 0;
#pragma unroll 1
  while (p < N - 1 && m >= tet_m0<N>(p + 1)) ++p;
  int rest = m - tet_m0<N>(p);
  q = 0;
#pragma unroll 1
  while (rest >= N - p - q) {
    rest -= N - p - q;
    ++q;
  }
  r = rest;
  pq = tet_pq0<N>(p) + q;
}

// Coefficients C (NC) -> values U (NQ); F (NPQ Q) and G (N Q^2) are scratch.
template <typename T, int N>
__device__ __forceinline__ void tet_bwd_stages(const T* C, T* F, T* G, T* U, const T* s, int t, int nt) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NPQ = S::NPQ;
  const T* B0 = s + S::O.B0;
  const T* B1 = s + S::O.B1;
  const T* B2 = s + S::O.B2;
  for (int idx = t; idx < NPQ * Q; idx += nt) {
    const int pq = idx / Q, k = idx - pq * Q;
    int p, q;
    tet_pair<N>(pq, p, q);
    const int m0 = tet_m0<N>(p) + q * (N - p) - q * (q - 1) / 2;
    const int len = N - p - q;
    T acc = 0;
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r < len) acc = fma(B2[(m0 + r) * Q + k], C[m0 + r], acc);
    F[idx] = acc;
  }
  __syncthreads();
  for (int idx = t; idx < N * Q * Q; idx += nt) {
    const int p = idx / (Q * Q), j = (idx / Q) % Q, k = idx % Q;
    const int pq0 = tet_pq0<N>(p);
    T acc = 0;
#pragma unroll
    for (int q = 0; q < N; ++q)
      if (q < N - p) acc = fma(B1[(pq0 + q) * Q + j], F[(pq0 + q) * Q + k], acc);
    if (p == 0) acc = fma(C[1] * B2[Q + k], B1[Q + j], acc);
    if (p == 1) {
      acc = fma(B1[Q + j], F[Q + k], acc);
      acc = fma(C[1] * B2[Q + k], B1[j] + B1[Q + j], acc);
    }
    G[idx] = acc;
  }
  __syncthreads();
  for (int idx = t; idx < S::NQ; idx += nt) {
    const int i = idx % Q0, j = (idx / Q0) % Q, k = idx / (Q0 * Q);
    T acc = 0;
#pragma unroll
    for (int p = 0; p < N; ++p) acc = fma(B0[p * Q0 + i], G[(p * Q + j) * Q + k], acc);
    U[idx] = acc;
  }
}

// Weighted values V (NQ) -> inner products C (NC) with tables A0, A1, A2.
template <typename T, int N>
__device__ __forceinline__ void tet_ipr_stages(const T* V, T* G, T* F, T* C, const T* A0, const T* A1, const T* A2,
                                               int t, int nt) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NPQ = S::NPQ, NC = S::NC;
  for (int idx = t; idx < N * Q * Q; idx += nt) {
    const int p = idx / (Q * Q), j = (idx / Q) % Q, k = idx % Q;
    T acc = 0;
#pragma unroll
    for (int i = 0; i < Q0; ++i) acc = fma(A0[p * Q0 + i], V[(k * Q + j) * Q0 + i], acc);
    G[idx] = acc;
  }
  __syncthreads();
  for (int idx = t; idx < NPQ * Q; idx += nt) {
    const int pq = idx / Q, k = idx - pq * Q;
    int p, q;
    tet_pair<N>(pq, p, q);
    T acc = 0;
#pragma unroll
    for (int j = 0; j < Q; ++j) acc = fma(A1[pq * Q + j], G[(p * Q + j) * Q + k], acc);
    if (pq == 1) {
#pragma unroll
      for (int j = 0; j < Q; ++j) acc = fma(A1[Q + j], G[(Q + j) * Q + k], acc);
    }
    F[idx] = acc;
  }
  __syncthreads();
  for (int m = t; m < NC; m += nt) {
    int p, q, r, pq;
    tet_mode<N>(m, p, q, r, pq);
    T acc = 0;
#pragma unroll
    for (int k = 0; k < Q; ++k) acc = fma(A2[m * Q + k], F[pq * Q + k], acc);
    if (m == 1) {
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        T g = 0;
#pragma unroll
        for (int j = 0; j < Q; ++j) {
          g = fma(A1[Q + j], G[j * Q + k], g);
          g = fma(A1[j] + A1[Q + j], G[(Q + j) * Q + k], g);
        }
        acc = fma(A2[Q + k], g, acc);
      }
    }
    C[m] = acc;
  }
}

// Collapsed derivatives of U at point (i, j, k).
template <typename T, int N>
__device__ __forceinline__ void tet_dcollapsed(const T* U, const T* s, int i, int j, int k, T& d0, T& d1, T& d2) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q;
  const T* D0 = s + S::O.D0;
  const T* D1 = s + S::O.D1;
  const T* D2 = s + S::O.D2;
  d0 = 0;
  d1 = 0;
  d2 = 0;
#pragma unroll
  for (int a = 0; a < Q0; ++a) d0 = fma(D0[a * Q0 + i], U[(k * Q + j) * Q0 + a], d0);
#pragma unroll
  for (int a = 0; a < Q; ++a) d1 = fma(D1[a * Q + j], U[(k * Q + a) * Q0 + i], d1);
#pragma unroll
  for (int a = 0; a < Q; ++a) d2 = fma(D2[a * Q + k], U[(a * Q + j) * Q0 + i], d2);
}

// sum_a D_a^T F_a at point (i, j, k).
template <typename T, int N>
__device__ __forceinline__ T tet_dtrans(const T* F0, const T* F1, const T* F2, const T* s, int i, int j, int k, T v) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q;
  const T* D0 = s + S::O.D0;
  const T* D1 = s + S::O.D1;
  const T* D2 = s + S::O.D2;
#pragma unroll
  for (int a = 0; a < Q0; ++a) v = fma(D0[i * Q0 + a], F0[(k * Q + j) * Q0 + a], v);
#pragma unroll
  for (int a = 0; a < Q; ++a) v = fma(D1[j * Q + a], F1[(k * Q + a) * Q0 + i], v);
#pragma unroll
  for (int a = 0; a < Q; ++a) v = fma(D2[k * Q + a], F2[(a * Q + j) * Q0 + i], v);
  return v;
}

// ---------------------------------------------------------------------------
template <typename T, int N, int TPE, bool GATHER>
__global__ void __launch_bounds__(256) tet_helm_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                        const T* __restrict__ tab, const T* __restrict__ jg,
                                                        T lambda, int E, const int* __restrict__ l2g, int ndir,
                                                        const int* __restrict__ skip, const T* __restrict__ lam_ptr) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NC = S::NC, NQ = S::NQ;
  constexpr int PPT = cdiv(NQ, TPE);
  if (skip != nullptr && *skip) return;
  if (lam_ptr != nullptr) lambda = *lam_ptr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.core);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* F2 = F1 + NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  for (int m = t; m < NC; m += TPE) {
    T v;
    if constexpr (GATHER) {
      const int code = l2g[(size_t)ee * NC + m];
      const int g = code >= 0 ? code : ~code;
      v = g < ndir ? T(0) : in[g];
      v = code >= 0 ? v : -v;
    } else {
      v = in[(size_t)ee * NC + m];
    }
    F2[m] = v;
  }
  __syncthreads();
  tet_bwd_stages<T, N>(F2, F1, F0, U, s, t, TPE);
  __syncthreads();
  T mreg[PPT];
  const T* g = jg + (size_t)ee * 7 * NQ;
#pragma unroll
  for (int rr = 0; rr < PPT; ++rr) {
    const int p = t + rr * TPE;
    if (p < NQ) {
      const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
      T d0, d1, d2;
      tet_dcollapsed<T, N>(U, s, i, j, k, d0, d1, d2);
      const T g00 = g[NQ + p], g01 = g[2 * NQ + p], g02 = g[3 * NQ + p];
      const T g11 = g[4 * NQ + p], g12 = g[5 * NQ + p], g22 = g[6 * NQ + p];
      F0[p] = fma(g00, d0, fma(g01, d1, g02 * d2));
      F1[p] = fma(g01, d0, fma(g11, d1, g12 * d2));
      F2[p] = fma(g02, d0, fma(g12, d1, g22 * d2));
      mreg[rr] = lambda * g[p] * U[p];
    }
  }
  __syncthreads();
#pragma unroll
  for (int rr = 0; rr < PPT; ++rr) {
    const int p = t + rr * TPE;
    if (p < NQ) {
      const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
      U[p] = tet_dtrans<T, N>(F0, F1, F2, s, i, j, k, mreg[rr]);
    }
  }
  __syncthreads();
  tet_ipr_stages<T, N>(U, F0, F1, F2, s + S::O.B0, s + S::O.B1, s + S::O.B2, t, TPE);
  __syncthreads();
  if (e < E)
    for (int m = t; m < NC; m += TPE) out[(size_t)e * NC + m] = F2[m];
}

template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tet_bwd_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                       const T* __restrict__ tab, int E) {
  using S = TetShape<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.core);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* G = U + S::NQ;
  T* F = G + S::NQ;
  T* C = F + S::NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  for (int m = t; m < S::NC; m += TPE) C[m] = in[(size_t)ee * S::NC + m];
  __syncthreads();
  tet_bwd_stages<T, N>(C, F, G, U, s, t, TPE);
  __syncthreads();
  if (e < E)
    for (int p = t; p < S::NQ; p += TPE) out[(size_t)e * S::NQ + p] = U[p];
}

template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tet_ipr_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                       const T* __restrict__ tab, const T* __restrict__ jg, int E) {
  using S = TetShape<N>;
  constexpr int NQ = S::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.core);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* G = U + NQ;
  T* F = G + NQ;
  T* C = F + NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  const T* g = jg + (size_t)ee * 7 * NQ;
  for (int p = t; p < NQ; p += TPE) U[p] = in[(size_t)ee * NQ + p] * g[p];
  __syncthreads();
  tet_ipr_stages<T, N>(U, G, F, C, s + S::O.B0, s + S::O.B1, s + S::O.B2, t, TPE);
  __syncthreads();
  if (e < E)
    for (int m = t; m < S::NC; m += TPE) out[(size_t)e * S::NC + m] = C[m];
}

// PhysDeriv (PhysDerivTetKernel): d/dxi0 = h2 h3 d0, d/dxi1 = h0 d/dxi0 + h3 d1,
// d/dxi2 = h0 d/dxi0 + h1 h3 d1 + d2, then the nine derivative factors.
template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tet_deriv_kernel(const T* __restrict__ in, T* __restrict__ o0,
                                                         T* __restrict__ o1, T* __restrict__ o2,
                                                         const T* __restrict__ tab, const T* __restrict__ df, int E) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NQ = S::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.core);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  for (int p = t; p < NQ; p += TPE) U[p] = in[(size_t)ee * NQ + p];
  __syncthreads();
  if (e >= E) return;
  const T* f = df + (size_t)e * 9 * NQ;
  for (int p = t; p < NQ; p += TPE) {
    const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
    T d0, d1, d2;
    tet_dcollapsed<T, N>(U, s, i, j, k, d0, d1, d2);
    const T h0 = s[S::O.h0 + i], h1 = s[S::O.h1 + j], h2 = s[S::O.h2 + j], h3 = s[S::O.h3 + k];
    const T x0 = h2 * h3 * d0;
    const T x1 = fma(h0, x0, h3 * d1);
    const T x2 = fma(h0, x0, fma(h1 * h3, d1, d2));
    T* o[3] = {o0, o1, o2};
#pragma unroll
    for (int c = 0; c < 3; ++c)
      o[c][(size_t)e * NQ + p] =
          fma(f[(3 * c) * NQ + p], x0, fma(f[(3 * c + 1) * NQ + p], x1, f[(3 * c + 2) * NQ + p] * x2));
  }
}

// IProductWRTDerivBase: t_j = sum_c df[c*3+j] in_c; G0 = Jw h2 h3 (t0 + h0 (t1 + t2)),
// G1 = Jw h3 (t1 + h1 t2), G2 = Jw t2; out = IProduct(sum_a D_a^T G_a).
template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tet_iprd_kernel(const T* __restrict__ in0, const T* __restrict__ in1,
                                                        const T* __restrict__ in2, T* __restrict__ out,
                                                        const T* __restrict__ tab, const T* __restrict__ jg,
                                                        const T* __restrict__ df, int E) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NQ = S::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.core);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* F2 = F1 + NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  const T* g = jg + (size_t)ee * 7 * NQ;
  const T* f = df + (size_t)ee * 9 * NQ;
  for (int p = t; p < NQ; p += TPE) {
    const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
    const size_t gi = (size_t)ee * NQ + p;
    const T a = in0[gi], b = in1[gi], c = in2[gi];
    T tj[3];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
      tj[jj] = fma(f[jj * NQ + p], a, fma(f[(3 + jj) * NQ + p], b, f[(6 + jj) * NQ + p] * c));
    const T h0 = s[S::O.h0 + i], h1 = s[S::O.h1 + j], h2 = s[S::O.h2 + j], h3 = s[S::O.h3 + k];
    const T jw = g[p];
    F0[p] = jw * h2 * h3 * fma(h0, tj[1] + tj[2], tj[0]);
    F1[p] = jw * h3 * fma(h1, tj[2], tj[1]);
    F2[p] = jw * tj[2];
  }
  __syncthreads();
  for (int p = t; p < NQ; p += TPE) {
    const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
    U[p] = tet_dtrans<T, N>(F0, F1, F2, s, i, j, k, T(0));
  }
  __syncthreads();
  tet_ipr_stages<T, N>(U, F0, F1, F2, s + S::O.B0, s + S::O.B1, s + S::O.B2, t, TPE);
  __syncthreads();
  if (e < E)
    for (int m = t; m < S::NC; m += TPE) out[(size_t)e * S::NC + m] = F2[m];
}

// Diagonal of each element's Helmholtz matrix. Every mode is a product X(i) Y(j) Z(k):
// X = B0[p], Y = B1[pq], Z = B2[m], except X = B0[0] + B0[1] for the modes (0, 1, r) and
// (0, 0, 1), and Y = B1[0] + B1[1] for (0, 0, 1) (the folded CORRECT terms).
template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tet_diag_kernel(T* __restrict__ out, const T* __restrict__ tab,
                                                        const T* __restrict__ jg, T lambda, int E) {
  using S = TetShape<N>;
  constexpr int Q0 = S::Q0, Q = S::Q, NQ = S::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  __syncthreads();
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  if (e >= E) return;
  const T* g = jg + (size_t)e * 7 * NQ;
  for (int m = threadIdx.x; m < S::NC; m += TPE) {
    int p, q, r, pq;
    tet_mode<N>(m, p, q, r, pq);
    const bool sumx = p == 0 && (q == 1 || (q == 0 && r == 1));
    const bool sumy = m == 1;
    T acc = 0;
    for (int k = 0; k < Q; ++k) {
      const T z = s[S::O.B2 + m * Q + k], dz = s[S::O.DB2 + m * Q + k];
      for (int j = 0; j < Q; ++j) {
        T y = s[S::O.B1 + pq * Q + j], dy = s[S::O.DB1 + pq * Q + j];
        if (sumy) {
          y = s[S::O.B1 + j] + s[S::O.B1 + Q + j];
          dy = s[S::O.DB1 + j] + s[S::O.DB1 + Q + j];
        }
        for (int i = 0; i < Q0; ++i) {
          T x = s[S::O.B0 + p * Q0 + i], dx = s[S::O.DB0 + p * Q0 + i];
          if (sumx) {
            x = s[S::O.B0 + i] + s[S::O.B0 + Q0 + i];
            dx = s[S::O.DB0 + i] + s[S::O.DB0 + Q0 + i];
          }
          const int pt = (k * Q + j) * Q0 + i;
          const T ph = x * y * z, a0 = dx * y * z, a1 = x * dy * z, a2 = x * y * dz;
          acc = fma(lambda * g[pt] * ph, ph, acc);
          acc = fma(g[NQ + pt] * a0, a0, acc);
          acc = fma(g[4 * NQ + pt] * a1, a1, acc);
          acc = fma(g[6 * NQ + pt] * a2, a2, acc);
          acc = fma(T(2) * g[2 * NQ + pt] * a0, a1, acc);
          acc = fma(T(2) * g[3 * NQ + pt] * a0, a2, acc);
          acc = fma(T(2) * g[5 * NQ + pt] * a1, a2, acc);
        }
      }
    }
    out[(size_t)e * S::NC + m] = acc;
  }
}

// ---------------------------------------------------------------------------
template <typename T, int N>
struct TetCfg {
  using S = TetShape<N>;
  static dim3 block() { return dim3(S::TPE, S::EB); }
  static dim3 grid(int E) { return dim3((E + S::EB - 1) / S::EB); }
  static size_t smem() { return S::template bytes<T>(); }
  template <class K>
  static void prep(K k, size_t bytes) {
    static bool done = false;
    if (!done) {
      ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
      done = true;
    }
  }
};

template <typename T, int N>
void tet_helm_n(int E, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g, int ndir,
                const int* skip, const T* lam_ptr, cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = l2g ? tet_helm_kernel<T, N, C::S::TPE, true> : tet_helm_kernel<T, N, C::S::TPE, false>;
  C::prep(k, C::smem());
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, lambda, E, l2g, ndir, skip, lam_ptr);
}

template <typename T, int N>
void tet_bwd_n(int E, const T* tab, const T* in, T* out, cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = tet_bwd_kernel<T, N, C::S::TPE>;
  C::prep(k, C::smem());
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, E);
}

template <typename T, int N>
void tet_ipr_n(int E, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = tet_ipr_kernel<T, N, C::S::TPE>;
  C::prep(k, C::smem());
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, E);
}

template <typename T, int N>
void tet_deriv_n(int E, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2, cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = tet_deriv_kernel<T, N, C::S::TPE>;
  C::prep(k, C::smem());
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, d0, d1, d2, tab, df, E);
}

template <typename T, int N>
void tet_iprd_n(int E, const T* tab, const T* jg, const T* df, const T* in0, const T* in1, const T* in2, T* out,
                cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = tet_iprd_kernel<T, N, C::S::TPE>;
  C::prep(k, C::smem());
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in0, in1, in2, out, tab, jg, df, E);
}

template <typename T, int N>
void tet_diag_n(int E, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s) {
  using C = TetCfg<T, N>;
  auto k = tet_diag_kernel<T, N, C::S::TPE>;
  const size_t bytes = sizeof(T) * (size_t)C::S::TSD;
  C::prep(k, bytes);
  k<<<C::grid(E), C::block(), bytes, s>>>(out, tab, jg, lambda, E);
}

}  // namespace dev

#define ITHACA_TET_CALL(NN) call(std::integral_constant<int, NN>{})

// Runs CALL(N) for 2 <= n <= 10 with Q == n + 1; false otherwise.
#define ITHACA_TET_DISPATCH(n, Q, CALL)        \
  if ((Q) != (n) + 1) return false;            \
  switch (n) {                                 \
    case 2: CALL(2); return true;              \
    case 3: CALL(3); return true;              \
    case 4: CALL(4); return true;              \
    case 5: CALL(5); return true;              \
    case 6: CALL(6); return true;              \
    case 7: CALL(7); return true;              \
    case 8: CALL(8); return true;              \
    case 9: CALL(9); return true;              \
    case 10: CALL(10); return true;            \
    default: return false;                     \
  }

#define ITHACA_TET_INSTANTIATE(T)                                                                                 \
  template <>                                                                                                     \
  bool TetApi<T>::helm(int n, int Q, int E, const T* tab, const T* jg, T lambda, const T* in, T* out,            \
                       const int* l2g, int ndir, const int* skip, const T* lam_ptr, cudaStream_t s) {             \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) {                                                                                    \
      dev::tet_helm_n<T, decltype(nn)::value>(E, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, s);          \
    };                                                                                                            \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }                                                                                                               \
  template <>                                                                                                     \
  bool TetApi<T>::bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s) {                   \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) { dev::tet_bwd_n<T, decltype(nn)::value>(E, tab, in, out, s); };                     \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }                                                                                                               \
  template <>                                                                                                     \
  bool TetApi<T>::ipr(int n, int Q, int E, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s) {      \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) { dev::tet_ipr_n<T, decltype(nn)::value>(E, tab, jg, in, out, s); };                 \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }                                                                                                               \
  template <>                                                                                                     \
  bool TetApi<T>::deriv(int n, int Q, int E, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2,        \
                        cudaStream_t s) {                                                                         \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) { dev::tet_deriv_n<T, decltype(nn)::value>(E, tab, df, in, d0, d1, d2, s); };        \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }                                                                                                               \
  template <>                                                                                                     \
  bool TetApi<T>::diag(int n, int Q, int E, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s) {        \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) { dev::tet_diag_n<T, decltype(nn)::value>(E, tab, jg, lambda, out, s); };           \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }                                                                                                               \
  template <>                                                                                                     \
  bool TetApi<T>::iprd(int n, int Q, int E, const T* tab, const T* jg, const T* df, const T* in0, const T* in1,   \
                       const T* in2, T* out, cudaStream_t s) {                                                    \
    if (E <= 0) return true;                                                                                      \
    auto call = [&](auto nn) {                                                                                    \
      dev::tet_iprd_n<T, decltype(nn)::value>(E, tab, jg, df, in0, in1, in2, out, s);                             \
    };                                                                                                            \
    ITHACA_TET_DISPATCH(n, Q, ITHACA_TET_CALL)                                                                    \
  }

}  // namespace ithaca
