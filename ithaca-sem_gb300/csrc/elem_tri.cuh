// Sum-factorised element operators for triangles in collapsed coordinates.
//
// Expansion: ModifiedA on Q0 = N + 1 GLL points along eta0, ModifiedB on Q1 = N
// Gauss-Radau-Jacobi (alpha 1, beta 0) points along eta1; NC = N (N + 1) / 2 modes
// m(p, q), q fastest. Values at points are stored u[j*Q0 + i] (i along eta0).
//
// The reference kernels (MatrixFreeOps/BwdTransKernels.hpp:78-125 BwdTransTriKernel,
// IProductKernels.hpp:136-234 IProductTriKernel, PhysDerivKernels.hpp:153-212,
// Helmholtz.h:505-635 HelmholtzTriImpl) work per SIMD lane; here a group of TPE threads
// works on one element with its tensors in shared memory:
//   BwdTrans   W[p][j] = sum_{q < N-p} B1[m(p,q)][j] c[m(p,q)]  (+ c_1 B1[1][j] for p = 1,
//              the singular-vertex term of CORRECT), then u[j][i] = sum_p W[p][j] B0[p][i];
//   IProduct   W[p][j] = sum_i B0[p][i] f[j][i], then out[m] = sum_j B1[m][j] W[p(m)][j]
//              (+ sum_j B1[1][j] W[1][j] for m = 1);
//   Helmholtz  the collocation form used for quads,
//                out = IProduct( lambda Jw u + D0^T G0 + D1^T G1 ),
//                G0 = Jw (m00 d0 + m01 d1), G1 = Jw (m01 d0 + m11 d1),
//              with d0, d1 the collapsed derivatives and m^{ab} the collapsed metric of
//              HelmholtzTriImpl (h0 = (1 + z0)/2, h1 = 2/(1 - z1)); it equals the reference's
//              three inner products with DB0 and DB1 because IProduct_{DB}(f) = IProduct_B(D^T f).
// Shared memory per element: three tensors of NQ = Q0 Q1 values (U, F0, F1); the mode
// work arrays (W of N Q1 values, C of NC) reuse F0 and F1 while those are dead.
#pragma once

#include <type_traits>

#include "elem.cuh"

namespace ithaca {
namespace dev {

template <int N>
struct TriShape {
  static constexpr int Q0 = N + 1, Q1 = N, NC = N * (N + 1) / 2, NQ = Q0 * Q1;
  static constexpr TriOff O = tri_off(N);
  static constexpr int TS = align_up(O.size, 4);
  static constexpr int SLAB = 3 * NQ;
  static constexpr int TPE = NQ <= 32 ? 32 : (NQ <= 64 ? 64 : 128);
  static constexpr int EB = 256 / TPE;
  template <typename T>
  static constexpr size_t bytes() {
    return sizeof(T) * ((size_t)TS + (size_t)EB * SLAB);
  }
};

// Row p of mode m (m(p, 0) = p N - p (p - 1) / 2).
template <int N>
__device__ __forceinline__ int tri_row(int m, int* m0_out) {
  int p = 0, m0 = 0;
#pragma unroll 1
  while (p < N - 1 && m >= m0 + (N - p)) {
    m0 += N - p;
    ++p;
  }
  *m0_out = m0;
  return p;
}

// Coefficients C (NC) -> values U (NQ); W (N*Q1) is scratch.
template <typename T, int N>
__device__ __forceinline__ void tri_bwd_stages(const T* C, T* W, T* U, const T* s, int t, int nt) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1;
  const T* B0 = s + S::O.B0;
  const T* B1 = s + S::O.B1;
  for (int idx = t; idx < N * Q1; idx += nt) {
    const int p = idx / Q1, j = idx - p * Q1;
    const int m0 = p * N - p * (p - 1) / 2;
    T acc = p == 1 ? C[1] * B1[Q1 + j] : T(0);
#pragma unroll
    for (int q = 0; q < N; ++q)
      if (q < N - p) acc = fma(B1[(m0 + q) * Q1 + j], C[m0 + q], acc);
    W[idx] = acc;
  }
  __syncthreads();
  for (int idx = t; idx < Q0 * Q1; idx += nt) {
    const int j = idx / Q0, i = idx - j * Q0;
    T acc = 0;
#pragma unroll
    for (int p = 0; p < N; ++p) acc = fma(W[p * Q1 + j], B0[p * Q0 + i], acc);
    U[idx] = acc;
  }
}

// Values V (NQ, already weighted) -> inner products C (NC) with tables A0 (N x Q0, along
// eta0) and A1 (NC x Q1, along eta1); W (N*Q1) is scratch.
template <typename T, int N>
__device__ __forceinline__ void tri_ipr_stages(const T* V, T* W, T* C, const T* A0, const T* A1, int t, int nt) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1, NC = S::NC;
  for (int idx = t; idx < N * Q1; idx += nt) {
    const int p = idx / Q1, j = idx - p * Q1;
    T acc = 0;
#pragma unroll
    for (int i = 0; i < Q0; ++i) acc = fma(A0[p * Q0 + i], V[j * Q0 + i], acc);
    W[idx] = acc;
  }
  __syncthreads();
  for (int m = t; m < NC; m += nt) {
    int m0;
    const int p = tri_row<N>(m, &m0);
    T acc = 0;
#pragma unroll
    for (int j = 0; j < Q1; ++j) acc = fma(A1[m * Q1 + j], W[p * Q1 + j], acc);
    if (m == 1) {
#pragma unroll
      for (int j = 0; j < Q1; ++j) acc = fma(A1[Q1 + j], W[Q1 + j], acc);
    }
    C[m] = acc;
  }
}

// Per-point geometry of the Helmholtz operator: Jw and G00, G01, G11 (= Jw m^{ab}).
// Deformed elements read them per point; regular ones hold J, J g00, J g01, J g11 per
// element (g^{ab} = sum_k df[k*2+a] df[k*2+b]) and the collapsed factors are added here:
//   m00 = h1^2 (g00 + 2 h0 g01 + h0^2 g11), m01 = h1 (g01 + h0 g11), m11 = g11.
template <typename T, int N, bool DEF>
__device__ __forceinline__ void tri_geo(const T* gbase, const T* s, int p, int i, int j, T& jw, T& g00, T& g01,
                                        T& g11) {
  using S = TriShape<N>;
  constexpr int NQ = S::NQ;
  if constexpr (DEF) {
    jw = gbase[p];
    g00 = gbase[NQ + p];
    g01 = gbase[2 * NQ + p];
    g11 = gbase[3 * NQ + p];
  } else {
    const T ww = s[S::O.w0 + i] * s[S::O.w1 + j];
    const T h0 = s[S::O.h0 + i], h1 = s[S::O.h1 + j];
    const T J = gbase[0], JA = gbase[1], JB = gbase[2], JC = gbase[3];
    jw = J * ww;
    g11 = JC * ww;
    g01 = fma(h0, JC, JB) * h1 * ww;
    g00 = fma(h0, fma(h0, JC, T(2) * JB), JA) * (h1 * h1) * ww;
  }
}

// ---------------------------------------------------------------------------
template <typename T, int N, int TPE, bool DEF, bool GATHER>
__global__ void __launch_bounds__(256) tri_helm_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                        const T* __restrict__ tab, const T* __restrict__ jg,
                                                        T lambda, int E, const int* __restrict__ l2g, int ndir,
                                                        const int* __restrict__ skip, const T* __restrict__ lam_ptr,
                                                        const int* __restrict__ esolve, int skip_stride) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1, NC = S::NC, NQ = S::NQ, NG = 4;
  constexpr int PPT = cdiv(NQ, TPE);
  if (esolve == nullptr && skip != nullptr && *skip) return;
  if (lam_ptr != nullptr) lambda = *lam_ptr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  const T* sD0 = s + S::O.D0;
  const T* sD1 = s + S::O.D1;
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* W = F0;
  T* C = F1;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const bool active = e < E && !(esolve != nullptr && skip[(size_t)esolve[ee] * skip_stride] != 0);
  if (esolve != nullptr && !__syncthreads_or(active)) return;
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
    C[m] = v;
  }
  __syncthreads();
  tri_bwd_stages<T, N>(C, W, U, s, t, TPE);
  __syncthreads();

  T mreg[PPT];
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
#pragma unroll
  for (int r = 0; r < PPT; ++r) {
    const int p = t + r * TPE;
    if (p < NQ) {
      const int j = p / Q0, i = p - j * Q0;
      T d0 = 0, d1 = 0;
#pragma unroll
      for (int a = 0; a < Q0; ++a) d0 = fma(sD0[a * Q0 + i], U[j * Q0 + a], d0);
#pragma unroll
      for (int a = 0; a < Q1; ++a) d1 = fma(sD1[a * Q1 + j], U[a * Q0 + i], d1);
      T jw, g00, g01, g11;
      tri_geo<T, N, DEF>(gbase, s, p, i, j, jw, g00, g01, g11);
      F0[p] = fma(g00, d0, g01 * d1);
      F1[p] = fma(g01, d0, g11 * d1);
      mreg[r] = lambda * jw * U[p];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PPT; ++r) {
    const int p = t + r * TPE;
    if (p < NQ) {
      const int j = p / Q0, i = p - j * Q0;
      T v = mreg[r];
#pragma unroll
      for (int a = 0; a < Q0; ++a) v = fma(sD0[i * Q0 + a], F0[j * Q0 + a], v);
#pragma unroll
      for (int a = 0; a < Q1; ++a) v = fma(sD1[j * Q1 + a], F1[a * Q0 + i], v);
      U[p] = v;
    }
  }
  __syncthreads();
  tri_ipr_stages<T, N>(U, W, C, s + S::O.B0, s + S::O.B1, t, TPE);
  __syncthreads();
  if (active)
    for (int m = t; m < NC; m += TPE) out[(size_t)e * NC + m] = C[m];
}

template <typename T, int N, int TPE>
__global__ void __launch_bounds__(256) tri_bwd_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                       const T* __restrict__ tab, int E) {
  using S = TriShape<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* W = U + S::NQ;
  T* C = W + S::NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  for (int m = t; m < S::NC; m += TPE) C[m] = in[(size_t)ee * S::NC + m];
  __syncthreads();
  tri_bwd_stages<T, N>(C, W, U, s, t, TPE);
  __syncthreads();
  if (e < E)
    for (int p = t; p < S::NQ; p += TPE) out[(size_t)e * S::NQ + p] = U[p];
}

template <typename T, int N, int TPE, bool DEF>
__global__ void __launch_bounds__(256) tri_ipr_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                       const T* __restrict__ tab, const T* __restrict__ jg, int E) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, NQ = S::NQ, NG = 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* W = U + NQ;
  T* C = W + NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
  for (int p = t; p < NQ; p += TPE) {
    const int j = p / Q0, i = p - j * Q0;
    const T jw = DEF ? gbase[p] : gbase[0] * s[S::O.w0 + i] * s[S::O.w1 + j];
    U[p] = in[(size_t)ee * NQ + p] * jw;
  }
  __syncthreads();
  tri_ipr_stages<T, N>(U, W, C, s + S::O.B0, s + S::O.B1, t, TPE);
  __syncthreads();
  if (e < E)
    for (int m = t; m < S::NC; m += TPE) out[(size_t)e * S::NC + m] = C[m];
}

// PhysDeriv: collapsed derivatives, d/dxi0 = h1 d/deta0, d/dxi1 = h0 h1 d/deta0 + d/deta1,
// then the derivative factors (PhysDerivTriKernel).
template <typename T, int N, int TPE, bool DEF>
__global__ void __launch_bounds__(256) tri_deriv_kernel(const T* __restrict__ in, T* __restrict__ o0,
                                                         T* __restrict__ o1, const T* __restrict__ tab,
                                                         const T* __restrict__ df, int E) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1, NQ = S::NQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  const T* sD0 = s + S::O.D0;
  const T* sD1 = s + S::O.D1;
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  for (int p = t; p < NQ; p += TPE) U[p] = in[(size_t)ee * NQ + p];
  __syncthreads();
  if (e >= E) return;
  const T* dbase = df + (size_t)e * 4 * (DEF ? NQ : 1);
  for (int p = t; p < NQ; p += TPE) {
    const int j = p / Q0, i = p - j * Q0;
    T d0 = 0, d1 = 0;
#pragma unroll
    for (int a = 0; a < Q0; ++a) d0 = fma(sD0[a * Q0 + i], U[j * Q0 + a], d0);
#pragma unroll
    for (int a = 0; a < Q1; ++a) d1 = fma(sD1[a * Q1 + j], U[a * Q0 + i], d1);
    const T x0 = s[S::O.h1 + j] * d0;
    const T x1 = fma(s[S::O.h0 + i], x0, d1);
    T f[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) f[c] = DEF ? dbase[c * NQ + p] : dbase[c];
    o0[(size_t)e * NQ + p] = fma(f[0], x0, f[1] * x1);
    o1[(size_t)e * NQ + p] = fma(f[2], x0, f[3] * x1);
  }
}

// IProductWRTDerivBase: t_j = sum_k df[k*2+j] in_k, G0 = Jw h1 (t_0 + h0 t_1), G1 = Jw t_1,
// out = IProduct(D0^T G0 + D1^T G1) (IProductWRTDerivBaseTriImpl in collocation form).
template <typename T, int N, int TPE, bool DEF>
__global__ void __launch_bounds__(256) tri_iprd_kernel(const T* __restrict__ in0, const T* __restrict__ in1,
                                                        T* __restrict__ out, const T* __restrict__ tab,
                                                        const T* __restrict__ jg, const T* __restrict__ df, int E) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1, NQ = S::NQ, NG = 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  const T* sD0 = s + S::O.D0;
  const T* sD1 = s + S::O.D1;
  T* U = s + S::TS + threadIdx.y * S::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const int ee = e < E ? e : E - 1;
  const int t = threadIdx.x;
  const T* gbase = jg + (size_t)ee * NG * (DEF ? NQ : 1);
  const T* dbase = df + (size_t)ee * 4 * (DEF ? NQ : 1);
  for (int p = t; p < NQ; p += TPE) {
    const int j = p / Q0, i = p - j * Q0;
    T f[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) f[c] = DEF ? dbase[c * NQ + p] : dbase[c];
    const T a = in0[(size_t)ee * NQ + p], b = in1[(size_t)ee * NQ + p];
    const T t0 = fma(f[0], a, f[2] * b);
    const T t1 = fma(f[1], a, f[3] * b);
    const T jw = DEF ? gbase[p] : gbase[0] * s[S::O.w0 + i] * s[S::O.w1 + j];
    F0[p] = jw * s[S::O.h1 + j] * fma(s[S::O.h0 + i], t1, t0);
    F1[p] = jw * t1;
  }
  __syncthreads();
  for (int p = t; p < NQ; p += TPE) {
    const int j = p / Q0, i = p - j * Q0;
    T v = 0;
#pragma unroll
    for (int a = 0; a < Q0; ++a) v = fma(sD0[i * Q0 + a], F0[j * Q0 + a], v);
#pragma unroll
    for (int a = 0; a < Q1; ++a) v = fma(sD1[j * Q1 + a], F1[a * Q0 + i], v);
    U[p] = v;
  }
  __syncthreads();
  tri_ipr_stages<T, N>(U, F0, F1, s + S::O.B0, s + S::O.B1, t, TPE);
  __syncthreads();
  if (e < E)
    for (int m = t; m < S::NC; m += TPE) out[(size_t)e * S::NC + m] = F1[m];
}

// Diagonal of each element's Helmholtz matrix: for mode m = (p, q) with
// phi = B0[p] x B1[m] (the top vertex m = 1: (B0[0] + B0[1]) x B1[1] = B1[1]),
//   diag = sum_points lambda Jw phi^2 + G00 phi_0^2 + 2 G01 phi_0 phi_1 + G11 phi_1^2,
// phi_0 = DB0[p] x B1[m], phi_1 = B0[p] x DB1[m].
template <typename T, int N, int TPE, bool DEF>
__global__ void __launch_bounds__(256) tri_diag_kernel(T* __restrict__ out, const T* __restrict__ tab,
                                                        const T* __restrict__ jg, T lambda, int E) {
  using S = TriShape<N>;
  constexpr int Q0 = S::Q0, Q1 = S::Q1, NQ = S::NQ, NG = 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  load_tables(s, tab, S::O.size);
  __syncthreads();
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  if (e >= E) return;
  const T* B0 = s + S::O.B0;
  const T* DB0 = s + S::O.DB0;
  const T* B1 = s + S::O.B1;
  const T* DB1 = s + S::O.DB1;
  const T* gbase = jg + (size_t)e * NG * (DEF ? NQ : 1);
  for (int m = threadIdx.x; m < S::NC; m += TPE) {
    int m0;
    const int p = tri_row<N>(m, &m0);
    T acc = 0;
    for (int j = 0; j < Q1; ++j) {
      const T b1 = B1[m * Q1 + j], db1 = DB1[m * Q1 + j];
      for (int i = 0; i < Q0; ++i) {
        T b0 = B0[p * Q0 + i], db0 = DB0[p * Q0 + i];
        if (m == 1) {
          b0 += B0[Q0 + i];
          db0 += DB0[Q0 + i];
        }
        const T ph = b0 * b1, ph0 = db0 * b1, ph1 = b0 * db1;
        T jw, g00, g01, g11;
        tri_geo<T, N, DEF>(gbase, s, j * Q0 + i, i, j, jw, g00, g01, g11);
        acc = fma(lambda * jw * ph, ph, acc);
        acc = fma(g00 * ph0, ph0, acc);
        acc = fma(T(2) * g01 * ph0, ph1, acc);
        acc = fma(g11 * ph1, ph1, acc);
      }
    }
    out[(size_t)e * S::NC + m] = acc;
  }
}

// ---------------------------------------------------------------------------
template <typename T, int N>
struct TriCfg {
  using S = TriShape<N>;
  static dim3 block() { return dim3(S::TPE, S::EB); }
  static dim3 grid(int E) { return dim3((E + S::EB - 1) / S::EB); }
  static size_t smem() { return S::template bytes<T>(); }
  template <class K>
  static void prep(K k) {
    static bool done = false;
    if (!done) {
      ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()));
      done = true;
    }
  }
};

template <typename T, int N>
void tri_helm_n(int E, int deformed, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g,
                int ndir, const int* skip, const T* lam_ptr, const int* esolve, int skip_stride, cudaStream_t s) {
  using C = TriCfg<T, N>;
  constexpr int TPE = C::S::TPE;
  auto k = deformed ? (l2g ? tri_helm_kernel<T, N, TPE, true, true> : tri_helm_kernel<T, N, TPE, true, false>)
                    : (l2g ? tri_helm_kernel<T, N, TPE, false, true> : tri_helm_kernel<T, N, TPE, false, false>);
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, lambda, E, l2g, ndir, skip, lam_ptr, esolve,
                                               skip_stride);
}

template <typename T, int N>
void tri_bwd_n(int E, const T* tab, const T* in, T* out, cudaStream_t s) {
  using C = TriCfg<T, N>;
  auto k = tri_bwd_kernel<T, N, C::S::TPE>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, E);
}

template <typename T, int N>
void tri_ipr_n(int E, int deformed, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s) {
  using C = TriCfg<T, N>;
  auto k = deformed ? tri_ipr_kernel<T, N, C::S::TPE, true> : tri_ipr_kernel<T, N, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, out, tab, jg, E);
}

template <typename T, int N>
void tri_deriv_n(int E, int deformed, const T* tab, const T* df, const T* in, T* d0, T* d1, cudaStream_t s) {
  using C = TriCfg<T, N>;
  auto k = deformed ? tri_deriv_kernel<T, N, C::S::TPE, true> : tri_deriv_kernel<T, N, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in, d0, d1, tab, df, E);
}

template <typename T, int N>
void tri_iprd_n(int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0, const T* in1, T* out,
                cudaStream_t s) {
  using C = TriCfg<T, N>;
  auto k = deformed ? tri_iprd_kernel<T, N, C::S::TPE, true> : tri_iprd_kernel<T, N, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(in0, in1, out, tab, jg, df, E);
}

template <typename T, int N>
void tri_diag_n(int E, int deformed, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s) {
  using C = TriCfg<T, N>;
  auto k = deformed ? tri_diag_kernel<T, N, C::S::TPE, true> : tri_diag_kernel<T, N, C::S::TPE, false>;
  C::prep(k);
  k<<<C::grid(E), C::block(), C::smem(), s>>>(out, tab, jg, lambda, E);
}

}  // namespace dev

// Runs CALL(N) for 2 <= n <= 12 with Q == n + 1; false otherwise.
#define ITHACA_TRI_DISPATCH(n, Q, CALL)        \
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
    case 11: CALL(11); return true;            \
    case 12: CALL(12); return true;            \
    default: return false;                     \
  }

#define ITHACA_TRI_INSTANTIATE(T)                                                                                \
  template <>                                                                                                    \
  bool TriApi<T>::helm(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, const T* in,     \
                       T* out, const int* l2g, int ndir, const int* skip, const T* lam_ptr, const int* esolve,   \
                       int skip_stride, cudaStream_t s) {                                                        \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) {                                                                                   \
      dev::tri_helm_n<T, decltype(nn)::value>(E, deformed, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr,  \
                                              esolve, skip_stride, s);                                           \
    };                                                                                                           \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }                                                                                                              \
  template <>                                                                                                    \
  bool TriApi<T>::bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s) {                  \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) { dev::tri_bwd_n<T, decltype(nn)::value>(E, tab, in, out, s); };                    \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }                                                                                                              \
  template <>                                                                                                    \
  bool TriApi<T>::ipr(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* in, T* out,        \
                      cudaStream_t s) {                                                                          \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) { dev::tri_ipr_n<T, decltype(nn)::value>(E, deformed, tab, jg, in, out, s); };      \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }                                                                                                              \
  template <>                                                                                                    \
  bool TriApi<T>::deriv(int n, int Q, int E, int deformed, const T* tab, const T* df, const T* in, T* d0,       \
                        T* d1, cudaStream_t s) {                                                                 \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) { dev::tri_deriv_n<T, decltype(nn)::value>(E, deformed, tab, df, in, d0, d1, s); }; \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }                                                                                                              \
  template <>                                                                                                    \
  bool TriApi<T>::diag(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, T* out,          \
                       cudaStream_t s) {                                                                         \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) { dev::tri_diag_n<T, decltype(nn)::value>(E, deformed, tab, jg, lambda, out, s); }; \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }                                                                                                              \
  template <>                                                                                                    \
  bool TriApi<T>::iprd(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0, \
                       const T* in1, T* out, cudaStream_t s) {                                                   \
    if (E <= 0) return true;                                                                                     \
    auto call = [&](auto nn) {                                                                                   \
      dev::tri_iprd_n<T, decltype(nn)::value>(E, deformed, tab, jg, df, in0, in1, out, s);                       \
    };                                                                                                           \
    ITHACA_TRI_DISPATCH(n, Q, ITHACA_TRI_CALL)                                                                   \
  }

#define ITHACA_TRI_CALL(NN) call(std::integral_constant<int, NN>{})

}  // namespace ithaca
