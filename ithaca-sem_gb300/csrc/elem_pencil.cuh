// Hexahedral Helmholtz kernel with register pencils and a TMA-staged geometry slab.
//
// Each element is worked on by Q*Q threads. Every 1-D contraction runs on a "pencil":
// one thread holds the Q (or N) values along the contraction direction in registers
// and multiplies by the 1-D table, which is a kernel parameter (constant bank), so the
// inner products use no shared-memory loads at all. Shared memory only re-lays the
// data out between directions (Q^3 fields with padded strides: at most 2-way bank
// conflicts). The geometry slab of the CTA's elements (J w and the six metric terms
// per point, 7 Q^3 values per element) is brought into shared memory by one
// cp.async.bulk (TMA) copy, issued first and waited for (bounded) only when the
// point-wise metric stage needs it, so the copy overlaps the sum-factorised BwdTrans.
//
// Arithmetic (collocation form, as elem.cuh):
//   u = B u^ ; g_a = D_a u ; f_a = sum_b G_ab g_b ; v = lambda Jw u + sum_a D_a^T f_a ; out = B^T v
#pragma once

#include <cstdint>

#include "elem.cuh"

namespace ithaca {
namespace dev {

// k-stride of a padded Q^3 work field (index i + Q j + PK k): at most 2-way bank
// conflicts for the column (i, j), pencil-i (j, k) and pencil-j (i, k) lane layouts.
// Q = 8: 73 = 9 (mod 32), which with the pipelined kernel's lane maps leaves 2-way
// conflicts only in its two pencil-j stages.
__host__ __device__ constexpr int pk_stride(int Q) {
  return Q == 2 ? 5 : Q == 3 ? 9 : Q == 4 ? 19 : Q == 5 ? 25 : Q == 6 ? 36 : Q == 7 ? 51 : Q == 8 ? 73
       : Q == 9 ? 81 : Q == 10 ? 101 : 121;
}

template <typename T, int N, int Q>
struct PTabs {
  T B[N * Q];  // B[p*Q + i]
  T D[Q * Q];  // D[k*Q + i] = l_k'(z_i)
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// Bulk (non-tensor) TMA copy global -> shared, completion counted on `bar`.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void tma_bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// The same copy with an L2 eviction-priority policy (for data streamed once per launch,
// so that it does not push the reused vectors out of L2).
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void tma_bulk_load_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                   uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Waits for phase `phase` of `bar` for at most ~`max_cycles` SM cycles.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, long long max_cycles) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, phase)) {
    if (clock64() - t0 > max_cycles) return false;
  }
  return true;
}

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz: far beyond any real copy

template <typename T, int N, int Q, int EB>
struct PencilLayout {
  static constexpr int NQ = Q * Q * Q, NG = 7, GEO = NG * NQ;
  static constexpr int PJ = Q, PK = pk_stride(Q), FS = PK * Q;
  static constexpr size_t GEO_BYTES = ((size_t)EB * GEO * sizeof(T) + 32 + 15) / 16 * 16;  // + window slack
  static constexpr size_t bytes() { return 16 + GEO_BYTES + (size_t)EB * 3 * FS * sizeof(T); }
};

template <typename T, int N, int Q, int EB, bool GATHER>
__global__ void __launch_bounds__(Q* Q* EB) helm3_pencil_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                                 const PTabs<T, N, Q> tab, const T* __restrict__ jg,
                                                                 T lambda, int E, const int* __restrict__ l2g,
                                                                 int ndir, const int* __restrict__ skip,
                                                                 const T* __restrict__ lam_ptr, int* __restrict__ err) {
  using L = PencilLayout<T, N, Q, EB>;
  constexpr int NQ = L::NQ, NM = N * N * N, TPE = Q * Q, GEO = L::GEO;
  constexpr int PJ = L::PJ, PK = L::PK, FS = L::FS;
  if (skip != nullptr && *skip) return;  // converged solve: the whole CTA leaves together
  if (lam_ptr != nullptr) lambda = *lam_ptr;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  T* geo = reinterpret_cast<T*>(smem + 16);
  T* work = reinterpret_cast<T*>(smem + 16 + L::GEO_BYTES);

  const int t = threadIdx.x, el = threadIdx.y;
  const int tid = t + el * TPE;
  const int e0 = blockIdx.x * EB;
  const int ne = min(EB, E - e0);
  const bool active = el < ne;
  const int e = active ? e0 + el : e0;
  T* SU = work + el * 3 * FS;
  T* S0 = SU + FS;
  T* S1 = S0 + FS;

  // ---- geometry window: elements [e0, e0 + ne), rounded out to 16-byte boundaries ----
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(jg + (size_t)e0 * GEO);
  const uintptr_t lo = a0 & ~uintptr_t(15);
  const uintptr_t hi = (a0 + (size_t)ne * GEO * sizeof(T) + 15) & ~uintptr_t(15);
  const int shift = static_cast<int>(a0 - lo);
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(bar, static_cast<uint32_t>(hi - lo));
    tma_bulk_load(geo, reinterpret_cast<const void*>(lo), static_cast<uint32_t>(hi - lo), bar);
  }
  const T* G = reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(geo) + shift) + el * GEO;

  // ---- 1: coefficients (gathered through the signed map) -> S0 as (p, q, r) ----
  if (active) {
    for (int m = t; m < NM; m += TPE) {
      T v;
      if constexpr (GATHER) {
        const int code = l2g[(size_t)e * NM + m];
        const int g = code >= 0 ? code : ~code;
        v = g < ndir ? T(0) : in[g];
        v = code >= 0 ? v : -v;
      } else {
        v = in[(size_t)e * NM + m];
      }
      const int p = m % N, q = (m / N) % N, r = m / (N * N);
      S0[p + PJ * q + PK * r] = v;
    }
  }
  __syncthreads();
  // ---- 2: BwdTrans along p: pencils (q, r) ----
  if (t < N * N) {
    const int q = t % N, r = t / N;
    T c[N];
#pragma unroll
    for (int p = 0; p < N; ++p) c[p] = S0[p + PJ * q + PK * r];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.B[i] * c[0];
#pragma unroll
      for (int p = 1; p < N; ++p) acc = fma(tab.B[p * Q + i], c[p], acc);
      S1[i + PJ * q + PK * r] = acc;
    }
  }
  __syncthreads();
  // ---- 3: along q: pencils (i, r) ----
  if (t < Q * N) {
    const int i = t % Q, r = t / Q;
    T c[N];
#pragma unroll
    for (int q = 0; q < N; ++q) c[q] = S1[i + PJ * q + PK * r];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = tab.B[j] * c[0];
#pragma unroll
      for (int q = 1; q < N; ++q) acc = fma(tab.B[q * Q + j], c[q], acc);
      S0[i + PJ * j + PK * r] = acc;
    }
  }
  __syncthreads();
  // ---- 4: along r: columns (i, j) -> u in registers; d/dxi_2 in registers ----
  const int ci = t % Q, cj = t / Q;  // column owned by this thread (t < Q*Q always)
  T u[Q], g2[Q];
  {
    T c[N];
#pragma unroll
    for (int r = 0; r < N; ++r) c[r] = S0[ci + PJ * cj + PK * r];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      T acc = tab.B[k] * c[0];
#pragma unroll
      for (int r = 1; r < N; ++r) acc = fma(tab.B[r * Q + k], c[r], acc);
      u[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      T acc = tab.D[k] * u[0];
#pragma unroll
      for (int c2 = 1; c2 < Q; ++c2) acc = fma(tab.D[c2 * Q + k], u[c2], acc);
      g2[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) SU[ci + PJ * cj + PK * k] = u[k];
  }
  __syncthreads();
  // ---- 5: d/dxi_0 on pencils (j, k) -> S0 ; d/dxi_1 on pencils (i, k) -> S1 ----
  {
    const int pj = t % Q, pk = t / Q;
    T c[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) c[a] = SU[a + PJ * pj + PK * pk];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.D[i] * c[0];
#pragma unroll
      for (int a = 1; a < Q; ++a) acc = fma(tab.D[a * Q + i], c[a], acc);
      S0[i + PJ * pj + PK * pk] = acc;
    }
    const int pi = t % Q;
#pragma unroll
    for (int a = 0; a < Q; ++a) c[a] = SU[pi + PJ * a + PK * pk];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = tab.D[j] * c[0];
#pragma unroll
      for (int a = 1; a < Q; ++a) acc = fma(tab.D[a * Q + j], c[a], acc);
      S1[pi + PJ * j + PK * pk] = acc;
    }
  }
  // geometry must have landed before the point-wise stage
  const bool ok = mbar_wait_bounded(bar, 0, kWaitCycles);
  if (!__syncthreads_and(ok)) {
    if (tid == 0 && err != nullptr) atomicExch(err, ITHACA_GPU_ERR_TIMEOUT);
    mbar_wait_bounded(bar, 0, kWaitCycles);  // give an in-flight copy time to finish
    return;
  }
  // ---- 6: point-wise metric on columns (i, j) ----
  T v[Q];
  {
    T f2[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const int s = ci + PJ * cj + PK * k;
      const int pt = ci + Q * cj + Q * Q * k;
      const T g0 = S0[s], g1 = S1[s];
      const T jw = G[pt];
      const T m00 = G[NQ + pt], m01 = G[2 * NQ + pt], m02 = G[3 * NQ + pt];
      const T m11 = G[4 * NQ + pt], m12 = G[5 * NQ + pt], m22 = G[6 * NQ + pt];
      S0[s] = fma(m00, g0, fma(m01, g1, m02 * g2[k]));
      S1[s] = fma(m01, g0, fma(m11, g1, m12 * g2[k]));
      f2[k] = fma(m02, g0, fma(m12, g1, m22 * g2[k]));
      v[k] = lambda * jw * u[k];
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      T acc = v[k];
#pragma unroll
      for (int c2 = 0; c2 < Q; ++c2) acc = fma(tab.D[k * Q + c2], f2[c2], acc);
      v[k] = acc;
    }
  }
  __syncthreads();
  // ---- 7: D^T along i on pencils (j, k) in S0, along j on pencils (i, k) in S1 (in place) ----
  {
    const int pj = t % Q, pk = t / Q;
    T c[Q], o[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) c[a] = S0[a + PJ * pj + PK * pk];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      T acc = tab.D[i * Q] * c[0];
#pragma unroll
      for (int a = 1; a < Q; ++a) acc = fma(tab.D[i * Q + a], c[a], acc);
      o[i] = acc;
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) S0[i + PJ * pj + PK * pk] = o[i];
    const int pi = t % Q;
#pragma unroll
    for (int a = 0; a < Q; ++a) c[a] = S1[pi + PJ * a + PK * pk];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      T acc = tab.D[j * Q] * c[0];
#pragma unroll
      for (int a = 1; a < Q; ++a) acc = fma(tab.D[j * Q + a], c[a], acc);
      o[j] = acc;
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) S1[pi + PJ * j + PK * pk] = o[j];
  }
  __syncthreads();
  // ---- 8: sum the three directions on columns, IProduct along k -> SU as (i, j, r) ----
  {
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const int s = ci + PJ * cj + PK * k;
      v[k] += S0[s] + S1[s];
    }
#pragma unroll
    for (int r = 0; r < N; ++r) {
      T acc = tab.B[r * Q] * v[0];
#pragma unroll
      for (int k = 1; k < Q; ++k) acc = fma(tab.B[r * Q + k], v[k], acc);
      SU[ci + PJ * cj + PK * r] = acc;
    }
  }
  __syncthreads();
  // ---- 9: along j: pencils (i, r) -> S0 as (i, q, r) ----
  if (t < Q * N) {
    const int i = t % Q, r = t / Q;
    T c[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) c[j] = SU[i + PJ * j + PK * r];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      T acc = tab.B[q * Q] * c[0];
#pragma unroll
      for (int j = 1; j < Q; ++j) acc = fma(tab.B[q * Q + j], c[j], acc);
      S0[i + PJ * q + PK * r] = acc;
    }
  }
  __syncthreads();
  // ---- 10: along i: pencils (q, r) -> S1 as (p, q, r) ----
  if (t < N * N) {
    const int q = t % N, r = t / N;
    T c[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) c[i] = S0[i + PJ * q + PK * r];
#pragma unroll
    for (int p = 0; p < N; ++p) {
      T acc = tab.B[p * Q] * c[0];
#pragma unroll
      for (int i = 1; i < Q; ++i) acc = fma(tab.B[p * Q + i], c[i], acc);
      S1[p + PJ * q + PK * r] = acc;
    }
  }
  __syncthreads();
  if (active) {
    for (int m = t; m < NM; m += TPE) {
      const int p = m % N, q = (m / N) % N, r = m / (N * N);
      out[(size_t)e * NM + m] = S1[p + PJ * q + PK * r];
    }
  }
}

}  // namespace dev
}  // namespace ithaca
