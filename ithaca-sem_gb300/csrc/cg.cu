// Global C0 Helmholtz system and its conjugate-gradient solvers.
//
//  * Assembly (AssemblyMapCG::v_Assemble, MultiRegions/AssemblyMap/AssemblyMapCG.cpp:2885-2910)
//    is an owner-computes CSR sum over the local dofs of each global dof, in a fixed
//    order: no atomics, so results and iteration counts are bit-reproducible.
//  * GlobalToLocal (:2853-2876) is fused into the element Helmholtz kernel (gather).
//  * PCG follows the single-reduction recurrence of NekLinSysIterCG::DoConjugateGradient
//    (LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp:104-263) with the Jacobi
//    preconditioner of PreconditionerDiagonal (MultiRegions/PreconditionerDiagonal.cpp:98-206)
//    and the ||b||^2 <= 1e-6 -> 1 floor of NekLinSysIter::Set_Rhs_Magnitude (NekLinSysIter.cpp:128-152).
//    Per iteration: update(p, q, x, r, w = M^-1 r; r.w, r.r) -> gather + element apply
//    -> assemble(s; s.w) -> scalars. Partial sums go through fixed-size per-CTA slots
//    and a one-CTA reduction in fixed order. Chunks of iterations run as one CUDA graph;
//    a device flag stops the remaining kernels of a chunk once the solve has converged.
//  * Mixed precision: FP64 residuals r = b - A x (FP64 operator), FP32 inner PCG on
//    the FP32 copy of the operator, x += ||r|| d, until ||r|| <= tol ||b||.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include <cuda_fp16.h>

#include "cg_shared.h"
#include "ithaca_internal.h"

namespace ithaca {

// Grids of the vector and assembly kernels: 5 and 8 CTAs per SM of the device (one wave at
// <= 51 and <= 32 registers per thread), capped at the partial-sum capacities below
constexpr int kRedPerSM = 5, kAsmPerSM = 8;
constexpr int RB = 760;      // capacity of a partial-sum slot of the vector kernels (5 x 152 SMs)
constexpr int RBA = 1216;    // capacity of slot 3 (assembly partials; 8 x 152 SMs)
constexpr int RT = 256;      // threads per reduction CTA
constexpr int NSLOT = 4;     // partial-sum slots: 0 r.w, 1 r.r, 2 b.b, 3 s.w
// 2-D systems up to this many global dofs run the persistent solver by default: below it
// the graph-captured kernels are bound by launch and drain rather than by their work
constexpr int kPersistMaxN = 1 << 20;


// ---- reductions -------------------------------------------------------------
template <int NC>
__device__ __forceinline__ void block_partials(double (&v)[NC], double* partials, const int* slots) {
  __shared__ double sm[NC][RT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], off);
    if (lane == 0) sm[c][warp] = v[c];
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double s = 0;
#pragma unroll
    for (int w = 0; w < RT / 32; ++w) s += sm[threadIdx.x][w];
    partials[slots[threadIdx.x] * RB + blockIdx.x] = s;
  }
}

// The same from FP32 per-thread values: the warp sums in FP32 (shuffles), only the sum of
// a CTA's warp sums in FP64, by one thread per slot. FP64 arithmetic runs at ~1/60 of the
// FP32 rate on this GPU, so FP64 shuffle trees over every lane of every CTA cost several
// microseconds at the end of each kernel.
template <int NC>
__device__ __forceinline__ void block_partials(float (&v)[NC], double* partials, const int* slots) {
  __shared__ double sm[NC][RT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], off);
    if (lane == 0) sm[c][warp] = (double)v[c];
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double s = sm[threadIdx.x][0];
#pragma unroll
    for (int w = 1; w < RT / 32; ++w) s += sm[threadIdx.x][w];
    partials[slots[threadIdx.x] * RB + blockIdx.x] = s;
  }
}

// Deterministic CTA sums of one double per thread and slot: warp shuffles, then the
// warps' sums in warp order. Every thread receives the totals.
template <int NS>
__device__ __forceinline__ void block_sum(double (&acc)[NS], double (&out)[NS]) {
  __shared__ double sm[NS][RT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], off);
    if (lane == 0) sm[k][warp] = acc[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    double t = sm[k][0];
#pragma unroll
    for (int w = 1; w < RT / 32; ++w) t += sm[k][w];
    out[k] = t;
  }
  __syncthreads();
}

// This thread's share of the first n entries of p (entries threadIdx.x + i RT): the first
// M loads are all issued before the first add (L2 loads: the entries may have been
// written by other CTAs of the same launch); entries beyond M RT follow in a loop.
template <int M>
__device__ __forceinline__ double thread_partials(const double* p, int n) {
  double v[M];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const int j = threadIdx.x + i * RT;
    v[i] = j < n ? __ldcg(p + j) : 0.0;
  }
  double t = v[0];
#pragma unroll
  for (int i = 1; i < M; ++i) t += v[i];
  for (int j = threadIdx.x + M * RT; j < n; j += RT) t += __ldcg(p + j);
  return t;
}
constexpr int kMaxP = (RBA + RT - 1) / RT;  // partials per thread of a full slot

// Sum of the first n partials of `slot` (n = the CTA count of the launch that wrote them).
__device__ __forceinline__ double reduce_slot(const double* partials, int slot, int n) {
  double a[1] = {thread_partials<kMaxP>(partials + slot * RB, n)}, o[1];
  block_sum<1>(a, o);
  return o[0];
}

// Several slots at once (same summation order as reduce_slot for each): the loads of
// all slots are in flight together and the tree steps are shared.
// nv: CTAs of the vector kernels (slots 0-2), na: CTAs of the assembly (slot 3).
template <int NS>
__device__ __forceinline__ void reduce_slots(const double* partials, const int (&slots)[NS], double (&out)[NS],
                                             int nv, int na) {
  double a[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) a[k] = thread_partials<kMaxP>(partials + slots[k] * RB, slots[k] == 3 ? na : nv);
  block_sum<NS>(a, out);
}

// ---- PCG vector kernels (T = double or float; reductions in double) ----------
template <typename T>
__global__ void __launch_bounds__(RT) pcg_init_kernel(int N, int ndir, const T* __restrict__ b, T* __restrict__ x,
                                                      T* __restrict__ r, T* __restrict__ w,
                                                      const T* __restrict__ dinv, double* partials) {
  double v[3] = {0, 0, 0};
  for (int g = blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) {
    const double bg = (double)b[g];
    v[2] += bg * bg;
    if (g >= ndir) {
      const T rg = b[g];
      const T wg = dinv[g] * rg;
      r[g] = rg;
      x[g] = T(0);
      w[g] = wg;
      v[0] += (double)rg * (double)wg;
      v[1] += (double)rg * (double)rg;
    } else {
      w[g] = T(0);
    }
  }
  const int slots[3] = {0, 1, 2};
  block_partials<3>(v, partials, slots);
}

template <typename T>
__global__ void __launch_bounds__(RT) pcg_update_kernel(int N, int ndir, const CgScalars* sc, T* __restrict__ x,
                                                        T* __restrict__ r, T* __restrict__ w,
                                                        const T* __restrict__ s, T* __restrict__ p,
                                                        T* __restrict__ q, const T* __restrict__ dinv,
                                                        double* partials) {
  if (sc->done) return;
  const T alpha = (T)sc->alpha, beta = (T)sc->beta;
  double v[2] = {0, 0};
  for (int g = ndir + blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) {
    const T pg = beta * p[g] + w[g];
    const T qg = beta * q[g] + s[g];
    p[g] = pg;
    q[g] = qg;
    x[g] += alpha * pg;
    const T rg = r[g] - alpha * qg;
    r[g] = rg;
    const T wg = dinv[g] * rg;
    w[g] = wg;
    v[0] += (double)rg * (double)wg;
    v[1] += (double)rg * (double)rg;
  }
  const int slots[2] = {0, 1};
  block_partials<2>(v, partials, slots);
}

// FP32 update on four dofs per step (16-byte loads and stores; the vectors are padded
// to a multiple of four entries). Lanes outside [ndir, N) are stored back unchanged.
// The per-thread sums r.w and r.r are accumulated in FP32 (a few dozen terms per
// thread) and only the CTA reduction is in FP64: FP64 throughput on this GPU is ~1/60
// of FP32, and per-dof FP64 products and conversions would dominate the kernel.
__global__ void __launch_bounds__(RT) pcg_update_f32x4_kernel(int N, int ndir, const CgScalars* sc,
                                                              float* __restrict__ x, float* __restrict__ r,
                                                              float* __restrict__ w, const float* __restrict__ s,
                                                              float* __restrict__ p, float* __restrict__ q,
                                                              const float* __restrict__ dinv, double* partials) {
  if (sc->done) return;
  const float alpha = (float)sc->alpha, beta = (float)sc->beta;
  float rw = 0.f, rr = 0.f;
  const int c0 = ndir >> 2, c1 = (N + 3) >> 2;
  for (int c = c0 + blockIdx.x * RT + threadIdx.x; c < c1; c += gridDim.x * RT) {
    float4 P = reinterpret_cast<const float4*>(p)[c], W = reinterpret_cast<const float4*>(w)[c];
    float4 Qv = reinterpret_cast<const float4*>(q)[c];
    const float4 S = reinterpret_cast<const float4*>(s)[c];
    float4 X = reinterpret_cast<const float4*>(x)[c], R = reinterpret_cast<const float4*>(r)[c];
    const float4 Dv = reinterpret_cast<const float4*>(dinv)[c];
    float* pa = &P.x;
    float* wa = &W.x;
    float* qa = &Qv.x;
    const float* sa = &S.x;
    float* xa = &X.x;
    float* ra = &R.x;
    const float* da = &Dv.x;
    const int g0 = 4 * c;
    const bool full = g0 >= ndir && g0 + 4 <= N;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (full || (g0 + j >= ndir && g0 + j < N)) {
        const float pg = fmaf(beta, pa[j], wa[j]);
        const float qg = fmaf(beta, qa[j], sa[j]);
        pa[j] = pg;
        qa[j] = qg;
        xa[j] = fmaf(alpha, pg, xa[j]);
        const float rg = fmaf(-alpha, qg, ra[j]);
        ra[j] = rg;
        const float wg = da[j] * rg;
        wa[j] = wg;
        rw = fmaf(rg, wg, rw);
        rr = fmaf(rg, rg, rr);
      }
    }
    reinterpret_cast<float4*>(p)[c] = P;
    reinterpret_cast<float4*>(q)[c] = Qv;
    reinterpret_cast<float4*>(x)[c] = X;
    reinterpret_cast<float4*>(r)[c] = R;
    reinterpret_cast<float4*>(w)[c] = W;
  }
  float v[2] = {rw, rr};
  const int slots[2] = {0, 1};
  block_partials<2>(v, partials, slots);
}

__device__ void scalars_iter_body(const double* partials, CgScalars* sc, const double* apart, int napart, int nv,
                                  int na);

template <typename T, bool SIGNED>
__device__ __forceinline__ T asm_value(const T* __restrict__ yloc, int c) {
  if (SIGNED) return c >= 0 ? yloc[c] : -yloc[~c];
  return yloc[c >= 0 ? c : ~c];  // sign^2 = 1 (diagonal assembly)
}

template <int K, typename T, bool SIGNED, bool PERM>
__device__ __forceinline__ void asm_class(const AsmPlan& P, int c, int cta, int ncta, bool skip_dir,
                                          const int* __restrict__ rows, const int* __restrict__ ecols,
                                          const T* __restrict__ yloc, T* __restrict__ s, const T* __restrict__ w,
                                          T& sw) {
  constexpr int U = K >= 4 ? 1 : 4 / K;  // rows per thread step (8 CTAs per SM hold the rest in flight)
  const int n = P.n[c];
  const int* R = rows + P.rows_off[c];
  const int stride = ncta * RT;
  for (int i = (skip_dir ? P.ndir[c] : 0) + cta * RT + threadIdx.x; i < n; i += U * stride) {
    int g[U];
    T val[U][K], wg[U];
    if constexpr (PERM) {
      // signed local values in the ELL layout: the row ids and the values load together
      const T* Y = yloc + P.col_off[c];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int ii = i + u * stride;
        const bool in = ii < n;
        g[u] = in ? R[ii] : -1;
#pragma unroll
        for (int j = 0; j < K; ++j) val[u][j] = in ? Y[(size_t)j * n + ii] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) wg[u] = (w != nullptr && g[u] >= 0) ? w[g[u]] : T(0);
    } else {
      const int* C = ecols + P.col_off[c];
      int idx[U][K];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int ii = i + u * stride;
        const bool in = ii < n;
        g[u] = in ? R[ii] : -1;
#pragma unroll
        for (int j = 0; j < K; ++j) idx[u][j] = in ? C[(size_t)j * n + ii] : 0;
      }
      // second level: every local value and w[g] of the U rows, all loads in flight
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int j = 0; j < K; ++j) val[u][j] = g[u] >= 0 ? asm_value<T, SIGNED>(yloc, idx[u][j]) : T(0);
        wg[u] = (w != nullptr && g[u] >= 0) ? w[g[u]] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (g[u] >= 0) {
        T acc = val[u][0];
#pragma unroll
        for (int j = 1; j < K; ++j) acc += val[u][j];
        s[g[u]] = acc;
        sw = fma(acc, wg[u], sw);
      }
    }
  }
}

// s[g] = sum_{local l of g} sign_l * yloc[l] over all rows (skip_dir: free rows only);
// partial s.w in slot 3. PERM: yloc is the assembly-ordered buffer of signed local values
// (ELL layout of P, tail rows at P.tail_off + rowptr[slot]), ecols and cols are unused. With fuse_sc != nullptr the last CTA to finish (ticket on
// `counter`) also runs the loop-tail scalar update, saving one launch per CG iteration;
// the reduction order of the partial sums does not depend on which CTA that is.
template <typename T, bool SIGNED = true, bool PERM = false>
__global__ void __launch_bounds__(RT, kAsmPerSM) assemble_dot_kernel(const AsmPlan P, bool skip_dir, const int* __restrict__ rows,
                                                          const int* __restrict__ ecols, const int* __restrict__ rowptr,
                                                          const int* __restrict__ cols, const T* __restrict__ yloc,
                                                          T* __restrict__ s, const T* __restrict__ w, const int* skip,
                                                          double* partials, CgScalars* fuse_sc = nullptr,
                                                          unsigned int* counter = nullptr,
                                                          const double* apart = nullptr, int napart = 0, int nv = RB) {
  if (skip != nullptr && *skip) return;
  int c = 0;
  while (c < kAsmK && (int)blockIdx.x >= P.cta0[c + 1]) ++c;
  const int cta = blockIdx.x - P.cta0[c], ncta = P.cta0[c + 1] - P.cta0[c];
  T sw = 0;  // per-thread s.w in T (FP32 sums stay off the slow FP64 pipe); CTA sum in FP64
  switch (c) {
    case 0: asm_class<1, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 1: asm_class<2, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 2: asm_class<3, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 3: asm_class<4, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 4: asm_class<5, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 5: asm_class<6, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 6: asm_class<7, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    case 7: asm_class<8, T, SIGNED, PERM>(P, c, cta, ncta, skip_dir, rows, ecols, yloc, s, w, sw); break;
    default: {  // longer rows: CSR
      const int n = P.n[kAsmK];
      const int* R = rows + P.rows_off[kAsmK];
      for (int i = (skip_dir ? P.ndir[kAsmK] : 0) + cta * RT + threadIdx.x; i < n; i += ncta * RT) {
        const int g = R[i];
        T acc = 0;
        if constexpr (PERM) {
          const T* Y = yloc + P.tail_off;
          for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) acc += Y[j];
        } else {
          for (int j = rowptr[g]; j < rowptr[g + 1]; ++j) acc += asm_value<T, SIGNED>(yloc, cols[j]);
        }
        s[g] = acc;
        if (w) sw = fma(acc, w[g], sw);
      }
    }
  }
  T v[1] = {sw};
  if (partials != nullptr && w != nullptr) {  // without w the element kernel summed s.w
    const int slots[1] = {3};
    block_partials<1>(v, partials, slots);
  }
  if (fuse_sc != nullptr) {
    __shared__ unsigned int ticket;
    if (threadIdx.x == 0) {  // thread 0 wrote this CTA's partial: visible before its ticket
      __threadfence();
      ticket = atomicAdd(counter, 1u);
    }
    __syncthreads();
    if (ticket == gridDim.x - 1) {
      __threadfence();
      scalars_iter_body(partials, fuse_sc, apart, napart, nv, w != nullptr ? (int)gridDim.x : 0);
      if (threadIdx.x == 0) *counter = 0u;  // re-armed for the next iteration
    }
  }
}

// ---- fused assembly + update of the FP32 inner iteration (scattered element output) ----
// One launch does what the assembly and the next update did: each free row g of each
// class gets s_g (an owned row: written by the element kernel; any other: the sum of its
// slots in the assembly-ordered buffer, in the assembly's order) and is updated at once,
// p, q, x, r, w = M^-1 r, with its r.w and r.r. The iteration's scalars (the reference
// loop tail, NekLinSysIterCG.cpp:219-261) come from a one-CTA kernel before it
// (scalars_fused_kernel): computing them in every CTA of the update had all CTAs read the
// same partials at once, and that hot spot in L2 cost more than the launch it saved.
// s is never written for the non-owned rows.
template <int K>
__device__ __forceinline__ void upd_class(const AsmPlan& P, int c, int cta, int ncta, const int* __restrict__ rows,
                                          const int* __restrict__ tail_ptr, const float* __restrict__ yslot,
                                          const float* __restrict__ s, float* __restrict__ x, float* __restrict__ r,
                                          float* __restrict__ w, float* __restrict__ p, float* __restrict__ q,
                                          const float* __restrict__ dinv, float alpha, float beta, float& rw,
                                          float& rr) {
  constexpr int U = (K >= 4 || K == 0) ? 2 : 4;  // rows per thread step, their loads in flight together
  const int n = P.n[c];
  const int* R = rows + P.rows_off[c];
  const int stride = ncta * RT;
  for (int i0 = P.ndir[c] + cta * RT + threadIdx.x; i0 < n; i0 += U * stride) {
    int g[U];
    float sg[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * stride;
      g[u] = i < n ? R[i] : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * stride;
      sg[u] = 0.f;
      if (g[u] < 0) continue;
      if constexpr (K == 1) {
        sg[u] = s[g[u]];  // owned row: the element kernel wrote it
      } else if constexpr (K > 1) {
        const float* Y = yslot + P.col_off[c];
        float v[K];
#pragma unroll
        for (int j = 0; j < K; ++j) v[j] = Y[(size_t)j * n + i];
        float acc = v[0];
#pragma unroll
        for (int j = 1; j < K; ++j) acc += v[j];
        sg[u] = acc;
      } else {  // K == 0: the tail class (more than kAsmK entries)
        const float* Y = yslot + P.tail_off;
        float acc = 0.f;
        for (int j = tail_ptr[i]; j < tail_ptr[i + 1]; ++j) acc += Y[j];
        sg[u] = acc;
      }
    }
    float pv[U], wv[U], qv[U], xv[U], rv[U], dv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int gg = g[u] >= 0 ? g[u] : 0;
      pv[u] = p[gg];
      wv[u] = w[gg];
      qv[u] = q[gg];
      xv[u] = x[gg];
      rv[u] = r[gg];
      dv[u] = dinv[gg];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (g[u] < 0) continue;
      const float pg = fmaf(beta, pv[u], wv[u]);
      const float qg = fmaf(beta, qv[u], sg[u]);
      p[g[u]] = pg;
      q[g[u]] = qg;
      x[g[u]] = fmaf(alpha, pg, xv[u]);
      const float rg = fmaf(-alpha, qg, rv[u]);
      r[g[u]] = rg;
      const float wg = dv[u] * rg;
      w[g[u]] = wg;
      rw = fmaf(rg, wg, rw);
      rr = fmaf(rg, rg, rr);
    }
  }
}

__global__ void __launch_bounds__(RT, kRedPerSM) asm_update_f32_kernel(const AsmPlan P, const int* __restrict__ rows,
                                                            const int* __restrict__ tail_ptr,
                                                            const float* __restrict__ yslot,
                                                            const float* __restrict__ s, float* __restrict__ x,
                                                            float* __restrict__ r, float* __restrict__ w,
                                                            float* __restrict__ p, float* __restrict__ q,
                                                            const float* __restrict__ dinv, double* partials,
                                                            const CgScalars* sc) {
  if (sc->done) return;
  const float alpha = (float)sc->alpha, beta = (float)sc->beta;
  float rw = 0.f, rr = 0.f;
  int c = 0;
  while (c < kAsmK && (int)blockIdx.x >= P.cta0[c + 1]) ++c;
  const int cta = blockIdx.x - P.cta0[c], ncta = P.cta0[c + 1] - P.cta0[c];
  switch (c) {
    case 0: upd_class<1>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 1: upd_class<2>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 2: upd_class<3>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 3: upd_class<4>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 4: upd_class<5>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 5: upd_class<6>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 6: upd_class<7>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    case 7: upd_class<8>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr); break;
    default: upd_class<0>(P, c, cta, ncta, rows, tail_ptr, yslot, s, x, r, w, p, q, dinv, alpha, beta, rw, rr);
  }
  float v[2] = {rw, rr};
  const int slots[2] = {0, 1};
  block_partials<2>(v, partials, slots);
}

// The loop tail of the fused iteration (one CTA): this iteration's scalars from the fused
// update's r.w, r.r and the element kernel's s.w (apart); right after the initial step
// (sc->fresh) they are already set and only the flag is cleared.
__global__ void __launch_bounds__(RT) scalars_fused_kernel(const double* partials, CgScalars* sc, const double* apart,
                                                           int napart, int nv) {
  if (sc->done) return;
  if (sc->fresh) {
    __syncthreads();
    if (threadIdx.x == 0) sc->fresh = 0;
    return;
  }
  scalars_iter_body(partials, sc, apart, napart, nv, 0);
}

// Reference initial step (NekLinSysIterCG.cpp:147-190). apart (napart entries): the
// element kernel's s.w partials, added to slot 3 where the element kernel summed s.w (the
// fused iteration's start); the scalars are then marked fresh for the first fused launch.
__global__ void __launch_bounds__(RT) scalars_init_kernel(const double* partials, CgScalars* sc, int nv, int na,
                                                          const double* apart = nullptr, int napart = 0) {
  const int slots[4] = {0, 1, 2, 3};
  double red[4];
  reduce_slots<4>(partials, slots, red, nv, na);
  double asw = 0.0;
  if (napart > 0) {
    double a[1] = {thread_partials<(RB + RT - 1) / RT>(apart, napart)}, o[1];
    block_sum<1>(a, o);
    asw = o[0];
  }
  const double rw = red[0], rr = red[1], bb = red[2], sw = red[3] + asw;
  if (threadIdx.x == 0) {
    sc->fresh = napart > 0 ? 1 : 0;
    sc->rhs_mag = sc->mag_override > 0 ? sc->mag_override : (bb > 1e-6 ? bb : 1.0);
    sc->eps = rr;
    sc->iters = 0;
    sc->k = 0;
    sc->status = ITHACA_GPU_OK;
    sc->done = 0;
    if (!isfinite(rr) || !isfinite(rw) || !isfinite(sw)) {
      sc->status = ITHACA_GPU_ERR_NUMERIC;
      sc->done = 1;
    } else if (rr < sc->tol2 * sc->rhs_mag) {
      sc->done = 1;
    } else {
      sc->rho = rw;
      sc->mu = sw;
      sc->beta = 0.0;
      sc->alpha = rw / sw;
      sc->iters = 1;
      if (sc->max_iter <= 0) {
        sc->status = ITHACA_GPU_ERR_NOT_CONVERGED;
        sc->done = 1;
      }
    }
  }
}

// Reference loop tail (NekLinSysIterCG.cpp:219-261).
__global__ void __launch_bounds__(RT) scalars_iter_kernel(const double* partials, CgScalars* sc, int nv, int na) {
  scalars_iter_body(partials, sc, nullptr, 0, nv, na);
}

// apart (napart entries): partials of s.w summed by the element kernel (the whole dot
// when it wrote the scattered output, the assembly's slot 3 then holding zeros), added
// to slot 3 (in a fixed order).
__device__ void scalars_iter_body(const double* partials, CgScalars* sc, const double* apart, int napart, int nv,
                                  int na) {
  if (sc->done) return;
  // Few FP64 instructions (one CTA does this between two kernels): each thread sums its
  // share of slots 0, 1, 3 and of the element kernel's partials (loads in flight
  // together, empty sources skipped), then warp 0 sums the 256 shares of each.
  constexpr int MV = (RB + RT - 1) / RT;
  double a[4];
  a[0] = thread_partials<MV>(partials + 0 * RB, nv);
  a[1] = thread_partials<MV>(partials + 1 * RB, nv);
  a[2] = na > 0 ? thread_partials<kMaxP>(partials + 3 * RB, na) : 0.0;
  a[3] = napart > 0 ? thread_partials<MV>(apart, napart) : 0.0;
  __shared__ double sh[4][RT];
#pragma unroll
  for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  if (threadIdx.x >= 32) return;
  constexpr int PER = RT / 32;
  double red[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double t = sh[k][threadIdx.x * PER];
#pragma unroll
    for (int i = 1; i < PER; ++i) t += sh[k][threadIdx.x * PER + i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    red[k] = t;
  }
  const double rho_new = red[0], eps = red[1], mu = red[2] + red[3];
  if (threadIdx.x == 0) {
    sc->eps = eps;
    sc->mu = mu;
    sc->iters += 1;
    if (!isfinite(eps) || !isfinite(rho_new) || !isfinite(mu)) {
      sc->status = ITHACA_GPU_ERR_NUMERIC;
      sc->done = 1;
    } else if (eps < sc->tol2 * sc->rhs_mag) {
      sc->done = 1;
    } else {
      const double beta = rho_new / sc->rho;
      sc->alpha = rho_new / (mu - rho_new * beta / sc->alpha);
      sc->beta = beta;
      sc->rho = rho_new;
      sc->k += 1;
      if (sc->k >= sc->max_iter) {
        sc->status = ITHACA_GPU_ERR_NOT_CONVERGED;
        sc->done = 1;
      }
    }
  }
}

// ---- FP64 outer-step kernels ----------------------------------------------------
// r[g] = b[g] - sum yloc (g >= ndir), partial r.r -> slot 1; b.b -> slot 2.
__global__ void __launch_bounds__(RT) residual_kernel(int N, int ndir, const int* __restrict__ rowptr,
                                                      const int* __restrict__ cols, const double* __restrict__ yloc,
                                                      const double* __restrict__ b, double* __restrict__ r,
                                                      double* partials) {
  double v[2] = {0, 0};
  for (int g = ndir + blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) {
    double acc = 0;
    if (yloc != nullptr)  // nullptr: x = 0, so r = b
      for (int j = rowptr[g]; j < rowptr[g + 1]; ++j) {
        const int c = cols[j];
        acc += c >= 0 ? yloc[c] : -yloc[~c];
      }
    const double rg = b[g] - acc;
    r[g] = rg;
    v[0] += rg * rg;
    v[1] += b[g] * b[g];
  }
  const int slots[2] = {1, 2};
  block_partials<2>(v, partials, slots);
}

__global__ void reduce_to_kernel(const double* partials, int slot, int n, double* out) {
  const double v = reduce_slot(partials, slot, n);
  if (threadIdx.x == 0) *out = v;
}

// r32 = r64 * scale on g >= ndir, zero below.
__global__ void __launch_bounds__(RT) scale_to_f32_kernel(int N, int ndir, const double* __restrict__ r,
                                                          const double* __restrict__ scale_src, float* __restrict__ r32) {
  const double sc = 1.0 / sqrt(*scale_src);
  for (int g = blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) r32[g] = g >= ndir ? (float)(r[g] * sc) : 0.f;
}

// x64 += sqrt(*scale_src) * d32 on g >= ndir.
__global__ void __launch_bounds__(RT) axpy_f32_kernel(int N, int ndir, const double* __restrict__ scale_src,
                                                      const float* __restrict__ d32, double* __restrict__ x) {
  const double sc = sqrt(*scale_src);
  for (int g = ndir + blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) x[g] += sc * (double)d32[g];
}

// b[g] -= y[g] for g in [first, N).
__global__ void __launch_bounds__(RT) sub_rows_kernel(int N, int first, const double* __restrict__ y,
                                                      double* __restrict__ b) {
  for (int g = first + blockIdx.x * RT + threadIdx.x; g < N; g += gridDim.x * RT) b[g] -= y[g];
}

__global__ void __launch_bounds__(RT) inv_kernel(int n, const double* __restrict__ d, double* __restrict__ dinv,
                                                 float* __restrict__ dinv32, int ndir) {
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    const double v = g >= ndir ? 1.0 / d[g] : 0.0;
    dinv[g] = v;
    if (dinv32) dinv32[g] = (float)v;
  }
}

// local[l] = sign * x[g] (AssemblyMapCG::GlobalToLocal), l2g signed-encoded.
__global__ void __launch_bounds__(RT) g2l_kernel(size_t nloc, const int* __restrict__ l2g,
                                                 const double* __restrict__ x, double* __restrict__ loc) {
  for (size_t l = (size_t)blockIdx.x * RT + threadIdx.x; l < nloc; l += (size_t)gridDim.x * RT) {
    const int c = l2g[l];
    loc[l] = c >= 0 ? x[c] : -x[~c];
  }
}

__global__ void __launch_bounds__(RT) neg_kernel(size_t n, double* __restrict__ a) {
  for (size_t i = (size_t)blockIdx.x * RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) a[i] = -a[i];
}

template <typename T>
__global__ void __launch_bounds__(RT) cast_kernel(size_t n, const double* __restrict__ a, T* __restrict__ b) {
  for (size_t i = (size_t)blockIdx.x * RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) b[i] = (T)a[i];
}

// ---- successive right-hand sides: small dense products with the stored solutions ----
constexpr int kMaxSuccessive = 64;
struct ProjCoef {
  double c[kMaxSuccessive];
};

// part[v * gridDim.x + cta] = this CTA's share of sum_i V[v ld + i] y[i], i < n (one
// CTA row of the grid per stored vector v = blockIdx.y; fixed summation order).
__global__ void __launch_bounds__(RT) multidot_part_kernel(int n, const double* __restrict__ V, size_t ld,
                                                           const double* __restrict__ y, double* part) {
  const double* v = V + (size_t)blockIdx.y * ld;
  double acc = 0;
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) acc = fma(v[i], y[i], acc);
  __shared__ double sh[RT / 32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < RT / 32; ++w) t += sh[w];
    part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
}

// out[v] = sum of the nparts partials of vector v (one CTA per v, fixed order).
__global__ void __launch_bounds__(RT) multidot_final_kernel(const double* part, int nparts, double* out) {
  const double* p = part + (size_t)blockIdx.x * nparts;
  double acc = 0;
  for (int i = threadIdx.x; i < nparts; i += RT) acc += p[i];
  __shared__ double sh[RT / 32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < RT / 32; ++w) t += sh[w];
    out[blockIdx.x] = t;
  }
}

// out[i] = sum_{v < nv} coef[v] V[v ld + i] for i < n.
__global__ void __launch_bounds__(RT) combine_kernel(int n, int nv, const double* __restrict__ V, size_t ld,
                                                     const ProjCoef coef, double* __restrict__ out) {
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    double acc = 0;
    for (int v = 0; v < nv; ++v) acc = fma(coef.c[v], V[(size_t)v * ld + i], acc);
    out[i] = acc;
  }
}

// dst[i] = a * src[i] (i < n); dst[i] += src[i] when add.
__global__ void __launch_bounds__(RT) scale_copy_kernel(int n, double a, const double* __restrict__ src,
                                                        double* __restrict__ dst, int add) {
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) dst[i] = add ? dst[i] + src[i] : a * src[i];
}

// ---- solver object --------------------------------------------------------------
// State of the successive-right-hand-side projection (GlobalLinSysIterative.cpp:156-482):
// up to m stored solutions (free part only, nf = N - ndir values each), normalised as
// the reference normalises them, and the symmetric coefficient matrix of their products.
struct SuccessiveRhs {
  int m = 0;             // buffer size (0: off)
  bool aconj = true;     // A-conjugate basis (the reference's positive SuccessiveRHS)
  int nprev = 0;         // solutions accepted so far (m_numPrevSols)
  int nstored = 0;       // vectors in the buffer (m_prevBasis.size())
  double lambda = NAN;   // the operator the stored solutions belong to
  std::vector<int> slot; // slot[i]: storage column of the reference's vector i
  std::vector<double> M; // coefficient matrix, nstored x nstored, row-major
  double* sols = nullptr;   // m x nf: x_i / norm_i
  double* basis = nullptr;  // m x nf: A x_i / ||A x_i|| (non-conjugate mode only)
  double *px = nullptr, *ax = nullptr, *bsave = nullptr, *part = nullptr, *dots = nullptr;
  int nparts = 0;
  void release() {
    for (double* p : {sols, basis, px, ax, bsave, part, dots}) cudaFree(p);
    sols = basis = px = ax = bsave = part = dots = nullptr;
  }
};

template <typename T>
struct Vecs {
  T *x = nullptr, *r = nullptr, *w = nullptr, *s = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr,
    *yloc = nullptr, *b = nullptr;
  void alloc(size_t N, size_t nloc) {
    T** v[] = {&x, &r, &w, &s, &p, &q, &dinv, &b};
    const size_t N4 = (N + 3) / 4 * 4;  // padded for the four-wide FP32 update
    for (auto pp : v) {
      ITHACA_CUDA(cudaMalloc(pp, sizeof(T) * N4));
      ITHACA_CUDA(cudaMemset(*pp, 0, sizeof(T) * N4));
    }
    ITHACA_CUDA(cudaMalloc(&yloc, sizeof(T) * nloc));
  }
  void release() {
    for (T* p0 : {x, r, w, s, p, q, dinv, yloc, b}) cudaFree(p0);
  }
};

struct Cg {
  Op* op = nullptr;
  int N = 0, ndir = 0;
  size_t nloc = 0;
  int* l2g = nullptr;     // signed-encoded
  int* rowptr = nullptr;  // N + 1
  int rbv = RB, rba = RBA;  // CTAs of the vector kernels and of the assembly (fewer for small systems)
  AsmPlan plan{};           // assembly by row classes (see AsmPlan)
  // Scattered output of the inner iteration's pipelined FP32 element kernel: it writes
  // the owned rows (one local entry, free) into s itself and every other signed local
  // value into its slot of the assembly-ordered buffer (the ELL layout of plan, then the
  // tail rows' entries at plan.tail_off + tail_ptr[slot] + j), which the assembly
  // (plan_own: the same classes without the owned rows) reads with unit stride.
  bool own_ok = false;
  int* ocode = nullptr;     // nloc output codes (see OwnedRows)
  int* tail_ptr = nullptr;  // rows of the tail class + 1: first slot of each row's entries
  AsmPlan plan_own{};
  // persistent small-system solver (2-D, cg_persist.cu): -1 automatic (N <= kPersistMaxN),
  // 0 off, 1 whenever the system is 2-D; grid-barrier state; SM count
  int persist = -1;
  long long dbg_polls = 0;            // failure-path test hooks of the persistent solver
  int dbg_drop = -1, dbg_delay = 0;   // (PersistArgs); zero / -1 in a solve
  unsigned* bar = nullptr;
  int sms = 0;
  double* opart = nullptr;  // per-CTA s.w partials of the element kernel
  int opart_cap = 0;
  int* asm_rows = nullptr;  // N: global rows, grouped by class
  int* asm_cols = nullptr;  // ELL entries of the classes with at most kAsmK entries
  int* cols = nullptr;    // nloc, signed-encoded local index
  Vecs<double> v64;
  Vecs<float> v32;
  bool have32 = false;
  float* jg32 = nullptr;   // FP32 copy of the geometry the solver uses
  // half-precision geometry with per-element, per-field scales (mixed mode with 16-bit
  // geometry, curved hexahedra); geo16 selects it for the FP32 applies of the solve
  void* jg16 = nullptr;
  float* jgs = nullptr;
  bool have16 = false, geo16 = false, graph32_geo16 = false;
  double* jgk64 = nullptr; // geometry with the metric scaled by a variable coefficient (else op->jg64)
  bool aniso = false;       // jgk64 holds an anisotropic (tensor) coefficient
  double* adj_scratch = nullptr;
  double* partials = nullptr;
  double* dscal = nullptr;  // scratch doubles (norms)
  unsigned int* counter = nullptr;  // CTA ticket of the fused assembly + scalar update
  // fused FP32 inner iteration (asm_update_f32_kernel): the full row classes with the CTAs
  // split by the update's work (upd_ok: every class with free rows has a CTA), the element
  // kernel's grid (its s.w partials), on / off
  AsmPlan plan_upd{};
  bool upd_ok = false;
  int own_ctas = -1;
  bool fuse_tail = false;
  bool graph32_fused = false;
  CgScalars* sc = nullptr;
  CgScalars* sc_host = nullptr;  // pinned
  double diag_lambda = NAN;
  cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
  int graph64_len = 0, graph32_len = 0;
  // geometry each graph was captured with: the kernels' parameters hold the pointer, so a
  // coefficient set later (a new geometry buffer) needs a new capture
  const void* graph64_geo = nullptr;
  const void* graph32_geo = nullptr;
  // element-kernel variant each graph was captured with (a variant set later needs a new
  // capture too: the captured launch names its kernel)
  int graph64_variant = -1, graph32_variant = -1;
  SuccessiveRhs proj;
  ~Cg();
};

Cg::~Cg() {
  proj.release();
  if (graph64) cudaGraphExecDestroy(graph64);
  if (graph32) cudaGraphExecDestroy(graph32);
  cudaFree(l2g);
  cudaFree(rowptr);
  cudaFree(asm_rows);
  cudaFree(ocode);
  cudaFree(tail_ptr);
  cudaFree(bar);
  cudaFree(opart);
  cudaFree(asm_cols);
  cudaFree(cols);
  v64.release();
  if (have32) v32.release();
  cudaFree(jg32);
  cudaFree(jg16);
  cudaFree(jgs);
  cudaFree(jgk64);
  cudaFree(adj_scratch);
  cudaFree(partials);
  cudaFree(dscal);
  cudaFree(counter);
  cudaFree(sc);
  if (sc_host) cudaFreeHost(sc_host);
}

static const int* skip_ptr(Cg* cg) { return &cg->sc->done; }

// FP64 geometry of the system: the operator's, or its variable-coefficient copy.
static const double* geo64(Cg* cg) { return cg->jgk64 ? cg->jgk64 : cg->op->jg64; }

// Gather (signed l2g; ids < ndir read as zero when zero_dir) + element Helmholtz into v.yloc.
// With own != nullptr (FP32) the pipelined kernels also assemble the owned rows into
// own->s and report how many partials they wrote in own->ctas (-1: not done, the caller
// assembles every row).
template <typename T>
static void launch_apply(Cg* cg, Vecs<T>& v, const T* tab, const T* jg, T lambda, const T* lam_ptr, const T* xin,
                         cudaStream_t s, bool zero_dir, const int* skip, OwnedRows* own = nullptr) {
  Op* op = cg->op;
  bool ok;
  if (own != nullptr) own->ctas = -1;
  if constexpr (sizeof(T) == 4) {
    const int* map = cg->l2g;
    if (own != nullptr) own->ocode = cg->ocode;
    if (cg->geo16)
      ok = launch_helm_pipe_geo16(op->n, op->Q, op->E, op->variant32, op->hB.data(), op->hD.data(), cg->jg16, cg->jgs, lambda, xin,
                                  v.yloc, map, zero_dir ? cg->ndir : 0, skip, lam_ptr, op->ctx->derr, s, own);
    else if (op->kdim == 3 && op->deformed && op->variant32 > 0)
      ok = launch_helm_pencil<float>(op->n, op->Q, op->E, op->variant32, op->hB.data(), op->hD.data(), jg, lambda,
                                     xin, v.yloc, map,
                                     zero_dir ? cg->ndir : 0, skip, lam_ptr, op->ctx->derr, s, own);
    else
      ok = launch_helmholtz<T>(op->kdim, op->n, op->Q, op->E, op->deformed, tab, jg, lambda, xin, v.yloc, cg->l2g,
                               zero_dir ? cg->ndir : 0, s, skip, lam_ptr);
  } else {
    ok = false;
    if (op->kdim == 3 && op->deformed && op->variant64 > 0)  // even-odd pencil kernel where it is built
      ok = launch_helm_pencil64(op->n, op->Q, op->E, op->variant64, op->hB.data(), op->hD.data(), jg, lambda, xin,
                                v.yloc, cg->l2g, zero_dir ? cg->ndir : 0, skip, lam_ptr, op->ctx->derr, s);
    if (!ok)
      ok = launch_helmholtz<T>(op->kdim, op->n, op->Q, op->E, op->deformed, tab, jg, lambda, xin, v.yloc, cg->l2g,
                               zero_dir ? cg->ndir : 0, s, skip, lam_ptr);
  }
  if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz: (modes, points) combination not built");
  op->ctx->launches++;
}

template <typename T>
static const T* lam_dev(Cg* cg);
template <>
const double* lam_dev<double>(Cg* cg) { return &cg->sc->lambda; }
template <>
const float* lam_dev<float>(Cg* cg) { return &cg->sc->lambda32; }

// One PCG iteration: update -> gather+apply -> assemble(+s.w, + scalars in the last CTA).
template <typename T>
static void enqueue_iteration(Cg* cg, Vecs<T>& v, const T* tab, const T* jg, cudaStream_t s) {
  if constexpr (sizeof(T) == 4)
    pcg_update_f32x4_kernel<<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, cg->sc, v.x, v.r, v.w, v.s, v.p, v.q, v.dinv,
                                              cg->partials);
  else
    pcg_update_kernel<T><<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, cg->sc, v.x, v.r, v.w, v.s, v.p, v.q, v.dinv,
                                           cg->partials);
  OwnedRows own;
  if constexpr (sizeof(T) == 4) {
    own.s = v.s;
    own.part = cg->opart;
  }
  const bool try_own = sizeof(T) == 4 && cg->own_ok;
  launch_apply<T>(cg, v, tab, jg, T(0), lam_dev<T>(cg), v.w, s, true, skip_ptr(cg), try_own ? &own : nullptr);
  if (try_own && own.ctas >= 0) {  // the element kernel wrote the owned rows of s
    if (own.ctas > cg->opart_cap) fail(ITHACA_GPU_ERR_ARG, "element kernel launched more CTAs than partial slots");
    // the element kernel summed the whole s.w (its partials in opart): no w here
    assemble_dot_kernel<T, true, true><<<cg->rba, RT, 0, s>>>(cg->plan_own, true, cg->asm_rows, nullptr, cg->tail_ptr,
                                                         nullptr, v.yloc, v.s, nullptr, skip_ptr(cg), cg->partials,
                                                         cg->sc, cg->counter, cg->opart, own.ctas, cg->rbv);
  } else {
    assemble_dot_kernel<T><<<cg->rba, RT, 0, s>>>(cg->plan, true, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols,
                                             v.yloc, v.s, v.w, skip_ptr(cg), cg->partials, cg->sc, cg->counter,
                                             nullptr, 0, cg->rbv);
  }
  cg->op->ctx->launches += 2;
}

// One fused FP32 iteration (scattered element output): the assembly and update of the
// previous apply's output with this iteration's scalars (asm_update_f32_kernel), then the
// gather + element apply of the new w, which writes the owned rows of s, the slots of the
// others and its s.w partials.
static void enqueue_iteration_fused(Cg* cg, Vecs<float>& v, const float* tab, const float* jg, cudaStream_t s) {
  scalars_fused_kernel<<<1, RT, 0, s>>>(cg->partials, cg->sc, cg->opart, cg->own_ctas, cg->rbv);
  asm_update_f32_kernel<<<cg->rbv, RT, 0, s>>>(cg->plan_upd, cg->asm_rows, cg->tail_ptr, v.yloc, v.s, v.x, v.r, v.w,
                                               v.p, v.q, v.dinv, cg->partials, cg->sc);
  OwnedRows own;
  own.s = v.s;
  own.part = cg->opart;
  launch_apply<float>(cg, v, tab, jg, 0.f, lam_dev<float>(cg), v.w, s, true, skip_ptr(cg), &own);
  if (own.ctas != cg->own_ctas) fail(ITHACA_GPU_ERR_ARG, "element kernel grid changed within a fused solve");
  cg->op->ctx->launches += 2;  // (+1 in launch_apply)
}

template <typename T>
static cudaGraphExec_t capture_chunk(Cg* cg, Vecs<T>& v, const T* tab, const T* jg, int iters, bool fused = false) {
  cudaStream_t s = cg->op->ctx->stream;
  cudaGraph_t g;
  ITHACA_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const long long before = cg->op->ctx->launches;
  for (int i = 0; i < iters; ++i) {
    if constexpr (sizeof(T) == 4) {
      if (fused) {
        enqueue_iteration_fused(cg, v, tab, jg, s);
        continue;
      }
    }
    enqueue_iteration<T>(cg, v, tab, jg, s);
  }
  cg->op->ctx->launches = before;  // captured, not launched
  ITHACA_CUDA(cudaStreamEndCapture(s, &g));
  cudaGraphExec_t ex;
  ITHACA_CUDA(cudaGraphInstantiate(&ex, g, 0));
  cudaGraphDestroy(g);
  return ex;
}

// Runs the reference PCG recurrence on vectors of type T with right-hand side v.b;
// the final scalars are left in sc_host. lambda is read from the device scalars.
template <typename T>
static void run_pcg(Cg* cg, Vecs<T>& v, const T* tab, const T* jg, double lambda, double tol2, double mag_override,
                    int max_iter, int chunk) {
  Ctx* c = cg->op->ctx;
  cudaStream_t s = c->stream;
  CgScalars init{};
  init.tol2 = tol2;
  init.mag_override = mag_override;
  init.max_iter = max_iter;
  init.lambda = lambda;
  init.lambda32 = (float)lambda;
  *cg->sc_host = init;
  ITHACA_CUDA(cudaMemcpyAsync(cg->sc, cg->sc_host, sizeof(CgScalars), cudaMemcpyHostToDevice, s));
  Op* op = cg->op;
  const bool persist = op->kdim == 2 && cg->own_ok && cg->bar != nullptr && !cg->geo16 &&
                       (cg->persist == 1 || (cg->persist < 0 && cg->N <= kPersistMaxN));
  if (persist) {  // the whole solve in one cooperative launch (cg_persist.cu)
    PersistArgs<T> a{};
    a.N = cg->N;
    a.ndir = cg->ndir;
    a.E = op->E;
    a.deformed = op->deformed;
    a.l2g = cg->l2g;
    a.ocode = cg->ocode;
    a.asm_rows = cg->asm_rows;
    a.tail_ptr = cg->tail_ptr;
    a.plan = cg->plan;
    a.x = v.x;
    a.r = v.r;
    a.w = v.w;
    a.s = v.s;
    a.p = v.p;
    a.q = v.q;
    a.yslot = v.yloc;
    a.b = v.b;
    a.dinv = v.dinv;
    a.tab = tab;
    a.jg = jg;
    a.part = cg->partials;
    a.bar = cg->bar;
    a.err = c->derr;
    a.sc = cg->sc;
    a.dbg_polls = cg->dbg_polls;
    a.dbg_drop_cta = cg->dbg_drop;
    a.dbg_delay_ns = cg->dbg_delay;
    if (launch_cg2_persistent<T>(op->n, op->Q, a, cg->sms, s)) {
      c->launches++;
      ITHACA_CUDA(cudaMemcpyAsync(cg->sc_host, cg->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s));
      ITHACA_CUDA(cudaStreamSynchronize(s));
      c->check_device_error();
      return;
    }
  }
  pcg_init_kernel<T><<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, v.b, v.x, v.r, v.w, v.dinv, cg->partials);
  // fused FP32 iterations need the scattered output of a pipelined element kernel: the
  // initial apply tries it, and the solve falls back to the separate assembly and update
  // where the kernel cannot write it
  bool fused = false, tried = false;
  OwnedRows own0;
  if constexpr (sizeof(T) == 4) {
    if (cg->fuse_tail && cg->own_ok && cg->upd_ok) {
      tried = true;
      own0.s = v.s;
      own0.part = cg->opart;
      launch_apply<float>(cg, v, tab, jg, 0.f, lam_dev<float>(cg), v.w, s, true, nullptr, &own0);
      if (own0.ctas > cg->opart_cap) fail(ITHACA_GPU_ERR_ARG, "element kernel launched more CTAs than partial slots");
      fused = own0.ctas >= 0;
    }
  }
  if (fused) {
    cg->own_ctas = own0.ctas;
    scalars_init_kernel<<<1, RT, 0, s>>>(cg->partials, cg->sc, cg->rbv, 0, cg->opart, own0.ctas);
    c->launches += 2;
  } else {
    // an attempt that could not scatter wrote the element-ordered output already
    if (!tried) launch_apply<T>(cg, v, tab, jg, T(0), lam_dev<T>(cg), v.w, s, true, nullptr);
    assemble_dot_kernel<T><<<cg->rba, RT, 0, s>>>(cg->plan, true, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols,
                                             v.yloc, v.s, v.w, nullptr, cg->partials);
    scalars_init_kernel<<<1, RT, 0, s>>>(cg->partials, cg->sc, cg->rbv, cg->rba);
    c->launches += 3;
  }
  ITHACA_CUDA(cudaGetLastError());
  cudaGraphExec_t& ex = sizeof(T) == 8 ? cg->graph64 : cg->graph32;
  int& len = sizeof(T) == 8 ? cg->graph64_len : cg->graph32_len;
  const void*& geo = sizeof(T) == 8 ? cg->graph64_geo : cg->graph32_geo;
  int& gvar = sizeof(T) == 8 ? cg->graph64_variant : cg->graph32_variant;
  const int var = sizeof(T) == 8 ? cg->op->variant64 : cg->op->variant32;
  const bool geo_changed = (sizeof(T) == 4 && cg->graph32_geo16 != cg->geo16) || geo != (const void*)jg;
  const bool fused_changed = sizeof(T) == 4 && cg->graph32_fused != fused;
  if (!ex || len != chunk || geo_changed || gvar != var || fused_changed) {
    if (ex) cudaGraphExecDestroy(ex);
    ex = nullptr;
    ex = capture_chunk<T>(cg, v, tab, jg, chunk, fused);
    len = chunk;
    geo = jg;
    gvar = var;
    if (sizeof(T) == 4) {
      cg->graph32_geo16 = cg->geo16;
      cg->graph32_fused = fused;
    }
  }
  // Bounded host loop: at most max_iter / chunk + 2 graph launches.
  const long long max_launches = (long long)max_iter / chunk + 2;
  for (long long it = 0;; ++it) {
    ITHACA_CUDA(cudaMemcpyAsync(cg->sc_host, cg->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaStreamSynchronize(s));
    if (cg->sc_host->done) break;
    if (it >= max_launches) fail(ITHACA_GPU_ERR_TIMEOUT, "CG did not flag completion within its iteration bound");
    ITHACA_CUDA(cudaGraphLaunch(ex, s));
    c->launches += 3LL * chunk;
  }
}

static void ensure_fp32(Cg* cg) {
  if (cg->have32) return;
  Op* op = cg->op;
  cg->v32.alloc(cg->N, cg->nloc);
  const size_t njg = (size_t)op->E * n_jg(op->dim) * (op->deformed ? op->nq : 1);
  ITHACA_CUDA(cudaMalloc(&cg->jg32, sizeof(float) * njg + kGeoPad));
  cast_kernel<float><<<RB, RT, 0, op->ctx->stream>>>(njg, geo64(cg), cg->jg32);
  op->ctx->launches++;
  cg->have32 = true;
  cg->diag_lambda = NAN;  // rebuild so that the FP32 inverse diagonal is filled too
}

// Half-precision geometry: one CTA per element; for each of the 7 fields the scale is the
// field's largest magnitude over the element's points and the stored halves are the
// values divided by it (|half| <= 1, round to nearest).
__global__ void __launch_bounds__(256) geo16_kernel(int nq, const double* __restrict__ jg, __half* __restrict__ jg16,
                                                    float* __restrict__ jgs) {
  __shared__ double red[256 / 32];
  const int e = blockIdx.x;
  for (int f = 0; f < 7; ++f) {
    const double* src = jg + ((size_t)e * 7 + f) * nq;
    double m = 0;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) m = fmax(m, fabs(src[q]));
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    double mx = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, red[w]);
    __syncthreads();
    const double sc = mx > 0 ? mx : 1.0;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) jg16[((size_t)e * 7 + f) * nq + q] = __double2half(src[q] / sc);
    if (threadIdx.x == 0) jgs[(size_t)e * 8 + f] = (float)sc;
  }
  if (threadIdx.x == 0) jgs[(size_t)e * 8 + 7] = 0.f;
}

static void build_geo16(Cg* cg) {
  Op* op = cg->op;
  geo16_kernel<<<op->E, 256, 0, op->ctx->stream>>>(op->nq, geo64(cg), static_cast<__half*>(cg->jg16), cg->jgs);
  op->ctx->launches++;
  ITHACA_CUDA(cudaGetLastError());
}

static void ensure_geo16(Cg* cg) {
  if (cg->have16) return;
  Op* op = cg->op;
  if (!(op->kdim == 3 && op->deformed))
    fail(ITHACA_GPU_ERR_UNSUPPORTED, "16-bit geometry is built for curved (deformed) hexahedra");
  const size_t njg = (size_t)op->E * 7 * op->nq;
  ITHACA_CUDA(cudaMalloc(&cg->jg16, sizeof(__half) * njg + kGeoPad));
  ITHACA_CUDA(cudaMalloc(&cg->jgs, sizeof(float) * 8 * op->E));
  build_geo16(cg);
  cg->have16 = true;
}

// Assembled Jacobi diagonal (sum of element diagonals, sign^2 = 1) and its inverse.
static void ensure_diag(Cg* cg, double lambda) {
  if (cg->diag_lambda == lambda) return;
  Op* op = cg->op;
  cudaStream_t s = op->ctx->stream;
  if (!launch_helm_diag<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, geo64(cg), lambda,
                                cg->v64.yloc, s))
    fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz diagonal: (modes, points) combination not built");
  assemble_dot_kernel<double, false><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, cg->v64.yloc, cg->v64.s,
                                                       nullptr, nullptr, nullptr);
  inv_kernel<<<RB, RT, 0, s>>>(cg->N, cg->v64.s, cg->v64.dinv, cg->have32 ? cg->v32.dinv : nullptr, cg->ndir);
  op->ctx->launches += 3;
  ITHACA_CUDA(cudaGetLastError());
  cg->diag_lambda = lambda;
}

// FP64 residual r = b - A x over the non-Dirichlet dofs; ||r||^2 -> dscal[0], ||b||^2 -> dscal[1].
// x == nullptr stands for x = 0 (r = b, no operator apply).
static void fp64_residual(Cg* cg, double lambda, const double* x, const double* b, double* r) {
  cudaStream_t s = cg->op->ctx->stream;
  if (x != nullptr) launch_apply<double>(cg, cg->v64, cg->op->t64.base, geo64(cg), lambda, nullptr, x, s, true, nullptr);
  residual_kernel<<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, cg->rowptr, cg->cols, x != nullptr ? cg->v64.yloc : nullptr, b,
                                    r, cg->partials);
  reduce_to_kernel<<<1, RT, 0, s>>>(cg->partials, 1, cg->rbv, cg->dscal);
  reduce_to_kernel<<<1, RT, 0, s>>>(cg->partials, 2, cg->rbv, cg->dscal + 1);
  cg->op->ctx->launches += 3;
}

static void solve_impl(Cg* cg, double lambda, const ithaca_gpu_cg_opts& o, ithaca_gpu_cg_result* res) {
  Ctx* c = cg->op->ctx;
  cudaStream_t s = c->stream;
  const bool mixed = o.mode == ITHACA_GPU_SOLVE_MIXED_FP32 || o.mode == ITHACA_GPU_SOLVE_MIXED_FP32_GEO16;
  if (mixed) ensure_fp32(cg);
  if (o.mode == ITHACA_GPU_SOLVE_MIXED_FP32_GEO16) ensure_geo16(cg);
  cg->geo16 = o.mode == ITHACA_GPU_SOLVE_MIXED_FP32_GEO16;
  struct Geo16Reset {  // the 16-bit geometry is selected for this solve only
    Cg* c;
    ~Geo16Reset() { c->geo16 = false; }
  } geo16_reset{cg};
  ensure_diag(cg, lambda);
  const int chunk = std::max(1, std::min(o.check_every, 64));
  const double tol = std::max(o.tol, 1e-16);  // tolerance floor of NekLinSysIter.cpp:83
  ithaca_gpu_cg_result out{};
  int status = ITHACA_GPU_OK;
  if (o.mode == ITHACA_GPU_SOLVE_FP64) {
    run_pcg<double>(cg, cg->v64, cg->op->t64.base, geo64(cg), lambda, tol * tol, 0.0, o.max_iter, chunk);
    out.iterations = cg->sc_host->iters;
    out.eps = cg->sc_host->eps;
    out.rhs_magnitude = cg->sc_host->rhs_mag;
    status = cg->sc_host->status;
  } else if (mixed) {
    double hs[2];
    // x64 = 0; r64 = b
    ITHACA_CUDA(cudaMemsetAsync(cg->v64.x, 0, sizeof(double) * cg->N, s));
    fp64_residual(cg, lambda, nullptr, cg->v64.b, cg->v64.r);
    ITHACA_CUDA(cudaMemcpyAsync(hs, cg->dscal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaStreamSynchronize(s));
    const double bnorm2 = hs[1];
    double rnorm2 = hs[0];
    int total_inner = 0, outer = 0;
    const double inner2 = o.inner_tol * o.inner_tol;
    while (rnorm2 > tol * tol * bnorm2 && bnorm2 > 0) {
      if (outer >= o.max_outer || total_inner >= o.max_iter) {
        status = ITHACA_GPU_ERR_NOT_CONVERGED;
        break;
      }
      if (!std::isfinite(rnorm2)) {
        status = ITHACA_GPU_ERR_NUMERIC;
        break;
      }
      // r32 = r64 / ||r64||, inner FP32 PCG from zero to relative inner_tol
      scale_to_f32_kernel<<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, cg->v64.r, cg->dscal, cg->v32.b);
      c->launches++;
      run_pcg<float>(cg, cg->v32, cg->op->t32.base, cg->jg32, lambda, inner2, 1.0, o.max_iter - total_inner, chunk);
      total_inner += cg->sc_host->iters;
      const int st = cg->sc_host->status;
      if (st == ITHACA_GPU_ERR_NUMERIC) {
        status = st;
        break;
      }
      // x64 += ||r|| d32 ; r64 = b - A x64
      axpy_f32_kernel<<<cg->rbv, RT, 0, s>>>(cg->N, cg->ndir, cg->dscal, cg->v32.x, cg->v64.x);
      c->launches++;
      fp64_residual(cg, lambda, cg->v64.x, cg->v64.b, cg->v64.r);
      ITHACA_CUDA(cudaMemcpyAsync(hs, cg->dscal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
      ITHACA_CUDA(cudaStreamSynchronize(s));
      rnorm2 = hs[0];
      ++outer;
    }
    out.iterations = total_inner;
    out.outer_iterations = outer;
    out.eps = rnorm2;
    out.rhs_magnitude = bnorm2 > 1e-6 ? bnorm2 : 1.0;
    // the last outer step's FP64 residual is the residual of the returned x
    out.rel_residual = bnorm2 > 0 ? std::sqrt(rnorm2 / bnorm2) : 0.0;
  } else {
    fail(ITHACA_GPU_ERR_ARG, "unknown solve mode");
  }
  if (!mixed) {  // final FP64 relative residual ||b - A x|| / ||b||
    double hs[2];
    fp64_residual(cg, lambda, cg->v64.x, cg->v64.b, cg->v64.w);
    ITHACA_CUDA(cudaMemcpyAsync(hs, cg->dscal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaStreamSynchronize(s));
    out.rel_residual = hs[1] > 0 ? std::sqrt(hs[0] / hs[1]) : 0.0;
  }
  if (res) *res = out;
  c->check_device_error();
  if (status == ITHACA_GPU_ERR_NOT_CONVERGED)
    fail(status, "Exceeded maximum number of iterations (" + std::to_string(out.iterations) + ")");
  if (status != ITHACA_GPU_OK) fail(status, "NaN or Inf in the CG recurrence");
}

// ---- successive right-hand sides (GlobalLinSysIterative.cpp:156-482) ----------------
constexpr double kZeroTol = 1.0e-12;          // NekConstants::kNekZeroTol
constexpr double kSparseNonZeroTol = 1e-16;   // NekConstants::kNekSparseNonZeroTol

// Solves M x = y (n x n, row-major, symmetric) by LDL^T without pivoting, in place in y.
// The reference factorises with Bunch-Kaufman (Lapack Dsptrf); the matrix here is SPD
// with a unit diagonal unless the stored solutions are dependent, and a non-positive
// pivot is treated as the reference treats a failed factorisation.
static bool ldlt_solve(const std::vector<double>& M, int n, std::vector<double>& y) {
  std::vector<double> L((size_t)n * n, 0.0), d(n, 0.0);
  for (int j = 0; j < n; ++j) {
    double dj = M[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) dj -= L[(size_t)j * n + k] * L[(size_t)j * n + k] * d[k];
    if (!(dj > 0.0)) return false;
    d[j] = dj;
    L[(size_t)j * n + j] = 1.0;
    for (int i = j + 1; i < n; ++i) {
      double v = M[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k] * d[k];
      L[(size_t)i * n + j] = v / dj;
    }
  }
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < i; ++k) y[i] -= L[(size_t)i * n + k] * y[k];
  for (int i = 0; i < n; ++i) y[i] /= d[i];
  for (int i = n - 1; i >= 0; --i)
    for (int k = i + 1; k < n; ++k) y[i] -= L[(size_t)k * n + i] * y[k];
  return true;
}

static void proj_alloc(Cg* cg) {
  SuccessiveRhs& P = cg->proj;
  if (P.sols) return;
  const size_t nf = (size_t)(cg->N - cg->ndir), N = cg->N;
  P.nparts = std::max(1, std::min(device_sm_count() * 2, (int)((nf + RT - 1) / RT)));
  ITHACA_CUDA(cudaMalloc(&P.sols, sizeof(double) * P.m * std::max<size_t>(nf, 1)));
  if (!P.aconj) ITHACA_CUDA(cudaMalloc(&P.basis, sizeof(double) * P.m * std::max<size_t>(nf, 1)));
  ITHACA_CUDA(cudaMalloc(&P.px, sizeof(double) * N));
  ITHACA_CUDA(cudaMalloc(&P.ax, sizeof(double) * N));
  ITHACA_CUDA(cudaMalloc(&P.bsave, sizeof(double) * N));
  ITHACA_CUDA(cudaMalloc(&P.part, sizeof(double) * P.nparts * P.m));
  ITHACA_CUDA(cudaMalloc(&P.dots, sizeof(double) * P.m));
  ITHACA_CUDA(cudaMemset(P.px, 0, sizeof(double) * N));
}

// Stored vector i of the reference's m_prevBasis (the solutions themselves when A-conjugate).
static double* proj_basis(Cg* cg) { return cg->proj.aconj ? cg->proj.sols : cg->proj.basis; }

// <V_i, y> over the free dofs for the nv stored vectors V (host result).
static std::vector<double> proj_dots(Cg* cg, const double* V, int nv, const double* yfree) {
  SuccessiveRhs& P = cg->proj;
  std::vector<double> out(nv, 0.0);
  if (nv == 0) return out;
  cudaStream_t s = cg->op->ctx->stream;
  const int nf = cg->N - cg->ndir;
  multidot_part_kernel<<<dim3(P.nparts, nv), RT, 0, s>>>(nf, V, (size_t)nf, yfree, P.part);
  multidot_final_kernel<<<nv, RT, 0, s>>>(P.part, P.nparts, P.dots);
  cg->op->ctx->launches += 2;
  ITHACA_CUDA(cudaMemcpyAsync(out.data(), P.dots, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
  ITHACA_CUDA(cudaStreamSynchronize(s));
  return out;
}

// ResetKnownSolutionsToLatestOne (:272-289): keep only the latest stored vector (moved to
// column 0, with its unit diagonal entry).
static int proj_reset_to_latest(Cg* cg) {
  SuccessiveRhs& P = cg->proj;
  if (P.nprev == 0) return -1;
  const int latest = (P.nprev - 1 + P.m) % P.m;
  const size_t nf = (size_t)(cg->N - cg->ndir);
  cudaStream_t s = cg->op->ctx->stream;
  if (latest != 0) {
    ITHACA_CUDA(cudaMemcpyAsync(P.sols, P.sols + latest * nf, sizeof(double) * nf, cudaMemcpyDeviceToDevice, s));
    if (!P.aconj)
      ITHACA_CUDA(cudaMemcpyAsync(P.basis, P.basis + latest * nf, sizeof(double) * nf, cudaMemcpyDeviceToDevice, s));
  }
  P.nstored = 1;
  P.M.assign(1, 1.0);
  P.nprev = 1;
  return latest;
}

// A x over the free dofs into P.ax (x gathered with its Dirichlet part read as zero).
static void proj_apply(Cg* cg, double lambda, const double* x) {
  cudaStream_t s = cg->op->ctx->stream;
  launch_apply<double>(cg, cg->v64, cg->op->t64.base, geo64(cg), lambda, nullptr, x, s, true, nullptr);
  assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols,
                                                  cg->v64.yloc, cg->proj.ax, nullptr, nullptr, nullptr);
  cg->op->ctx->launches++;
}

// UpdateKnownSolutions (:295-482) with the solution in cg->v64.x.
static void proj_update(Cg* cg, double lambda) {
  SuccessiveRhs& P = cg->proj;
  const int m = P.m, nf = cg->N - cg->ndir, nd = cg->ndir;
  cudaStream_t s = cg->op->ctx->stream;
  const int grid = std::max(1, std::min(RB, (nf + RT - 1) / RT));
  int insert = P.nprev % m;
  bool full = P.nstored == m;
  proj_apply(cg, lambda, cg->v64.x);
  double* axf = P.ax + nd;
  const double* xf = cg->v64.x + nd;
  const double sol_norm = proj_dots(cg, P.aconj ? xf : axf, 1, axf)[0];
  if (sol_norm < 22.2 * kSparseNonZeroTol) return;
  const double inv = 1.0 / std::sqrt(sol_norm);
  scale_copy_kernel<<<grid, RT, 0, s>>>(nf, inv, axf, axf, 0);
  cg->op->ctx->launches++;
  const std::vector<double> all = proj_dots(cg, proj_basis(cg), P.nstored, axf);
  std::vector<double> y;
  for (int i = 0; i < P.nstored; ++i)
    if (i != insert) y.push_back(all[i]);
  // the coefficient matrix without the vector about to be replaced
  int nt = 0;
  std::vector<double> tilM;
  if (full && m > 1) {
    nt = m - 1;
    tilM.resize((size_t)nt * nt);
    for (int i = 0, a = 0; i < m; ++i) {
      if (i == insert) continue;
      for (int j = 0, b = 0; j < m; ++j) {
        if (j == insert) continue;
        tilM[(size_t)a * nt + b++] = P.M[(size_t)i * m + j];
      }
      ++a;
    }
  } else if (!full && P.nstored > 0) {
    nt = P.nstored;
    tilM = P.M;
  }
  std::vector<double> invy = y;
  bool ok = true;
  if (!y.empty()) ok = ldlt_solve(tilM, nt, invy);
  if (!ok) {
    const int latest = proj_reset_to_latest(cg);
    y.assign(1, y[latest - (latest > insert)]);
    invy = y;
    insert = P.nprev % m;
    full = P.nstored == m;
  }
  double residual = 1.0;
  for (int i = 0; i < P.nstored - (full ? 1 : 0); ++i) residual -= y[i] * invy[i];
  if (residual < 10.0 * kZeroTol) return;
  // new coefficient matrix
  const int nn = full ? m : P.nstored + 1;
  std::vector<double> newM((size_t)nn * nn, 0.0);
  const int no = P.nstored;
  for (int i = 0; i < no; ++i)
    for (int j = 0; j < no; ++j) newM[(size_t)i * nn + j] = P.M[(size_t)i * no + j];
  newM[(size_t)insert * nn + insert] = 1.0;
  for (int i = 0; i < nn; ++i) {
    if (i == insert) continue;
    const double v = y[i - (i > insert)];
    newM[(size_t)insert * nn + i] = newM[(size_t)i * nn + insert] = v;
  }
  std::vector<double> probe(nn, 1.0);
  if (!ldlt_solve(newM, nn, probe)) return;
  // accept: store x / sqrt(solNorm) (and A x / sqrt(solNorm) for the non-conjugate basis)
  scale_copy_kernel<<<grid, RT, 0, s>>>(nf, inv, xf, P.sols + (size_t)insert * nf, 0);
  if (!P.aconj) ITHACA_CUDA(cudaMemcpyAsync(P.basis + (size_t)insert * nf, axf, sizeof(double) * nf,
                                            cudaMemcpyDeviceToDevice, s));
  cg->op->ctx->launches++;
  if (P.nstored < m) P.nstored++;
  P.M = newM;
  P.nprev++;
}

// DoProjection (:156-266) around solve_impl: rhs in cg->v64.b, solution into cg->v64.x.
static void solve_projected(Cg* cg, double lambda, const ithaca_gpu_cg_opts& o, ithaca_gpu_cg_result* res) {
  SuccessiveRhs& P = cg->proj;
  if (P.m == 0) {
    solve_impl(cg, lambda, o, res);
    return;
  }
  if (!(P.lambda == lambda)) {  // another operator: the stored solutions do not apply
    P.nprev = P.nstored = 0;
    P.M.clear();
    P.lambda = lambda;
  }
  proj_alloc(cg);
  const int nf = cg->N - cg->ndir, nd = cg->ndir;
  cudaStream_t s = cg->op->ctx->stream;
  const int grid = std::max(1, std::min(RB, (nf + RT - 1) / RT));
  ithaca_gpu_cg_result r{};
  if (P.nprev == 0) {
    solve_impl(cg, lambda, o, &r);
  } else {
    ITHACA_CUDA(cudaMemcpyAsync(P.bsave, cg->v64.b, sizeof(double) * cg->N, cudaMemcpyDeviceToDevice, s));
    std::vector<double> alpha = proj_dots(cg, proj_basis(cg), P.nstored, P.bsave + nd);
    const std::vector<double> alphaback = alpha;
    if (!ldlt_solve(P.M, P.nstored, alpha)) {
      const int latest = proj_reset_to_latest(cg);
      alpha.assign(1, alphaback[latest]);
    }
    ProjCoef coef{};
    for (int i = 0; i < P.nstored; ++i) coef.c[i] = alpha[i];
    combine_kernel<<<grid, RT, 0, s>>>(nf, P.nstored, P.sols, (size_t)nf, coef, P.px + nd);
    cg->op->ctx->launches++;
    // pb = b - A px on the free dofs, zero on the Dirichlet ones
    if (nd > 0) ITHACA_CUDA(cudaMemsetAsync(cg->v64.b, 0, sizeof(double) * nd, s));
    fp64_residual(cg, lambda, P.px, P.bsave, cg->v64.b);
    solve_impl(cg, lambda, o, &r);
    // x = tmpx + px; the reported residual is that of x against the given rhs
    scale_copy_kernel<<<grid, RT, 0, s>>>(nf, 1.0, P.px + nd, cg->v64.x + nd, 1);
    ITHACA_CUDA(cudaMemcpyAsync(cg->v64.b, P.bsave, sizeof(double) * cg->N, cudaMemcpyDeviceToDevice, s));
    cg->op->ctx->launches++;
    double hs[2];
    fp64_residual(cg, lambda, cg->v64.x, cg->v64.b, cg->v64.w);
    ITHACA_CUDA(cudaMemcpyAsync(hs, cg->dscal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaStreamSynchronize(s));
    r.rel_residual = hs[1] > 0 ? std::sqrt(hs[0] / hs[1]) : 0.0;
  }
  if (r.iterations > 0) proj_update(cg, lambda);
  if (res) *res = r;
}

}  // namespace ithaca

using namespace ithaca;

struct ithaca_gpu_cg : public Cg {};

template <typename F>
static int cg_guarded(F f) {
  try {
    f();
    return ITHACA_GPU_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return ITHACA_GPU_ERR_NOMEM;
  }
}

static void req(bool ok, const char* msg) {
  if (!ok) fail(ITHACA_GPU_ERR_ARG, msg);
}

static ithaca_gpu_cg_opts opts_or_default(const ithaca_gpu_cg_opts* o);

extern "C" {

void ithaca_gpu_cg_default_opts(ithaca_gpu_cg_opts* o) {
  if (!o) return;
  o->tol = 1e-9;
  o->max_iter = 5000;
  o->mode = ITHACA_GPU_SOLVE_FP64;
  o->inner_tol = 1e-2;
  o->max_outer = 50;
  o->check_every = 16;
}

int ithaca_gpu_cg_create(ithaca_gpu_op* opp, const int* l2g, const double* sign, int nglobal, int ndir,
                         ithaca_gpu_cg** out) {
  return cg_guarded([&] {
    Op* op = reinterpret_cast<Op*>(opp);
    req(op && l2g && sign && out, "null argument");
    req(op->precision == ITHACA_GPU_FP64, "the global system needs an FP64 operator");
    req(nglobal > 0 && ndir >= 0 && ndir <= nglobal, "bad nglobal / ndir");
    const size_t nloc = (size_t)op->E * op->nm;
    req(nloc < (size_t)0x7fffffff, "too many local dofs for 32-bit indices");
    std::vector<int> code(nloc), cnt(nglobal + 1, 0);
    for (size_t l = 0; l < nloc; ++l) {
      const int g = l2g[l];
      if (g < 0 || g >= nglobal) fail(ITHACA_GPU_ERR_ARG, "l2g entry out of range");
      if (!(sign[l] == 1.0 || sign[l] == -1.0)) fail(ITHACA_GPU_ERR_ARG, "sign entries must be +1 or -1");
      code[l] = sign[l] > 0 ? g : ~g;
      cnt[g + 1]++;
    }
    for (int g = 0; g < nglobal; ++g) cnt[g + 1] += cnt[g];
    std::vector<int> cols(nloc), fill(cnt.begin(), cnt.end() - 1);
    for (size_t l = 0; l < nloc; ++l) {
      const int g = l2g[l];
      cols[fill[g]++] = sign[l] > 0 ? (int)l : ~(int)l;
    }
    // assembly plan: rows by number of entries (class c < kAsmK: c + 1 entries, ELL)
    AsmPlan plan{};
    std::vector<int> cls_of(nglobal);
    long long entries[kAsmK + 1] = {};
    for (int g = 0; g < nglobal; ++g) {
      const int k = cnt[g + 1] - cnt[g];
      if (k == 0) fail(ITHACA_GPU_ERR_ARG, "global dof " + std::to_string(g) + " has no local dof");
      const int c = k <= kAsmK ? k - 1 : kAsmK;
      cls_of[g] = c;
      plan.n[c]++;
      if (g < ndir) plan.ndir[c]++;
      entries[c] += k;
    }
    long long col_total = 0;
    for (int c = 0, off = 0; c <= kAsmK; ++c) {
      plan.rows_off[c] = off;
      off += plan.n[c];
      if (c < kAsmK) {
        plan.col_off[c] = col_total;
        col_total += entries[c];
      }
    }
    plan.tail_off = col_total;
    // Output codes of the scattered inner apply (see OwnedRows): owned rows (free, one
    // local entry) -> g | kOwnedBit; other free rows -> the entry's slot in the
    // assembly-ordered buffer (the ELL position of asm_cols, or tail_off + tail_ptr[i] + j);
    // Dirichlet rows -> -1. The slots number the local entries once, so they fit in nloc.
    const bool own_ok = nglobal < kOwnedBit && nloc < (size_t)kOwnedBit;
    std::vector<int> ocode(own_ok ? nloc : 0, -1), tail_ptr(plan.n[kAsmK] + 1, 0);
    std::vector<int> asm_rows(nglobal), asm_cols((size_t)std::max<long long>(col_total, 1));
    {
      int fillc[kAsmK + 1];
      for (int c = 0; c <= kAsmK; ++c) fillc[c] = 0;
      for (int g = 0; g < nglobal; ++g) {
        const int c = cls_of[g], i = fillc[c]++;
        asm_rows[(size_t)plan.rows_off[c] + i] = g;
        const int k = cnt[g + 1] - cnt[g];
        if (c == kAsmK) tail_ptr[i + 1] = tail_ptr[i] + k;
        for (int j = 0; j < k; ++j) {
          const long long pos = c < kAsmK ? plan.col_off[c] + (long long)j * plan.n[c] + i
                                          : plan.tail_off + tail_ptr[i] + j;
          if (c < kAsmK) asm_cols[(size_t)pos] = cols[cnt[g] + j];
          if (own_ok && g >= ndir) {
            const int cl = cols[cnt[g] + j], l = cl >= 0 ? cl : ~cl;
            ocode[(size_t)l] = k == 1 ? (g | kOwnedBit) : (int)pos;
          }
        }
      }
    }
    // Grid sizes: the full grids for large systems, about 2 rows per thread for small
    // ones (enough threads to keep a small system's loads in parallel, without the
    // partial sums of CTAs that have no rows).
    int nonempty_all = 0;
    for (int c = 0; c <= kAsmK; ++c) nonempty_all += plan.n[c] > 0;
    int dev = 0, sms = 0;
    ITHACA_CUDA(cudaGetDevice(&dev));
    ITHACA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long per2 = ((long long)nglobal + 2 * RT - 1) / (2 * RT);
    const int rb_full = std::min(RB, kRedPerSM * sms), rba_full = std::min(RBA, kAsmPerSM * sms);
    const int rbv = (int)std::min<long long>(rb_full, std::max<long long>(1, per2));
    const int rba = (int)std::min<long long>(std::max(rba_full, nonempty_all), std::max<long long>(nonempty_all, per2));
    // CTAs per class in proportion to its entries, at least one for a non-empty class
    auto split_ctas = [&](AsmPlan& P, const long long* ent) {
      long long total = 0;
      int nonempty = 0;
      for (int c = 0; c <= kAsmK; ++c) {
        total += ent[c];
        nonempty += P.n[c] > 0;
      }
      int share[kAsmK + 1], used = 0, big = 0;
      for (int c = 0; c <= kAsmK; ++c) {
        share[c] = P.n[c] > 0 ? std::max(1, (int)((double)(rba - nonempty) * ent[c] / std::max(total, 1LL))) : 0;
        used += share[c];
        if (ent[c] > ent[big]) big = c;
      }
      share[big] += rba - used;  // the rounding remainder goes to the largest class
      P.cta0[0] = 0;
      for (int c = 0; c <= kAsmK; ++c) P.cta0[c + 1] = P.cta0[c] + share[c];
    };
    split_ctas(plan, entries);
    // Owned rows: the free rows with a single local entry. The inner FP32 iteration's
    // element kernel writes them, so its plan keeps only class 0's Dirichlet rows (which
    // lead the class and are skipped) and gives class 0's CTAs to the other classes.
    AsmPlan plan_own = plan;
    if (own_ok) {
      plan_own.n[0] = plan.ndir[0];
      long long ent_own[kAsmK + 1];
      for (int c = 0; c <= kAsmK; ++c) ent_own[c] = entries[c];
      ent_own[0] = plan.ndir[0];
      split_ctas(plan_own, ent_own);
    }
    // The fused inner iteration (asm_update_f32_kernel): every class, over a vector-kernel
    // grid (rbv CTAs: its r.w / r.r partials fill at most RB slots), the CTAs split by the
    // update's work per class: 11 vector accesses per free row plus the row's s or slot
    // reads. Needs a CTA for every class that has free rows.
    AsmPlan plan_upd = plan;
    bool upd_ok = false;
    if (own_ok) {
      long long wgt[kAsmK + 1], total = 0;
      int nonempty = 0, big = 0;
      for (int c = 0; c <= kAsmK; ++c) {
        const long long nfree = plan.n[c] - plan.ndir[c];
        const long long efree = c < kAsmK ? (long long)(c + 1) * nfree : (nfree > 0 ? entries[c] * nfree / plan.n[c] : 0);
        wgt[c] = nfree > 0 ? 11 * nfree + efree : 0;
        total += wgt[c];
        nonempty += nfree > 0;
        if (wgt[c] > wgt[big]) big = c;
      }
      if (nonempty > 0 && rbv >= nonempty) {
        int share[kAsmK + 1], used = 0;
        for (int c = 0; c <= kAsmK; ++c) {
          share[c] = wgt[c] > 0 ? std::max(1, (int)((double)(rbv - nonempty) * wgt[c] / std::max(total, 1LL))) : 0;
          used += share[c];
        }
        share[big] += rbv - used;
        plan_upd.cta0[0] = 0;
        for (int c = 0; c <= kAsmK; ++c) plan_upd.cta0[c + 1] = plan_upd.cta0[c] + share[c];
        upd_ok = plan_upd.cta0[kAsmK + 1] == rbv;
      }
    }
    auto cg = std::make_unique<ithaca_gpu_cg>();
    cg->op = op;
    cg->N = nglobal;
    cg->ndir = ndir;
    cg->rbv = rbv;
    cg->rba = rba;
    cg->nloc = nloc;
    cudaStream_t s = op->ctx->stream;
    ITHACA_CUDA(cudaMalloc(&cg->l2g, sizeof(int) * nloc));
    ITHACA_CUDA(cudaMalloc(&cg->rowptr, sizeof(int) * (nglobal + 1)));
    ITHACA_CUDA(cudaMalloc(&cg->cols, sizeof(int) * nloc));
    ITHACA_CUDA(cudaMalloc(&cg->asm_rows, sizeof(int) * nglobal));
    if (own_ok) {
      cg->opart_cap = sms * 32;  // at most 32 resident CTAs per SM
      cg->sms = sms;
      ITHACA_CUDA(cudaMalloc(&cg->bar, 2 * sizeof(unsigned)));
      ITHACA_CUDA(cudaMalloc(&cg->ocode, sizeof(int) * nloc));
      ITHACA_CUDA(cudaMalloc(&cg->tail_ptr, sizeof(int) * tail_ptr.size()));
      ITHACA_CUDA(cudaMalloc(&cg->opart, sizeof(double) * cg->opart_cap));
      ITHACA_CUDA(cudaMemcpyAsync(cg->ocode, ocode.data(), sizeof(int) * nloc, cudaMemcpyHostToDevice, s));
      ITHACA_CUDA(cudaMemcpyAsync(cg->tail_ptr, tail_ptr.data(), sizeof(int) * tail_ptr.size(),
                                  cudaMemcpyHostToDevice, s));
      cg->own_ok = true;
      cg->plan_own = plan_own;
      cg->plan_upd = plan_upd;
      cg->upd_ok = upd_ok;
    }
    ITHACA_CUDA(cudaMalloc(&cg->asm_cols, sizeof(int) * asm_cols.size()));
    ITHACA_CUDA(cudaMemcpyAsync(cg->l2g, code.data(), sizeof(int) * nloc, cudaMemcpyHostToDevice, s));
    ITHACA_CUDA(cudaMemcpyAsync(cg->rowptr, cnt.data(), sizeof(int) * (nglobal + 1), cudaMemcpyHostToDevice, s));
    ITHACA_CUDA(cudaMemcpyAsync(cg->cols, cols.data(), sizeof(int) * nloc, cudaMemcpyHostToDevice, s));
    ITHACA_CUDA(cudaMemcpyAsync(cg->asm_rows, asm_rows.data(), sizeof(int) * nglobal, cudaMemcpyHostToDevice, s));
    ITHACA_CUDA(
        cudaMemcpyAsync(cg->asm_cols, asm_cols.data(), sizeof(int) * asm_cols.size(), cudaMemcpyHostToDevice, s));
    cg->plan = plan;
    cg->v64.alloc(nglobal, nloc);
    ITHACA_CUDA(cudaMalloc(&cg->partials, sizeof(double) * ((NSLOT - 1) * RB + RBA)));
    ITHACA_CUDA(cudaMalloc(&cg->dscal, sizeof(double) * 8));
    ITHACA_CUDA(cudaMalloc(&cg->counter, sizeof(unsigned int)));
    ITHACA_CUDA(cudaMemset(cg->counter, 0, sizeof(unsigned int)));
    ITHACA_CUDA(cudaMalloc(&cg->sc, sizeof(CgScalars)));
    ITHACA_CUDA(cudaMallocHost(&cg->sc_host, sizeof(CgScalars)));
    *cg->sc_host = CgScalars{};
    ITHACA_CUDA(cudaStreamSynchronize(s));
    retain_op(op);  // the solver holds its operator (and through it the context)
    *out = cg.release();
  });
}

int ithaca_gpu_cg_set_persistent(ithaca_gpu_cg* cg, int mode) {
  return cg_guarded([&] {
    req(cg != nullptr, "null solver");
    req(mode >= -1 && mode <= 1, "persistent mode must be -1, 0 or 1");
    cg->persist = mode;
  });
}

int ithaca_gpu_cg_set_fused_update(ithaca_gpu_cg* cg, int on) {
  return cg_guarded([&] {
    req(cg != nullptr, "null solver");
    req(on == 0 || on == 1, "on must be 0 or 1");
    cg->fuse_tail = on != 0;
  });
}

int ithaca_gpu_cg_set_successive_rhs(ithaca_gpu_cg* cg, int nsuccessive) {
  return cg_guarded([&] {
    req(cg != nullptr, "null solver");
    req(std::abs(nsuccessive) <= kMaxSuccessive, "at most 64 stored solutions");
    cudaStreamSynchronize(cg->op->ctx->stream);
    cg->proj.release();
    cg->proj = SuccessiveRhs{};
    cg->proj.m = std::abs(nsuccessive);
    cg->proj.aconj = nsuccessive > 0;
  });
}

int ithaca_gpu_cg_set_wait_test(ithaca_gpu_cg* cg, long long barrier_polls, int drop_cta, int delay_ns) {
  return cg_guarded([&] {
    req(cg != nullptr, "null solver");
    req(barrier_polls >= 0 && barrier_polls <= (1LL << 24), "barrier_polls must be in [0, 2^24]");
    req(drop_cta >= -1, "drop_cta must be -1 or a CTA index");
    req(delay_ns >= 0 && delay_ns <= 1000000, "delay_ns must be in [0, 1e6]");
    cg->dbg_polls = barrier_polls;
    cg->dbg_drop = drop_cta;
    cg->dbg_delay = delay_ns;
  });
}

int ithaca_gpu_cg_destroy(ithaca_gpu_cg* cg) {
  return cg_guarded([&] {
    if (!cg) return;
    cudaStreamSynchronize(cg->op->ctx->stream);
    Op* op = cg->op;
    delete cg;
    release_op(op);  // the solver held its operator
  });
}

int ithaca_gpu_cg_apply(ithaca_gpu_cg* cg, double lambda, const double* x, double* y, int on_device) {
  return cg_guarded([&] {
    req(cg && x && y, "null argument");
    StreamOrder order_(cg->op->ctx);
    Ctx* c = cg->op->ctx;
    cudaStream_t s = c->stream;
    const size_t bytes = sizeof(double) * cg->N;
    const double* dx = x;
    if (!on_device) {
      ITHACA_CUDA(cudaMemcpyAsync(cg->v64.p, x, bytes, cudaMemcpyHostToDevice, s));
      dx = cg->v64.p;
    }
    double* dy = on_device ? y : cg->v64.q;
    launch_apply<double>(cg, cg->v64, cg->op->t64.base, geo64(cg), lambda, nullptr, dx, s, false, nullptr);
    assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, cg->v64.yloc, dy, nullptr,
                                                  nullptr, nullptr);
    c->launches++;
    if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    if (!on_device) ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_cg_assemble(ithaca_gpu_cg* cg, const double* local, double* global, int on_device) {
  return cg_guarded([&] {
    req(cg && local && global, "null argument");
    StreamOrder order_(cg->op->ctx);
    Ctx* c = cg->op->ctx;
    cudaStream_t s = c->stream;
    const double* dl = local;
    if (!on_device) {
      double* d = (double*)c->stage_ptr(0, sizeof(double) * cg->nloc);
      ITHACA_CUDA(cudaMemcpyAsync(d, local, sizeof(double) * cg->nloc, cudaMemcpyHostToDevice, s));
      dl = d;
    }
    double* dg = on_device ? global : (double*)c->stage_ptr(1, sizeof(double) * cg->N);
    assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, dl, dg, nullptr, nullptr, nullptr);
    c->launches++;
    if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(global, dg, sizeof(double) * cg->N, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    if (!on_device) ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_cg_global_to_local(ithaca_gpu_cg* cg, const double* global, double* local, int on_device) {
  return cg_guarded([&] {
    req(cg && local && global, "null argument");
    StreamOrder order_(cg->op->ctx);
    Ctx* c = cg->op->ctx;
    cudaStream_t s = c->stream;
    const double* dg = global;
    if (!on_device) {
      double* d = (double*)c->stage_ptr(0, sizeof(double) * cg->N);
      ITHACA_CUDA(cudaMemcpyAsync(d, global, sizeof(double) * cg->N, cudaMemcpyHostToDevice, s));
      dg = d;
    }
    double* dl = on_device ? local : (double*)c->stage_ptr(1, sizeof(double) * cg->nloc);
    g2l_kernel<<<RB, RT, 0, s>>>(cg->nloc, cg->l2g, dg, dl);
    c->launches++;
    if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(local, dl, sizeof(double) * cg->nloc, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    if (!on_device) ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_cg_diagonal(ithaca_gpu_cg* cg, double lambda, double* diag, int on_device) {
  return cg_guarded([&] {
    req(cg && diag, "null argument");
    StreamOrder order_(cg->op->ctx);
    cudaStream_t s = cg->op->ctx->stream;
    cg->diag_lambda = NAN;
    ensure_diag(cg, lambda);
    const size_t bytes = sizeof(double) * (cg->N - cg->ndir);
    ITHACA_CUDA(cudaMemcpyAsync(diag, cg->v64.s + cg->ndir, bytes,
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    if (!on_device) ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_cg_solve(ithaca_gpu_cg* cg, double lambda, const double* rhs, double* x,
                        const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device) {
  return cg_guarded([&] {
    req(cg && rhs && x, "null argument");
    StreamOrder order_(cg->op->ctx);
    const ithaca_gpu_cg_opts o = opts_or_default(opts);
    Ctx* c = cg->op->ctx;
    cudaStream_t s = c->stream;
    const size_t bytes = sizeof(double) * cg->N;
    ITHACA_CUDA(cudaMemcpyAsync(cg->v64.b, rhs, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                s));
    struct Copyback {
      Cg* cg;
      double* x;
      int on_device;
      size_t off, bytes;
      ~Copyback() {
        // the solution (non-Dirichlet part) goes back even when the solve failed to converge
        cudaMemcpyAsync(x + off, cg->v64.x + off, bytes,
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, cg->op->ctx->stream);
        cudaStreamSynchronize(cg->op->ctx->stream);
      }
    } cb{cg, x, on_device, (size_t)cg->ndir, sizeof(double) * (cg->N - cg->ndir)};
    solve_projected(cg, lambda, o, res);
  });
}

int ithaca_gpu_helmsolve(ithaca_gpu_cg* cg, double lambda, const double* forcing, double* out_local,
                         const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device) {
  return ithaca_gpu_helmsolve_dirichlet(cg, lambda, forcing, nullptr, out_local, opts, res, on_device);
}

int ithaca_gpu_helmsolve_dirichlet(ithaca_gpu_cg* cg, double lambda, const double* forcing, const double* dirichlet,
                                   double* out_local, const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res,
                                   int on_device) {
  return cg_guarded([&] {
    req(cg && forcing && out_local, "null argument");
    StreamOrder order_(cg->op->ctx);
    const ithaca_gpu_cg_opts o = opts_or_default(opts);
    Op* op = cg->op;
    Ctx* c = op->ctx;
    cudaStream_t s = c->stream;
    const size_t nphys = (size_t)op->E * op->nq, nloc = cg->nloc;
    const double* f = forcing;
    if (!on_device) {
      double* d = (double*)c->stage_ptr(0, sizeof(double) * nphys);
      ITHACA_CUDA(cudaMemcpyAsync(d, forcing, sizeof(double) * nphys, cudaMemcpyHostToDevice, s));
      f = d;
    }
    // wsp = -IProductWRTBase(f) (ContField.cpp:895-900); b = Assemble(wsp)
    if (!launch_iproduct<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64, f,
                                 cg->v64.yloc, s))
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "IProductWRTBase: (modes, points) combination not built");
    neg_kernel<<<RB, RT, 0, s>>>(nloc, cg->v64.yloc);
    assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, cg->v64.yloc, cg->v64.b, nullptr,
                                                  nullptr, nullptr);
    c->launches += 3;
    const double* dvals = nullptr;  // Dirichlet values on the device (ndir entries)
    if (dirichlet != nullptr && cg->ndir > 0) {
      // lift (ContField.cpp:908-930): x_D = the given boundary values, b_F -= (A x_D)_F
      double* xd = cg->v64.p;  // scratch until the solve
      ITHACA_CUDA(cudaMemsetAsync(xd, 0, sizeof(double) * cg->N, s));
      ITHACA_CUDA(cudaMemcpyAsync(xd, dirichlet, sizeof(double) * cg->ndir,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
      launch_apply<double>(cg, cg->v64, op->t64.base, geo64(cg), lambda, nullptr, xd, s, false, nullptr);
      assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr,
                                                    cg->cols, cg->v64.yloc, cg->v64.s, nullptr, nullptr, nullptr);
      // every row, the Dirichlet ones included: the reference assembles the lifted local
      // rhs (GlobalLinSysIterativeFull.cpp:182-186) and its CG takes ||b||^2 over the whole
      // assembled vector (NekLinSysIter.cpp:128-142); the solve reads only the free rows
      sub_rows_kernel<<<RB, RT, 0, s>>>(cg->N, 0, cg->v64.s, cg->v64.b);
      c->launches += 2;
      double* keep = (double*)c->stage_ptr(2, sizeof(double) * cg->ndir);  // the solve reuses v64.p
      ITHACA_CUDA(cudaMemcpyAsync(keep, xd, sizeof(double) * cg->ndir, cudaMemcpyDeviceToDevice, s));
      dvals = keep;
    }
    solve_projected(cg, lambda, o, res);
    // Dirichlet values (zero, or the given ones), then GlobalToLocal
    if (dvals != nullptr)
      ITHACA_CUDA(cudaMemcpyAsync(cg->v64.x, dvals, sizeof(double) * cg->ndir, cudaMemcpyDeviceToDevice, s));
    else
      ITHACA_CUDA(cudaMemsetAsync(cg->v64.x, 0, sizeof(double) * cg->ndir, s));
    double* dout = on_device ? out_local : (double*)c->stage_ptr(1, sizeof(double) * nloc);
    g2l_kernel<<<RB, RT, 0, s>>>(nloc, cg->l2g, cg->v64.x, dout);
    c->launches++;
    if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(out_local, dout, sizeof(double) * nloc, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

// VelocityCorrectionScheme_ROM::v_SolveViscous: per field, lambda = 1 / aii_dt / diff_coeff,
// HelmSolve into the field's coefficients, BwdTrans into its physical values.
int ithaca_gpu_vcs_solve_viscous(ithaca_gpu_cg* cg, int nfields, const double* const* forcing,
                                 const double* const* dirichlet, double aii_dt, const double* diff_coeff,
                                 double* const* coeffs, double* const* phys, const ithaca_gpu_cg_opts* opts,
                                 ithaca_gpu_cg_result* res, int on_device) {
  return cg_guarded([&] {
    req(cg && forcing && coeffs && diff_coeff, "null argument");
    req(nfields > 0, "nfields must be positive");
    req(aii_dt > 0 && std::isfinite(aii_dt), "aii_dt must be positive and finite");
    for (int i = 0; i < nfields; ++i) {
      req(forcing[i] != nullptr && coeffs[i] != nullptr, "null field pointer");
      req(diff_coeff[i] > 0 && std::isfinite(diff_coeff[i]), "diffusion coefficients must be positive and finite");
    }
    for (int i = 0; i < nfields; ++i) {
      const double lambda = 1.0 / aii_dt / diff_coeff[i];
      int rc = ithaca_gpu_helmsolve_dirichlet(cg, lambda, forcing[i], dirichlet ? dirichlet[i] : nullptr, coeffs[i],
                                              opts, res ? res + i : nullptr, on_device);
      if (rc != ITHACA_GPU_OK) fail(rc, "field " + std::to_string(i) + ": " + last_error_text());
      if (phys != nullptr && phys[i] != nullptr) {
        rc = ithaca_gpu_bwdtrans(reinterpret_cast<ithaca_gpu_op*>(cg->op), coeffs[i], phys[i], on_device);
        if (rc != ITHACA_GPU_OK) fail(rc, "field " + std::to_string(i) + ": " + last_error_text());
      }
    }
  });
}

// VelocityCorrectionScheme_ROM::v_SolvePressure: the pressure Poisson equation, HelmSolve
// with lambda = 0.
int ithaca_gpu_vcs_solve_pressure(ithaca_gpu_cg* cg, const double* forcing, const double* dirichlet,
                                  double* coeffs, const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res,
                                  int on_device) {
  return cg_guarded([&] {
    req(cg && forcing && coeffs, "null argument");
    req(cg->ndir > 0, "the pressure system needs Dirichlet dofs (a pure-Neumann Poisson system is singular)");
    const int rc = ithaca_gpu_helmsolve_dirichlet(cg, 0.0, forcing, dirichlet, coeffs, opts, res, on_device);
    if (rc != ITHACA_GPU_OK) fail(rc, last_error_text());
  });
}

int ithaca_gpu_cg_profile_apply(ithaca_gpu_cg* cg, int mode, double lambda, int reps, double* avg_ms,
                                double* bytes_per_launch) {
  return cg_guarded([&] {
    req(cg && avg_ms && reps > 0, "bad argument");
    StreamOrder order_(cg->op->ctx);
    Op* op = cg->op;
    cudaStream_t s = op->ctx->stream;
    const bool half = mode == ITHACA_GPU_SOLVE_MIXED_FP32_GEO16;
    const bool f32 = mode == ITHACA_GPU_SOLVE_MIXED_FP32 || half;
    if (f32) ensure_fp32(cg);
    if (half) ensure_geo16(cg);
    cg->geo16 = half;
    struct Geo16Reset {
      Cg* c;
      ~Geo16Reset() { c->geo16 = false; }
    } geo16_reset{cg};
    cudaEvent_t e0, e1;
    ITHACA_CUDA(cudaEventCreate(&e0));
    ITHACA_CUDA(cudaEventCreate(&e1));
    // the FP32 apply exactly as the inner iteration launches it (owned rows included)
    OwnedRows own;
    own.s = cg->v32.s;
    own.part = cg->opart;
    auto run = [&] {
      if (f32)
        launch_apply<float>(cg, cg->v32, op->t32.base, cg->jg32, (float)lambda, nullptr, cg->v32.w, s, true, nullptr,
                            cg->own_ok ? &own : nullptr);
      else
        launch_apply<double>(cg, cg->v64, op->t64.base, geo64(cg), lambda, nullptr, cg->v64.w, s, true, nullptr);
    };
    run();  // warm-up
    ITHACA_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < reps; ++i) run();
    ITHACA_CUDA(cudaEventRecord(e1, s));
    ITHACA_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    ITHACA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *avg_ms = ms / reps;
    if (bytes_per_launch) {
      // algorithmic bytes per element: the signed l2g index (4 B), the gathered input and
      // the output per local dof, and J w plus the symmetric metric per point (+ 8 scales
      // per element for 16-bit geometry). The output codes of the scattered FP32 output
      // (4 B per local dof) are this kernel's layout choice and are not counted.
      const double es = f32 ? 4.0 : 8.0, gs = half ? 2.0 : es;
      const double npt = op->deformed ? op->nq : 1;
      *bytes_per_launch =
          (double)op->E * (op->nm * (4.0 + 2.0 * es) + n_jg(op->dim) * npt * gs + (half ? 32.0 : 0.0));
    }
  });
}

}  // extern "C"

static ithaca_gpu_cg_opts opts_or_default(const ithaca_gpu_cg_opts* o) {
  ithaca_gpu_cg_opts d;
  ithaca_gpu_cg_default_opts(&d);
  if (!o) return d;
  d = *o;
  if (d.max_iter <= 0) d.max_iter = 5000;
  if (d.check_every <= 0) d.check_every = 16;
  if (d.max_outer <= 0) d.max_outer = 50;
  if (!(d.inner_tol > 0 && d.inner_tol < 1)) d.inner_tol = 1e-2;
  return d;
}

namespace ithaca {

int cg_sizes(ithaca_gpu_cg* cg, int* nglobal, int* ndir, Ctx** ctx) {
  *nglobal = cg->N;
  *ndir = cg->ndir;
  *ctx = cg->op->ctx;
  return 0;
}

// Columns of X (nglobal rows each): LX = Assemble(Laplacian(GlobalToLocal x)) and
// MX = Assemble(IProduct(BwdTrans(GlobalToLocal x))), the lambda-free pieces of the
// affine operator A(lambda) = L + lambda M (Dirichlet entries of x read as zero).
void cg_apply_LM(ithaca_gpu_cg* cg, int ncols, const double* X, double* LX, double* MX) {
  Op* op = cg->op;
  Ctx* c = op->ctx;
  cudaStream_t s = c->stream;
  double* phys = (double*)c->stage_ptr(2, sizeof(double) * op->E * op->nq);
  double* loc = (double*)c->stage_ptr(3, sizeof(double) * cg->nloc);
  for (int j = 0; j < ncols; ++j) {
    const double* x = X + (size_t)j * cg->N;
    launch_apply<double>(cg, cg->v64, op->t64.base, geo64(cg), 0.0, nullptr, x, s, true, nullptr);
    assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, cg->v64.yloc,
                                                  LX + (size_t)j * cg->N, nullptr, nullptr, nullptr);
    g2l_kernel<<<RB, RT, 0, s>>>(cg->nloc, cg->l2g, x, loc);
    if (!launch_bwdtrans<double>(op->kdim, op->n, op->Q, op->E, op->t64.base, loc, phys, s) ||
        !launch_iproduct<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64, phys, loc, s))
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "mass operator: (modes, points) combination not built");
    assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, loc, MX + (size_t)j * cg->N,
                                                  nullptr, nullptr, nullptr);
    c->launches += 5;
  }
  ITHACA_CUDA(cudaGetLastError());
}

// adjoint.cu
void launch_scale_metric(int E, int ng, int nq, const double* src, const double* kappa, double* dst, cudaStream_t s);
void launch_tensor_metric(int E, int dim, int nq, const double* jg, const double* dfe, const double* K, double* dst,
                          cudaStream_t s);
void launch_misfit(int E, int ng, int nq, const double* jg, double* u, const double* t, double* partial, double* out,
                   cudaStream_t s);
void launch_kappa_grad(int E, int ng, int nq, int dim, const double* jg, const double* du, const double* dp,
                       double* grad, cudaStream_t s);
void launch_zero_head(int n, double* a, cudaStream_t s);

// (2 dim + 2) physical-size FP64 arrays for the misfit / gradient pipelines.
static double* adj_buffers(Cg* cg) {
  if (!cg->adj_scratch) {
    const size_t nphys = (size_t)cg->op->E * cg->op->nq;
    ITHACA_CUDA(cudaMalloc(&cg->adj_scratch, sizeof(double) * nphys * (2 * cg->op->dim + 2)));
  }
  return cg->adj_scratch;
}

}  // namespace ithaca

extern "C" {

int ithaca_gpu_cg_set_varcoeff(ithaca_gpu_cg* cg, const double* kappa, int on_device) {
  return cg_guarded([&] {
    req(cg != nullptr, "null argument");
    StreamOrder order_(cg->op->ctx);
    Op* op = cg->op;
    cudaStream_t s = op->ctx->stream;
    const size_t njg = (size_t)op->E * n_jg(op->dim) * op->nq;
    if (kappa == nullptr) {  // back to kappa = 1
      cudaFree(cg->jgk64);
      cg->jgk64 = nullptr;
    } else {
      req(op->deformed != 0, "a quadrature-point coefficient needs a deformed (per-point) collection");
      const double* dk = kappa;
      if (!on_device) {
        double* d = (double*)op->ctx->stage_ptr(0, sizeof(double) * op->E * op->nq);
        ITHACA_CUDA(cudaMemcpyAsync(d, kappa, sizeof(double) * op->E * op->nq, cudaMemcpyHostToDevice, s));
        dk = d;
      }
      if (!cg->jgk64) ITHACA_CUDA(cudaMalloc(&cg->jgk64, sizeof(double) * njg));
      launch_scale_metric(op->E, n_jg(op->dim), op->nq, op->jg64, dk, cg->jgk64, s);
      op->ctx->launches++;
    }
    if (cg->have32) {
      cast_kernel<float><<<RB, RT, 0, s>>>(njg / (op->deformed ? 1 : op->nq), geo64(cg), cg->jg32);
      op->ctx->launches++;
    }
    if (cg->have16) build_geo16(cg);
    cg->diag_lambda = NAN;
    cg->proj.lambda = NAN;  // a new operator: stored solutions of the old one no longer apply
    cg->aniso = false;
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_cg_set_varcoeff_tensor(ithaca_gpu_cg* cg, const double* K, int on_device) {
  return cg_guarded([&] {
    req(cg != nullptr && K != nullptr, "null argument");
    StreamOrder order_(cg->op->ctx);
    Op* op = cg->op;
    req(op->deformed != 0, "a quadrature-point coefficient needs a deformed (per-point) collection");
    if (op->kdim != op->dim)
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "the coefficient tensor is built for quadrilaterals and hexahedra");
    cudaStream_t s = op->ctx->stream;
    const int dim = op->dim, nk = dim * (dim + 1) / 2;
    const size_t npts = (size_t)op->E * op->nq, njg = (size_t)op->E * n_jg(dim) * op->nq;
    const double* dk = K;
    if (!on_device) {
      double* d = (double*)op->ctx->stage_ptr(0, sizeof(double) * nk * npts);
      ITHACA_CUDA(cudaMemcpyAsync(d, K, sizeof(double) * nk * npts, cudaMemcpyHostToDevice, s));
      dk = d;
    }
    if (!cg->jgk64) ITHACA_CUDA(cudaMalloc(&cg->jgk64, sizeof(double) * njg));
    launch_tensor_metric(op->E, dim, op->nq, op->jg64, op->df64, dk, cg->jgk64, s);
    op->ctx->launches++;
    if (cg->have32) {
      cast_kernel<float><<<RB, RT, 0, s>>>(njg, geo64(cg), cg->jg32);
      op->ctx->launches++;
    }
    if (cg->have16) build_geo16(cg);
    cg->diag_lambda = NAN;
    cg->proj.lambda = NAN;
    cg->aniso = true;
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_misfit(ithaca_gpu_cg* cg, const double* x, const double* u_target, double* J, double* dJdx,
                      int on_device) {
  return cg_guarded([&] {
    req(cg && x && u_target && J, "null argument");
    if (cg->op->kdim != cg->op->dim)
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "the adjoint misfit is built for quadrilaterals and hexahedra");
    StreamOrder order_(cg->op->ctx);
    Op* op = cg->op;
    Ctx* c = op->ctx;
    cudaStream_t s = c->stream;
    const size_t nphys = (size_t)op->E * op->nq;
    double* buf = adj_buffers(cg);
    double *phys = buf, *tgt = buf + nphys;
    const double* dx = x;
    if (!on_device) {
      ITHACA_CUDA(cudaMemcpyAsync(cg->v64.p, x, sizeof(double) * cg->N, cudaMemcpyHostToDevice, s));
      dx = cg->v64.p;
    }
    ITHACA_CUDA(cudaMemcpyAsync(tgt, u_target, sizeof(double) * nphys,
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    // u at the points from the non-Dirichlet part of x (Dirichlet values are zero)
    ITHACA_CUDA(cudaMemcpyAsync(cg->v64.q, dx, sizeof(double) * cg->N, cudaMemcpyDeviceToDevice, s));
    launch_zero_head(cg->ndir, cg->v64.q, s);
    g2l_kernel<<<RB, RT, 0, s>>>(cg->nloc, cg->l2g, cg->v64.q, cg->v64.yloc);
    if (!launch_bwdtrans<double>(op->kdim, op->n, op->Q, op->E, op->t64.base, cg->v64.yloc, phys, s))
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "BwdTrans: (modes, points) combination not built");
    launch_misfit(op->E, n_jg(op->dim), op->nq, op->jg64, phys, tgt, cg->partials, cg->dscal + 2, s);
    c->launches += 5;
    if (dJdx) {
      // dJ/dx = Assemble(IProduct(2 (u - t))), zero on Dirichlet dofs
      if (!launch_iproduct<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64, phys,
                                   cg->v64.yloc, s))
        fail(ITHACA_GPU_ERR_UNSUPPORTED, "IProductWRTBase: (modes, points) combination not built");
      double* dg = on_device ? dJdx : cg->v64.q;
      assemble_dot_kernel<double><<<cg->rba, RT, 0, s>>>(cg->plan, false, cg->asm_rows, cg->asm_cols, cg->rowptr, cg->cols, cg->v64.yloc, dg, nullptr,
                                                    nullptr, nullptr);
      launch_zero_head(cg->ndir, dg, s);
      c->launches += 3;
      if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(dJdx, dg, sizeof(double) * cg->N, cudaMemcpyDeviceToHost, s));
    }
    ITHACA_CUDA(cudaMemcpyAsync(J, cg->dscal + 2, sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_kappa_gradient(ithaca_gpu_cg* cg, const double* x, const double* psi, double* grad, int on_device) {
  return cg_guarded([&] {
    req(cg && x && psi && grad, "null argument");
    if (cg->aniso) fail(ITHACA_GPU_ERR_UNSUPPORTED, "the kappa gradient is for an isotropic coefficient");
    if (cg->op->kdim != cg->op->dim)
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "the kappa gradient is built for quadrilaterals and hexahedra");
    StreamOrder order_(cg->op->ctx);
    Op* op = cg->op;
    Ctx* c = op->ctx;
    cudaStream_t s = c->stream;
    const int dim = op->dim;
    const size_t nphys = (size_t)op->E * op->nq;
    double* buf = adj_buffers(cg);
    double *du = buf, *dp = buf + dim * nphys, *phys = buf + 2 * dim * nphys;
    const double* src[2] = {x, psi};
    double* outs[2] = {du, dp};
    for (int k = 0; k < 2; ++k) {
      ITHACA_CUDA(cudaMemcpyAsync(cg->v64.q, src[k], sizeof(double) * cg->N,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
      launch_zero_head(cg->ndir, cg->v64.q, s);
      g2l_kernel<<<RB, RT, 0, s>>>(cg->nloc, cg->l2g, cg->v64.q, cg->v64.yloc);
      if (!launch_bwdtrans<double>(dim, op->n, op->Q, op->E, op->t64.base, cg->v64.yloc, phys, s) ||
          !launch_physderiv<double>(dim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->df64, phys, outs[k],
                                    outs[k] + nphys, dim == 3 ? outs[k] + 2 * nphys : nullptr, s))
        fail(ITHACA_GPU_ERR_UNSUPPORTED, "BwdTrans/PhysDeriv: (modes, points) combination not built");
      c->launches += 4;
    }
    double* dgrad = on_device ? grad : phys;
    launch_kappa_grad(op->E, n_jg(dim), op->nq, dim, op->jg64, du, dp, dgrad, s);
    c->launches++;
    if (!on_device) ITHACA_CUDA(cudaMemcpyAsync(grad, dgrad, sizeof(double) * nphys, cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
