// Batched parametric Helmholtz solves: many independent C0 systems (different meshes,
// orders and lambdas) solved together.
//
// In the reference each parameter sample is a separate FOM solve (the snapshot loop
// of the ITHACA offline phase, CoupledLinearNS_ROM.cpp:1208-1283 loads one solution per
// parameter; each comes from ContField::HelmSolve -> NekLinSysIterCG). Here the solves
// are grouped by polynomial order; a group is one block-diagonal system:
//  * elements of all its solves concatenated, lambda_s folded into J w of solve s;
//  * global ids renumbered: every solve's Dirichlet dofs first, then the free dofs of
//    solve 0, 1, ... as contiguous segments;
//  * per-solve CG scalars (the recurrence of NekLinSysIterCG.cpp:104-263 per segment),
//    reductions over fixed chunks of a segment, summed in order by one CTA per solve;
//  * elements of converged solves skip their I/O in the element kernel.
// One CUDA graph holds `check_every` iterations of every group, one parallel branch per
// group, and is launched until all solves flag convergence. Mixed mode wraps the FP32
// inner batch in per-solve FP64 iterative refinement.
#include <algorithm>
#include <cmath>
#include <map>
#include <functional>
#include <memory>
#include <vector>

#include "ithaca_internal.h"

namespace ithaca {
namespace batch {

constexpr int BT = 256;        // threads per CTA
constexpr int CH = 4096;       // dofs per reduction chunk
constexpr int kChunkPerSM = 4;  // CTAs per SM of the chunk kernels
// CTAs of a full chunk-kernel grid on the current device
inline int chunk_grid() { return kChunkPerSM * device_sm_count(); }

struct Scal {
  double alpha, beta, rho, mu, eps, rhs_mag, tol2, mag_override, bb_dir;
  double rn2, bn2, scale;  // mixed mode: outer residual, rhs norm, inner scaling
  int iters, k, done, status, max_iter, outer_done;
};
constexpr int kDoneStride = sizeof(Scal) / sizeof(int);
static_assert(sizeof(Scal) % sizeof(int) == 0, "Scal must be int-aligned");

struct Chunk {
  int solve, begin, end;
};

template <int NC>
__device__ __forceinline__ void block_sum(double (&v)[NC], double* out /* NC values */) {
  __shared__ double sm[NC][BT / 32];
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
    for (int w = 0; w < BT / 32; ++w) s += sm[threadIdx.x][w];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// FP32 per-thread values: warp sums in FP32 (shuffles) and only the sum of the warp sums
// in FP64. FP64 runs at ~1/60 of the FP32 rate on this GPU, and an FP64 shuffle tree over
// every lane for every chunk keeps the SMs' FP64 pipes busy for tens of microseconds
// per iteration of the batch.
template <int NC>
__device__ __forceinline__ void block_sum(float (&v)[NC], double* out /* NC values */) {
  __shared__ double sm[NC][BT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], off);
    if (lane == 0) sm[c][warp] = (double)v[c];
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double t = sm[threadIdx.x][0];
#pragma unroll
    for (int w = 1; w < BT / 32; ++w) t += sm[threadIdx.x][w];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// part layout: part[slot * nchunks + chunk]; slots 0 r.w, 1 r.r, 2 b.b, 3 s.w
template <typename T>
__global__ void __launch_bounds__(BT) binit_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                   const Scal* __restrict__ sc, const T* __restrict__ b,
                                                   T* __restrict__ x, T* __restrict__ r, T* __restrict__ w,
                                                   const T* __restrict__ dinv, double* __restrict__ part) {
  __shared__ double res[3];
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    if (sc[ch.solve].done) continue;  // converged (or idle) solve: no work, no partials
    double v[3] = {0, 0, 0};
    if (!sc[ch.solve].done) {
      for (int g = ch.begin + threadIdx.x; g < ch.end; g += BT) {
        const T rg = b[g];
        const T wg = dinv[g] * rg;
        r[g] = rg;
        x[g] = T(0);
        w[g] = wg;
        v[0] += (double)rg * (double)wg;
        v[1] += (double)rg * (double)rg;
        v[2] += (double)rg * (double)rg;
      }
    }
    block_sum<3>(v, res);
    if (threadIdx.x < 3) part[threadIdx.x * nchunks + c] = res[threadIdx.x];
  }
}

template <typename T>
__global__ void __launch_bounds__(BT, kChunkPerSM) bupdate_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                     const Scal* __restrict__ sc, T* __restrict__ x,
                                                     T* __restrict__ r, T* __restrict__ w, const T* __restrict__ s,
                                                     T* __restrict__ p, T* __restrict__ q,
                                                     const T* __restrict__ dinv, double* __restrict__ part) {
  __shared__ double res[2];
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const Scal& S = sc[ch.solve];
    if (S.done) continue;  // converged solve: no work, no partials (its scalars step skips it)
    // per-thread sums in T (a chunk gives each thread 16 dofs; FP32 sums keep the
    // FP32 solve off the slow FP64 pipe), CTA sums in FP64
    T rw = 0, rr = 0;
    if constexpr (sizeof(T) == 4) {
      // FP32: the 16-byte-aligned interior of the chunk as float4 groups (one group per
      // thread step, every vector moved with 16-byte loads and stores), the ragged ends
      // (fewer than 4 dofs each) one dof per thread
      const float alpha = (float)S.alpha, beta = (float)S.beta;
      auto upd = [&](float& pv, float& qv, float& xv, float& rv, float& wv, float dv, float sv) {
        pv = beta * pv + wv;
        qv = beta * qv + sv;
        xv = xv + alpha * pv;
        rv = rv - alpha * qv;
        wv = dv * rv;
        rw = fma(rv, wv, rw);
        rr = fma(rv, rv, rr);
      };
      const int a0 = min((ch.begin + 3) & ~3, ch.end), a1 = max(ch.end & ~3, a0);
      const int nh = a0 - ch.begin, nt = ch.end - a1;
      if ((int)threadIdx.x < nh + nt) {
        const int g = (int)threadIdx.x < nh ? ch.begin + threadIdx.x : a1 + (threadIdx.x - nh);
        float pv = p[g], qv = q[g], xv = x[g], rv = r[g], wv = w[g];
        upd(pv, qv, xv, rv, wv, dinv[g], s[g]);
        p[g] = pv;
        q[g] = qv;
        x[g] = xv;
        r[g] = rv;
        w[g] = wv;
      }
      for (int q4 = (a0 >> 2) + threadIdx.x; q4 < (a1 >> 2); q4 += BT) {
        float4 P4 = reinterpret_cast<const float4*>(p)[q4], W4 = reinterpret_cast<const float4*>(w)[q4];
        float4 Q4 = reinterpret_cast<const float4*>(q)[q4], X4 = reinterpret_cast<const float4*>(x)[q4];
        float4 R4 = reinterpret_cast<const float4*>(r)[q4];
        const float4 S4 = reinterpret_cast<const float4*>(s)[q4], D4 = reinterpret_cast<const float4*>(dinv)[q4];
        upd(P4.x, Q4.x, X4.x, R4.x, W4.x, D4.x, S4.x);
        upd(P4.y, Q4.y, X4.y, R4.y, W4.y, D4.y, S4.y);
        upd(P4.z, Q4.z, X4.z, R4.z, W4.z, D4.z, S4.z);
        upd(P4.w, Q4.w, X4.w, R4.w, W4.w, D4.w, S4.w);
        reinterpret_cast<float4*>(p)[q4] = P4;
        reinterpret_cast<float4*>(q)[q4] = Q4;
        reinterpret_cast<float4*>(x)[q4] = X4;
        reinterpret_cast<float4*>(r)[q4] = R4;
        reinterpret_cast<float4*>(w)[q4] = W4;
      }
    } else {
      const T alpha = (T)S.alpha, beta = (T)S.beta;
      // U dofs per thread step with their loads issued together (memory-level parallelism)
      constexpr int U = 2;
      for (int g0 = ch.begin + threadIdx.x; g0 < ch.end; g0 += U * BT) {
        T pv[U], wv[U], qv[U], sv[U], xv[U], rv[U], dv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int g = g0 + u * BT;
          const bool in = g < ch.end;
          pv[u] = in ? p[g] : T(0);
          wv[u] = in ? w[g] : T(0);
          qv[u] = in ? q[g] : T(0);
          sv[u] = in ? s[g] : T(0);
          xv[u] = in ? x[g] : T(0);
          rv[u] = in ? r[g] : T(0);
          dv[u] = in ? dinv[g] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int g = g0 + u * BT;
          if (g < ch.end) {
            const T pg = beta * pv[u] + wv[u];
            const T qg = beta * qv[u] + sv[u];
            p[g] = pg;
            q[g] = qg;
            x[g] = xv[u] + alpha * pg;
            const T rg = rv[u] - alpha * qg;
            r[g] = rg;
            const T wg = dv[u] * rg;
            w[g] = wg;
            rw = fma(rg, wg, rw);
            rr = fma(rg, rg, rr);
          }
        }
      }
    }
    T v[2] = {rw, rr};
    block_sum<2>(v, res);
    if (threadIdx.x < 2) part[threadIdx.x * nchunks + c] = res[threadIdx.x];
  }
}

template <typename T>
__global__ void __launch_bounds__(BT) bassemble_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                       const Scal* __restrict__ sc, const int* __restrict__ rowptr,
                                                       const int* __restrict__ cols, const T* __restrict__ yloc,
                                                       T* __restrict__ s, const T* __restrict__ w,
                                                       double* __restrict__ part) {
  __shared__ double res[1];
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    if (sc[ch.solve].done) continue;  // converged solve: no work, no partials
    T sw = 0;  // per-thread s.w in T, CTA sum in FP64
    if (!sc[ch.solve].done) {
      // U rows per thread step (2 in FP64), each row's entries summed in CSR order. The first K
      // entries of every row (a quad-mesh vertex has 4, an edge mode 2, an interior
      // mode 1) are loaded without a loop: all column indices of the U rows in flight
      // together, then all their values, so a row costs three dependent loads (rowptr,
      // cols, yloc) rather than two per entry. Longer rows finish in a loop.
      constexpr int U = sizeof(T) == 8 ? 2 : 4, K = 4;
      for (int g0 = ch.begin + threadIdx.x; g0 < ch.end; g0 += U * BT) {
        int a[U], b[U], cc[U][K];
        T wv[U], acc[U], val[U][K];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int g = g0 + u * BT;
          const bool in = g < ch.end;
          a[u] = in ? rowptr[g] : 0;
          b[u] = in ? rowptr[g + 1] : 0;
          wv[u] = in ? w[g] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int j = 0; j < K; ++j) cc[u][j] = a[u] + j < b[u] ? cols[a[u] + j] : 0;
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int j = 0; j < K; ++j) {
            const int c = cc[u][j];
            val[u][j] = a[u] + j < b[u] ? (c >= 0 ? yloc[c] : -yloc[~c]) : T(0);
          }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          acc[u] = val[u][0];
#pragma unroll
          for (int j = 1; j < K; ++j)
            if (a[u] + j < b[u]) acc[u] += val[u][j];
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
          for (int j = a[u] + K; j < b[u]; ++j) {
            const int c = cols[j];
            acc[u] += c >= 0 ? yloc[c] : -yloc[~c];
          }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int g = g0 + u * BT;
          if (g < ch.end) {
            s[g] = acc[u];
            sw = fma(acc[u], wv[u], sw);
          }
        }
      }
    }
    T v[1] = {sw};
    block_sum<1>(v, res);
    if (threadIdx.x == 0) part[3 * nchunks + c] = res[0];
  }
}

// Sums over chunks [c0, c1) of several partial slots at once: every load of a thread in
// flight together, one shared-memory tree (one barrier per level) for all slots.
template <int NS>
__device__ __forceinline__ void sum_ranges(const double* part, int nchunks, const int (&slots)[NS], int c0, int c1,
                                           double (&out)[NS]) {
  __shared__ double sm[NS][BT];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    double t = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += BT) t += part[slots[k] * nchunks + c];
    sm[k][threadIdx.x] = t;
  }
  __syncthreads();
  for (int wdt = BT / 2; wdt > 0; wdt >>= 1) {
    if (threadIdx.x < wdt) {
#pragma unroll
      for (int k = 0; k < NS; ++k) sm[k][threadIdx.x] += sm[k][threadIdx.x + wdt];
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < NS; ++k) out[k] = sm[k][0];
  __syncthreads();
}

// One CTA per solve: the reference's initial step (NekLinSysIterCG.cpp:147-190).
__global__ void __launch_bounds__(BT) bscalars_init_kernel(Scal* __restrict__ sc, const double* __restrict__ part,
                                                           int nchunks, const int* __restrict__ cstart) {
  const int sv = blockIdx.x;
  Scal& S = sc[sv];
  if (S.done) return;  // solves that need no (more) work were flagged on entry
  const int c0 = cstart[sv], c1 = cstart[sv + 1];
  const int slots[4] = {0, 1, 2, 3};
  double red[4];
  sum_ranges<4>(part, nchunks, slots, c0, c1, red);
  const double rw = red[0], rr = red[1], bb = red[2] + S.bb_dir, sw = red[3];
  if (threadIdx.x == 0) {
    S.rhs_mag = S.mag_override > 0 ? S.mag_override : (bb > 1e-6 ? bb : 1.0);
    S.eps = rr;
    S.iters = 0;
    S.k = 0;
    S.status = ITHACA_GPU_OK;
    if (!isfinite(rr) || !isfinite(rw) || !isfinite(sw)) {
      S.status = ITHACA_GPU_ERR_NUMERIC;
      S.done = 1;
    } else if (rr < S.tol2 * S.rhs_mag) {
      S.done = 1;
    } else {
      S.rho = rw;
      S.mu = sw;
      S.beta = 0.0;
      S.alpha = rw / sw;
      S.iters = 1;
      if (S.max_iter <= 0) {
        S.status = ITHACA_GPU_ERR_NOT_CONVERGED;
        S.done = 1;
      }
    }
  }
}

// One CTA per solve: the reference loop tail (NekLinSysIterCG.cpp:219-261).
__global__ void __launch_bounds__(BT) bscalars_iter_kernel(Scal* __restrict__ sc, const double* __restrict__ part,
                                                           int nchunks, const int* __restrict__ cstart) {
  const int sv = blockIdx.x;
  Scal& S = sc[sv];
  if (S.done) return;
  const int c0 = cstart[sv], c1 = cstart[sv + 1];
  const int slots[3] = {0, 1, 3};
  double red[3];
  sum_ranges<3>(part, nchunks, slots, c0, c1, red);
  const double rho_new = red[0], eps = red[1], mu = red[2];
  if (threadIdx.x == 0) {
    S.eps = eps;
    S.mu = mu;
    S.iters += 1;
    if (!isfinite(eps) || !isfinite(rho_new) || !isfinite(mu)) {
      S.status = ITHACA_GPU_ERR_NUMERIC;
      S.done = 1;
    } else if (eps < S.tol2 * S.rhs_mag) {
      S.done = 1;
    } else {
      const double beta = rho_new / S.rho;
      S.alpha = rho_new / (mu - rho_new * beta / S.alpha);
      S.beta = beta;
      S.rho = rho_new;
      S.k += 1;
      if (S.k >= S.max_iter) {
        S.status = ITHACA_GPU_ERR_NOT_CONVERGED;
        S.done = 1;
      }
    }
  }
}

// ---- mixed-precision outer step kernels (FP64) ----
// r = b - sum yloc on the free dofs; partial r.r (slot 1), b.b (slot 2). With skip_done the
// solves already converged (outer_done) are left out: their x no longer changes, and their
// norms stay as the outer kernel last recorded them.
__global__ void __launch_bounds__(BT) bresidual_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                       const Scal* __restrict__ sc, const int* __restrict__ rowptr,
                                                       const int* __restrict__ cols, const double* __restrict__ yloc,
                                                       const double* __restrict__ b, double* __restrict__ r,
                                                       double* __restrict__ part, int skip_done) {
  __shared__ double res[2];
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    if (skip_done && sc[ch.solve].outer_done) continue;
    double v[2] = {0, 0};
    for (int g = ch.begin + threadIdx.x; g < ch.end; g += BT) {
      // the first K entries' indices, then their values, in flight together (as in
      // bassemble_kernel); summed in CSR order
      constexpr int K = 4;
      const int a0 = rowptr[g], a1 = rowptr[g + 1];
      int cc[K];
      double val[K];
#pragma unroll
      for (int j = 0; j < K; ++j) cc[j] = a0 + j < a1 ? cols[a0 + j] : 0;
#pragma unroll
      for (int j = 0; j < K; ++j) val[j] = a0 + j < a1 ? (cc[j] >= 0 ? yloc[cc[j]] : -yloc[~cc[j]]) : 0.0;
      double acc = 0;
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (a0 + j < a1) acc += val[j];
      for (int j = a0 + K; j < a1; ++j) {
        const int c2 = cols[j];
        acc += c2 >= 0 ? yloc[c2] : -yloc[~c2];
      }
      const double rg = b[g] - acc;
      r[g] = rg;
      v[0] += rg * rg;
      v[1] += b[g] * b[g];
    }
    block_sum<2>(v, res);
    if (threadIdx.x < 2) part[(1 + threadIdx.x) * nchunks + c] = res[threadIdx.x];
  }
}

// One CTA per solve: outer convergence test; arms the inner solve of the others.
__global__ void __launch_bounds__(BT) bouter_kernel(Scal* __restrict__ outer, Scal* __restrict__ inner,
                                                    const double* __restrict__ part, int nchunks,
                                                    const int* __restrict__ cstart, double tol2, double inner_tol2,
                                                    int max_iter_inner, int skip_done) {
  const int sv = blockIdx.x;
  const int c0 = cstart[sv], c1 = cstart[sv + 1];
  const bool was_done = skip_done && outer[sv].outer_done;  // its residual was not recomputed
  const int slots[2] = {1, 2};
  double red[2];
  sum_ranges<2>(part, nchunks, slots, c0, c1, red);
  const double rr = red[0], bb = red[1];
  if (threadIdx.x == 0) {
    Scal& O = outer[sv];
    if (!was_done) {
      O.rn2 = rr;
      O.bn2 = bb;
    }
    if (!was_done && !isfinite(rr)) O.status = ITHACA_GPU_ERR_NUMERIC;
    O.outer_done = (O.outer_done || !(rr > tol2 * bb) || bb == 0 || O.status != ITHACA_GPU_OK) ? 1 : 0;
    Scal I = Scal{};
    I.tol2 = inner_tol2;
    I.mag_override = 1.0;
    I.max_iter = max_iter_inner;
    I.done = O.outer_done;
    I.scale = O.outer_done ? 0.0 : 1.0 / sqrt(rr);
    inner[sv] = I;
  }
}

// r32 = r64 * scale_s (solves still refining), x64 += d32 / scale_s after the inner solve
__global__ void __launch_bounds__(BT) bscale_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                    const Scal* __restrict__ inner, const double* __restrict__ r,
                                                    float* __restrict__ r32) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const double sc = inner[ch.solve].done ? 0.0 : inner[ch.solve].scale;
    for (int g = ch.begin + threadIdx.x; g < ch.end; g += BT) r32[g] = (float)(r[g] * sc);
  }
}

__global__ void __launch_bounds__(BT) baxpy_kernel(const Chunk* __restrict__ chunks, int nchunks,
                                                   const Scal* __restrict__ outer, const float* __restrict__ d32,
                                                   double* __restrict__ x) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const Scal& O = outer[ch.solve];
    if (O.outer_done) continue;
    const double sc = sqrt(O.rn2);
    for (int g = ch.begin + threadIdx.x; g < ch.end; g += BT) x[g] += sc * (double)d32[g];
  }
}

// ---- device-side loop control of the one-launch solve ----
// One CTA: is any solve of any group still active (inner loop: !done; outer loop:
// !outer_done)? Advances the loop counter and sets the conditional node(s) to
// (active && counter < bound): the bound makes every device-side loop finite even if a
// flag were never set.
__global__ void __launch_bounds__(BT) bactive_kernel(Scal* const* __restrict__ scs, const int* __restrict__ nsolve,
                                                     int ngroups, int outer, unsigned* counter, unsigned bound,
                                                     cudaGraphConditionalHandle h, cudaGraphConditionalHandle h2,
                                                     int set2) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  int mine = 0;
  for (int g = 0; g < ngroups; ++g) {
    const Scal* sc = scs[g];
    for (int k = threadIdx.x; k < nsolve[g]; k += BT) mine |= outer ? !sc[k].outer_done : !sc[k].done;
  }
  if (mine) any = 1;  // every writer stores the same value
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned c = ++*counter;
    const unsigned v = (any && c < bound) ? 1u : 0u;
    cudaGraphSetConditional(h, v);
    if (set2) cudaGraphSetConditional(h2, v);
  }
}

// Sets a conditional handle. A WHILE node nested in another conditional's body keeps the
// value its loop ended with (the handle's default is applied at the top-level graph
// launch only), so each entry into the inner loop re-arms it first.
__global__ void bset_cond_kernel(cudaGraphConditionalHandle h, unsigned v) { cudaGraphSetConditional(h, v); }

// After an inner solve of the mixed mode: its iterations into the outer scalars' totals
// (iters: inner iterations, k: refinement steps that iterated), and a NaN/Inf status.
__global__ void baccum_kernel(Scal* __restrict__ outer, const Scal* __restrict__ inner, int n) {
  for (int k = blockIdx.x * BT + threadIdx.x; k < n; k += gridDim.x * BT) {
    outer[k].iters += inner[k].iters;
    if (inner[k].iters > 0) outer[k].k += 1;
    if (inner[k].status == ITHACA_GPU_ERR_NUMERIC) outer[k].status = ITHACA_GPU_ERR_NUMERIC;
  }
}

// ---- setup kernels ----
__global__ void scale_jw_kernel(int E, int ng, int nq, double lambda, double* __restrict__ jg) {
  const size_t total = (size_t)E * nq;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    jg[(i / nq) * ng * nq + i % nq] *= lambda;
}

__global__ void assemble_abs_kernel(int N, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                    const double* __restrict__ loc, double* __restrict__ out) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < N; g += gridDim.x * blockDim.x) {
    double acc = 0;
    for (int j = rowptr[g]; j < rowptr[g + 1]; ++j) {
      const int cc = cols[j];
      acc += loc[cc >= 0 ? cc : ~cc];
    }
    out[g] = acc;
  }
}

__global__ void inv_free_kernel(int N, int ndir, const double* __restrict__ d, double* __restrict__ dinv,
                                float* __restrict__ dinv32) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < N; g += gridDim.x * blockDim.x) {
    const double v = g >= ndir ? 1.0 / d[g] : 0.0;
    dinv[g] = v;
    dinv32[g] = (float)v;
  }
}

__global__ void cast_f32_kernel(size_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

template <typename T>
struct Vec {
  T *x = nullptr, *r = nullptr, *w = nullptr, *s = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr,
    *b = nullptr, *yloc = nullptr;
  void alloc(size_t N, size_t nloc) {
    for (T** pp : {&x, &r, &w, &s, &p, &q, &dinv, &b}) {
      ITHACA_CUDA(cudaMalloc(pp, sizeof(T) * N));
      ITHACA_CUDA(cudaMemset(*pp, 0, sizeof(T) * N));
    }
    ITHACA_CUDA(cudaMalloc(&yloc, sizeof(T) * nloc));
  }
  void release() {
    for (T* p0 : {x, r, w, s, p, q, dinv, b, yloc}) cudaFree(p0);
  }
};

struct Group {
  int n = 0, Q = 0, dim = 2, E = 0, nm = 0, nq = 0;
  int N = 0, ndir = 0, nsolve = 0, nchunks = 0;
  std::vector<int> solves;          // batch index of each solve in this group
  std::vector<int> dir_off, free_off, nfree, nglobal_s, ndir_s;
  std::vector<double> bbdir_host;   // squared norm of each solve's Dirichlet rhs entries
  double* t64 = nullptr;
  float* t32 = nullptr;
  double* jg64 = nullptr;
  float* jg32 = nullptr;
  int *l2g = nullptr, *rowptr = nullptr, *cols = nullptr, *esolve = nullptr, *cstart = nullptr;
  Chunk* chunks = nullptr;
  double* part = nullptr;
  Scal *sc = nullptr, *sc_outer = nullptr;
  Vec<double> v64;
  Vec<float> v32;
  cudaStream_t stream = nullptr;
  cudaEvent_t done_ev = nullptr;
  // element-kernel variant of the group's applies (tile shape; -1 the default), chosen
  // per order by ithaca_gpu_batch_autotune
  int var32 = -1, var64 = -1;
  size_t nloc() const { return (size_t)E * nm; }
  ~Group() {
    cudaFree(t64);
    cudaFree(t32);
    cudaFree(jg64);
    cudaFree(jg32);
    for (void* p : {(void*)l2g, (void*)rowptr, (void*)cols, (void*)esolve, (void*)cstart, (void*)chunks,
                    (void*)part, (void*)sc, (void*)sc_outer})
      cudaFree(p);
    v64.release();
    v32.release();
    if (stream) cudaStreamDestroy(stream);
    if (done_ev) cudaEventDestroy(done_ev);
  }
};

template <typename T>
static void upload_tabs(T** dst, const BasisTables& b) {
  const int n = b.n, Q = b.Q;
  std::vector<T> h((size_t)4 * n * Q + 2 * Q * Q + Q);
  for (int p = 0; p < n; ++p)
    for (int i = 0; i < Q; ++i) {
      h[off_B(n, Q) + p * Q + i] = (T)b.B[p * Q + i];
      h[off_Bt(n, Q) + i * n + p] = (T)b.B[p * Q + i];
      h[off_DB(n, Q) + p * Q + i] = (T)b.DB[p * Q + i];
      h[off_DBt(n, Q) + i * n + p] = (T)b.DB[p * Q + i];
    }
  for (int k = 0; k < Q; ++k)
    for (int i = 0; i < Q; ++i) {
      h[off_D(n, Q) + k * Q + i] = (T)b.D[k * Q + i];
      h[off_Dt(n, Q) + i * Q + k] = (T)b.D[k * Q + i];
    }
  for (int i = 0; i < Q; ++i) h[off_w(n, Q) + i] = (T)b.w[i];
  ITHACA_CUDA(cudaMalloc(dst, h.size() * sizeof(T)));
  ITHACA_CUDA(cudaMemcpy(*dst, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

}  // namespace batch

struct Batch {
  Ctx* ctx = nullptr;
  int dim = 2, nsolve = 0;
  std::vector<std::unique_ptr<batch::Group>> groups;
  std::vector<std::pair<int, int>> where;  // batch solve -> (group, index in group)
  cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
  int graph64_len = 0, graph32_len = 0;
  cudaEvent_t fork = nullptr;
  // the whole solve as one graph launch with device-side loops (conditional nodes):
  // 1 (default) on, 0 the host-checked chunk launches
  int one_launch = 1;
  cudaGraphExec_t solve64 = nullptr, solve_mixed = nullptr;
  long long solve64_key = -1, solve_mixed_key = -1;  // chunk, bounds the graphs were built for
  cudaStream_t cap[3] = {nullptr, nullptr, nullptr};  // capture streams of the loop bodies
  batch::Scal** d_sc = nullptr;      // per group: inner scalars
  batch::Scal** d_outer = nullptr;   // per group: outer scalars
  int* d_nsolve = nullptr;
  unsigned* d_counter = nullptr;     // [0] inner loop, [1] outer loop
  ~Batch() {
    if (graph64) cudaGraphExecDestroy(graph64);
    if (graph32) cudaGraphExecDestroy(graph32);
    if (solve64) cudaGraphExecDestroy(solve64);
    if (solve_mixed) cudaGraphExecDestroy(solve_mixed);
    if (fork) cudaEventDestroy(fork);
    for (cudaStream_t c : cap)
      if (c) cudaStreamDestroy(c);
    cudaFree(d_sc);
    cudaFree(d_outer);
    cudaFree(d_nsolve);
    cudaFree(d_counter);
  }
};

}  // namespace ithaca

#include "batched_api.inc"
