// Persistent solver for small 2-D systems: the whole Jacobi-PCG of one system in one
// cooperative launch.
//
// The graph-captured solver (cg.cu) runs three kernels per iteration. On a 32 x 32 quad
// mesh (37 k unknowns) each of them is a few microseconds of work behind a few
// microseconds of launch and drain, so an iteration costs ~28 us. Here one CTA per
// resident slot loops over the iterations itself, with two grid barriers per iteration:
//
//   phase A (elements): gather w, element Helmholtz, scattered output (owned rows into s,
//            the others into assembly-ordered slots) and the CTA's share of s.w = y.(P w)
//   -- barrier --
//   scalars: every CTA sums the same partials in the same order, so all hold the same
//            alpha, beta, rho and the same stop decision (the reference loop tail,
//            NekLinSysIterCG.cpp:219-261)
//   phase B (rows): assemble the non-owned rows from their slots and update p, q, x, r,
//            w = M^-1 r with the CTA's share of r.w and r.r
//   -- barrier --
//
// Values written by other CTAs inside the launch (w, the owned rows of s, the slots, the
// partials) are read with L2 loads (ld.global.cg): the L1 caches are not coherent. A row
// of p, q, x, r is read and written by the same thread in every iteration.
//
// The recurrence, stop rule and summation structure are those of cg.cu, so the iteration
// counts agree with the graph-captured solver. Every barrier wait is bounded: a CTA that
// waits too long sets ITHACA_GPU_ERR_TIMEOUT and leaves, and so do the others.
#include <algorithm>

#include "cg_shared.h"
#include "elem.cuh"

namespace ithaca {
namespace dev {

constexpr int PT = 256;                       // threads per CTA
constexpr int RC = 4;                         // free rows per thread kept in registers
constexpr long long kBarrierPolls = 1 << 24;  // ~1 s of polling at 64 ns per poll

// Grid barrier (arrival counter + generation). Returns false on timeout in any thread.
// polls bounds the wait (kBarrierPolls unless a test hook shortens it). A CTA with
// drop set does not arrive: it reports the timeout at once, and every other CTA's wait
// then runs out (the failure-path test hook; never set in a solve).
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err, long long polls_max, bool drop = false) {
  __syncthreads();
  bool ok = true;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();  // this CTA's writes are visible before it arrives
    if (drop) {
      ok = false;
      if (err != nullptr) atomicExch(err, ITHACA_GPU_ERR_TIMEOUT);
    } else if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      bar[0] = 0u;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long polls = 0;
      while (*gen == g) {
        if (++polls > polls_max) {
          ok = false;
          if (err != nullptr) atomicExch(err, ITHACA_GPU_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

// Sums of NS per-CTA partials (part[slot[k] * G + cta]) in a fixed order; every thread
// of every CTA gets the same values.
template <int NS>
__device__ __forceinline__ void sum_partials(const double* part, const int (&slot)[NS], int G, double (&out)[NS],
                                             double* sh) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
#pragma unroll
  for (int k = 0; k < NS; ++k) sh[k * PT + tid] = tid < G ? __ldcg(part + slot[k] * G + tid) : 0.0;
  __syncthreads();
  if (tid < 32) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      double t = sh[k * PT + tid * 8];
#pragma unroll
      for (int i = 1; i < 8; ++i) t += sh[k * PT + tid * 8 + i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (tid == 0) sh[NS * PT + k] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NS; ++k) out[k] = sh[NS * PT + k];
  __syncthreads();
}

// This CTA's partials: FP32/FP64 per-thread values, warp sums in T, CTA sum in FP64.
template <typename T, int NS>
__device__ __forceinline__ void cta_partials(T (&v)[NS], double* part, int G, double* sh) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    if (lane == 0) sh[k * (PT / 32) + warp] = (double)v[k];
  }
  __syncthreads();
  if (tid < NS) {
    double t = sh[tid * (PT / 32)];
    for (int w = 1; w < PT / 32; ++w) t += sh[tid * (PT / 32) + w];
    part[tid * G + blockIdx.x] = t;
  }
  __syncthreads();
}

template <typename T, int N, int Q>
__global__ void __launch_bounds__(PT) cg2_persist_kernel(const PersistArgs<T> a) {
  using S = Shape<2, Q>;
  using L = Layout<T, 2, N, Q>;
  constexpr int TPE = S::TPE, EB = S::EB, NM = N * N, NQ = Q * Q, MPT = cdiv(NM, TPE), PPT = cdiv(NQ, TPE);
  static_assert(TPE * EB == PT, "one CTA is EB elements of TPE threads");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const T* sB = sm + off_B(N, Q);
  const T* sBt = sm + off_Bt(N, Q);
  const T* sD = sm + off_D(N, Q);
  const T* sw = sm + off_w(N, Q);
  T* U = sm + L::TS + threadIdx.y * L::SLAB;
  T* F0 = U + NQ;
  T* F1 = F0 + NQ;
  T* C = F1;
  __shared__ double sh[4 * PT + 8];
  const int t = threadIdx.x, tid = threadIdx.x + threadIdx.y * TPE, G = gridDim.x;
  const int N_ = a.N, ndir = a.ndir, E = a.E;
  load_tables(sm, a.tab, tables_size(N, Q));
  const CgScalars in = *a.sc;
  const T lambda = (T)in.lambda;

  // ---- this thread's free rows: flat free-row index f = thread + k G PT, in class
  // order (class c holds the free slots [ndir_c, n_c) of the plan); x, r, p, q and the
  // inverse diagonal of these rows live in registers for the whole solve, only w (which
  // the element phase gathers) and x (at the end) go to memory ----
  const AsmPlan& P = a.plan;
  int rc[RC], ri[RC], rg[RC];
  T xr[RC], rr_[RC], pr[RC], qr[RC], wr[RC], dr[RC];
  int nrows = 0;
#pragma unroll
  for (int k = 0; k < RC; ++k) {
    rc[k] = 0;
    ri[k] = 0;
    rg[k] = 0;
    long long f = (long long)blockIdx.x * PT + tid + (long long)k * G * PT;
    int c = 0;
    for (; c <= kAsmK; ++c) {
      const int nf = P.n[c] - P.ndir[c];
      if (f < nf) break;
      f -= nf;
    }
    if (c <= kAsmK) {
      rc[k] = c;
      ri[k] = P.ndir[c] + (int)f;
      rg[k] = a.asm_rows[P.rows_off[c] + ri[k]];
      nrows = k + 1;
    }
  }

  // ---- initial step (NekLinSysIterCG.cpp:147-190): x = 0, r = b, w = M^-1 r ----
  {
    T v[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < RC; ++k) {
      xr[k] = rr_[k] = pr[k] = qr[k] = wr[k] = dr[k] = T(0);
      if (k < nrows) {
        const T bg = a.b[rg[k]];
        dr[k] = a.dinv[rg[k]];
        rr_[k] = bg;
        wr[k] = dr[k] * bg;
        a.w[rg[k]] = wr[k];
        v[0] = fma(bg, wr[k], v[0]);
        v[1] = fma(bg, bg, v[1]);
        v[2] = fma(bg, bg, v[2]);
      }
    }
    // ||b||^2 runs over every global entry, the Dirichlet ones included
    for (int g = blockIdx.x * PT + tid; g < ndir; g += G * PT) {
      const T bg = a.b[g];
      v[2] = fma(bg, bg, v[2]);
    }
    cta_partials<T, 3>(v, a.part, G, sh);  // slots 0 r.w, 1 r.r (parity 0), 2 b.b
  }

  // ---- phase A: s = A w on the elements, scattered output, the CTA's share of s.w ----
  auto phase_a = [&]() {
    T sw_loc = 0;
    const int ngroups = (E + EB - 1) / EB;
    for (int grp = blockIdx.x; grp < ngroups; grp += G) {
      const int e = grp * EB + threadIdx.y;
      const bool active = e < E;
      const int ee = active ? e : E - 1;
      T wv[MPT];
#pragma unroll
      for (int j = 0; j < MPT; ++j) {
        const int m = t + j * TPE;
        wv[j] = T(0);
        if (m < NM) {
          const int code = a.l2g[(size_t)ee * NM + m];
          const int g = code >= 0 ? code : ~code;
          const T v = g < ndir ? T(0) : __ldcg(a.w + g);  // written by other CTAs: L2
          wv[j] = code >= 0 ? v : -v;
          C[m] = wv[j];
        }
      }
      __syncthreads();
      bwd_stages<T, 2, N, Q>(C, F0, F1, U, sB, t, TPE);
      __syncthreads();
      T mreg[PPT];
      const T* gb = a.jg + (size_t)ee * 4 * (a.deformed ? NQ : 1);
#pragma unroll
      for (int rr = 0; rr < PPT; ++rr) {
        const int pnt = t + rr * TPE;
        if (pnt < NQ) {
          const int i = pnt % Q, j = pnt / Q;
          T g0 = 0, g1 = 0;
#pragma unroll
          for (int c = 0; c < Q; ++c) {
            g0 = fma(sD[c * Q + i], U[pnt + (c - i)], g0);
            g1 = fma(sD[c * Q + j], U[pnt + (c - j) * Q], g1);
          }
          T jw, m0, m1, m2;
          if (a.deformed) {
            jw = gb[pnt];
            m0 = gb[NQ + pnt];
            m1 = gb[2 * NQ + pnt];
            m2 = gb[3 * NQ + pnt];
          } else {
            const T wp = wprod<T, 2, Q>(sw, pnt);
            jw = gb[0] * wp;
            m0 = gb[1] * wp;
            m1 = gb[2] * wp;
            m2 = gb[3] * wp;
          }
          F0[pnt] = fma(m0, g0, m1 * g1);
          F1[pnt] = fma(m1, g0, m2 * g1);
          mreg[rr] = lambda * jw * U[pnt];
        }
      }
      __syncthreads();
#pragma unroll
      for (int rr = 0; rr < PPT; ++rr) {
        const int pnt = t + rr * TPE;
        if (pnt < NQ) {
          const int i = pnt % Q, j = pnt / Q;
          T v = mreg[rr];
#pragma unroll
          for (int c = 0; c < Q; ++c) {
            v = fma(sD[i * Q + c], F0[pnt + (c - i)], v);
            v = fma(sD[j * Q + c], F1[pnt + (c - j) * Q], v);
          }
          U[pnt] = v;
        }
      }
      __syncthreads();
      ipr_stages<T, 2, N, Q>(U, F0, F1, C, sBt, t, TPE);
      __syncthreads();
      if (active) {
#pragma unroll
        for (int j = 0; j < MPT; ++j) {
          const int m = t + j * TPE;
          if (m < NM) {
            const int code = a.l2g[(size_t)e * NM + m];
            const int oc = a.ocode[(size_t)e * NM + m];
            const T sv = code >= 0 ? C[m] : -C[m];
            if (oc >= 0 && (oc & kOwnedBit))
              a.s[oc & (kOwnedBit - 1)] = sv;
            else if (oc >= 0)
              a.yslot[oc] = sv;
            sw_loc = fma(C[m], wv[j], sw_loc);  // y.(P w): unsigned value, signed input
          }
        }
      }
    }
    T v1[1] = {sw_loc};
    cta_partials<T, 1>(v1, a.part + 3 * G, G, sh);  // slot 3 s.w
  };

  // ---- phase B: assemble this thread's non-owned rows and update its rows ----
  auto phase_b = [&](T alpha, T beta, int parity) {
    T rw = 0, rrs = 0;
#pragma unroll
    for (int k = 0; k < RC; ++k) {
      if (k < nrows) {
        const int c = rc[k], i = ri[k];
        T sg;
        if (c == 0) {
          sg = __ldcg(a.s + rg[k]);  // owned row, written in phase A (maybe by another CTA)
        } else if (c < kAsmK) {
          const int n = P.n[c];
          const T* Y = a.yslot + P.col_off[c];
          sg = __ldcg(Y + i);
          for (int j = 1; j <= c; ++j) sg += __ldcg(Y + (size_t)j * n + i);
        } else {
          const T* Y = a.yslot + P.tail_off;
          sg = 0;
          for (int j = a.tail_ptr[i]; j < a.tail_ptr[i + 1]; ++j) sg += __ldcg(Y + j);
        }
        pr[k] = fma(beta, pr[k], wr[k]);
        qr[k] = fma(beta, qr[k], sg);
        xr[k] = fma(alpha, pr[k], xr[k]);
        rr_[k] = fma(-alpha, qr[k], rr_[k]);
        wr[k] = dr[k] * rr_[k];
        a.w[rg[k]] = wr[k];
        rw = fma(rr_[k], wr[k], rw);
        rrs = fma(rr_[k], rr_[k], rrs);
      }
    }
    T v[2] = {rw, rrs};
    cta_partials<T, 2>(v, a.part + (parity ? 4 : 0) * G, G, sh);  // slots 0, 1 or 4, 5: r.w, r.r
  };

  // Every CTA's copy of the recurrence's scalars, in shared memory: thread 0 updates it
  // (FP64 divisions by every thread cost microseconds here), the others read it.
  struct State {
    double rho, alpha, beta, mu, eps, rhs_mag;
    int iters, k, done, status;
  };
  __shared__ State st;
  if (tid == 0) st = State{0, 0, 0, 0, 0, 1, 0, 0, 0, ITHACA_GPU_OK};
  // Test hooks (zero in a solve): a shorter barrier wait, one CTA that never arrives,
  // and a pause of some CTAs right after each barrier, which lets the others run ahead.
  const long long polls = a.dbg_polls > 0 ? a.dbg_polls : kBarrierPolls;
  const bool drop = a.dbg_drop_cta == (int)blockIdx.x;
  auto lag = [&]() {
    if (a.dbg_delay_ns > 0 && blockIdx.x % 3 == 1) __nanosleep(a.dbg_delay_ns);
  };
  // r.w and r.r alternate between slots {0, 1} and {4, 5} from one iteration to the
  // next: a CTA that leaves the second barrier early writes its next phase-B partials
  // while slower CTAs may still be summing this iteration's, and the parity keeps the two
  // apart. The writes of the iteration after next come behind two more barriers, which
  // every CTA reaches only after its sums.
  int parity = 0;
  bool ok = grid_barrier(a.bar, a.err, polls, drop);  // also publishes st to the CTA
  if (ok) {
    phase_a();
    ok = grid_barrier(a.bar, a.err, polls);
  }
  if (ok) {  // the reference's initial step
    lag();
    double red[4];
    sum_partials<4>(a.part, {0, 1, 2, 3}, G, red, sh);
    if (tid == 0) {
      const double rw = red[0], rrs = red[1], bb = red[2], swv = red[3];
      st.rhs_mag = in.mag_override > 0 ? in.mag_override : (bb > 1e-6 ? bb : 1.0);
      st.eps = rrs;
      if (!isfinite(rrs) || !isfinite(rw) || !isfinite(swv)) {
        st.status = ITHACA_GPU_ERR_NUMERIC;
        st.done = 1;
      } else if (rrs < in.tol2 * st.rhs_mag) {
        st.done = 1;
      } else {
        st.rho = rw;
        st.mu = swv;
        st.beta = 0.0;
        st.alpha = rw / swv;
        st.iters = 1;
        if (in.max_iter <= 0) {
          st.status = ITHACA_GPU_ERR_NOT_CONVERGED;
          st.done = 1;
        }
      }
    }
    __syncthreads();
  }
  while (ok && !st.done) {
    parity ^= 1;
    phase_b((T)st.alpha, (T)st.beta, parity);
    ok = grid_barrier(a.bar, a.err, polls);
    if (!ok) break;
    phase_a();
    ok = grid_barrier(a.bar, a.err, polls);
    if (!ok) break;
    lag();
    // the reference loop tail: r.w, r.r (phase B, this parity's slots), 3 s.w (phase A)
    double red[4];
    if (parity)
      sum_partials<4>(a.part, {4, 5, 2, 3}, G, red, sh);
    else
      sum_partials<4>(a.part, {0, 1, 2, 3}, G, red, sh);
    if (tid == 0) {
      const double rho_new = red[0];
      st.eps = red[1];
      st.mu = red[3];
      st.iters += 1;
      if (!isfinite(st.eps) || !isfinite(rho_new) || !isfinite(st.mu)) {
        st.status = ITHACA_GPU_ERR_NUMERIC;
        st.done = 1;
      } else if (st.eps < in.tol2 * st.rhs_mag) {
        st.done = 1;
      } else {
        const double bnew = rho_new / st.rho;
        st.alpha = rho_new / (st.mu - rho_new * bnew / st.alpha);
        st.beta = bnew;
        st.rho = rho_new;
        st.k += 1;
        if (st.k >= in.max_iter) {
          st.status = ITHACA_GPU_ERR_NOT_CONVERGED;
          st.done = 1;
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < RC; ++k)
    if (k < nrows) a.x[rg[k]] = xr[k];
  if (blockIdx.x == 0 && tid == 0) {
    CgScalars o = in;
    o.alpha = st.alpha;
    o.beta = st.beta;
    o.rho = st.rho;
    o.mu = st.mu;
    o.eps = st.eps;
    o.rhs_mag = st.rhs_mag;
    o.iters = st.iters;
    o.k = st.k;
    o.done = 1;
    o.status = ok ? st.status : ITHACA_GPU_ERR_TIMEOUT;
    *a.sc = o;
  }
}

template <typename T, int N, int Q>
static bool persist_nq(const PersistArgs<T>& a, int sms, cudaStream_t s) {
  using L = Layout<T, 2, N, Q>;
  using Sh = Shape<2, Q>;
  auto k = cg2_persist_kernel<T, N, Q>;
  const size_t smem = L::bytes(Sh::EB);
  static int per_sm = -1;
  if (per_sm < 0) {
    ITHACA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ITHACA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, PT, smem));
  }
  if (per_sm < 1) return false;
  const int ngroups = (a.E + Sh::EB - 1) / Sh::EB;
  const int rows = (a.N + PT - 1) / PT;
  // at most PT CTAs (one partial per thread in the scalar sums), all co-resident
  const int G = std::max(1, std::min({PT, sms * per_sm, std::max(ngroups, rows)}));
  if ((long long)(a.N - a.ndir) > (long long)RC * G * PT) return false;  // rows must fit the registers
  ITHACA_CUDA(cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned), s));
  PersistArgs<T> args = a;
  void* params[] = {&args};
  ITHACA_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k), dim3(G), dim3(Sh::TPE, Sh::EB), params,
                                          smem, s));
  return true;
}

}  // namespace dev

template <typename T>
bool launch_cg2_persistent(int n, int Q, const PersistArgs<T>& a, int sms, cudaStream_t s) {
  if (Q != n + 1) return false;
  switch (n) {
#define ITHACA_PERSIST_CASE(NN) \
  case NN:                      \
    return dev::persist_nq<T, NN, NN + 1>(a, sms, s);
    ITHACA_PERSIST_CASE(2)
    ITHACA_PERSIST_CASE(3)
    ITHACA_PERSIST_CASE(4)
    ITHACA_PERSIST_CASE(5)
    ITHACA_PERSIST_CASE(6)
    ITHACA_PERSIST_CASE(7)
    ITHACA_PERSIST_CASE(8)
    ITHACA_PERSIST_CASE(9)
    ITHACA_PERSIST_CASE(10)
#undef ITHACA_PERSIST_CASE
    default:
      return false;
  }
}

template bool launch_cg2_persistent<float>(int, int, const PersistArgs<float>&, int, cudaStream_t);
template bool launch_cg2_persistent<double>(int, int, const PersistArgs<double>&, int, cudaStream_t);

}  // namespace ithaca
