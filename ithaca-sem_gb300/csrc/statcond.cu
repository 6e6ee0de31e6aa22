// Statically condensed C0 Helmholtz solve: the reference's IterativeStaticCond global
// system (MultiRegions/GlobalLinSysIterativeStaticCond.cpp, GlobalLinSysStaticCond.cpp).
//
// Per element, the dense Helmholtz matrix is split into boundary (vertex, edge, face)
// and interior modes, A = [A_bb A_bi; A_ib A_ii], and condensed:
//   S = A_bb - A_bi A_ii^-1 A_ib (m_schurCompl), BinvD = A_bi A_ii^-1 (m_BinvD),
//   C = A_ib (m_C), invD = A_ii^-1 (m_invD).
// The element matrices are the library's own matrix-free element operator applied to
// every unit mode (so they are exactly the operator the full solver iterates with); the
// condensation is a Gauss-Jordan inverse of the SPD interior block per element. The
// boundary system is solved by the reference CG recurrence (NekLinSysIterCG.cpp:104-263)
// with the diagonal of the assembled Schur complement as Jacobi preconditioner
// (PreconditionerDiagonal::StaticCondDiagonalPreconditionerSum,
// PreconditionerDiagonal.cpp:164-189); its operator is GlobalToLocalBnd, the element
// Schur complements, AssembleBnd (v_DoMatrixMultiply, GlobalLinSysIterativeStaticCond.cpp:392-424).
// The solve follows GlobalLinSysStaticCond::v_Solve (GlobalLinSysStaticCond.cpp:104-238),
// and the CG's rhs magnitude is set as v_PreSolve sets it (:431-460).
//
// Layouts: element blocks contiguous per element; S (nb x nb, symmetric, so row i of a
// column-major block is read with unit stride by consecutive threads), BinvD (nb x ni,
// row-major), C (ni x nb, row-major), invD (ni x ni, row-major). Boundary vectors are
// compacted global ids of the boundary modes, Dirichlet ids first.
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <algorithm>

#include "ithaca_internal.h"

namespace ithaca {
namespace sc {

constexpr int BT = 256;   // threads per CTA of the vector kernels
constexpr int WPB = 4;    // warps (elements) per CTA of the element kernels
constexpr double kUnset = -9999.0;  // NekConstants::kNekUnsetDouble
constexpr int kMaxInterior = 512;   // interior modes per element (8^3: hexes up to 10 modes)

struct Scal {
  double alpha, beta, rho, mu, eps, rhs_mag, tol2;
  int iters, k, done, status, max_iter, pad;
};

// ---- setup kernels ----------------------------------------------------------------
// u[e*nm + m] = (m == j)
__global__ void unit_kernel(size_t n, int nm, int j, double* u) {
  for (size_t i = (size_t)blockIdx.x * BT + threadIdx.x; i < n; i += (size_t)gridDim.x * BT)
    u[i] = (int)(i % nm) == j ? 1.0 : 0.0;
}

// A[e][i][j] = col[e*nm + i] (row-major element matrices)
__global__ void column_kernel(size_t n, int nm, int j, const double* col, double* A) {
  for (size_t t = (size_t)blockIdx.x * BT + threadIdx.x; t < n; t += (size_t)gridDim.x * BT) {
    const size_t e = t / nm, i = t % nm;
    A[(e * nm + i) * nm + j] = col[t];
  }
}

// One CTA per element: Gauss-Jordan inverse of A_ii (SPD: no pivoting) in the work block
// [A_ii | I] (ni x 2 ni), then BinvD = A_bi invD, S = A_bb - BinvD A_ib, C = A_ib. A
// non-positive pivot sets *bad (the element matrix is not SPD).
__global__ void __launch_bounds__(BT) condense_kernel(int nm, int nb, int ni, const int* __restrict__ bm,
                                                      const int* __restrict__ im, const double* __restrict__ A,
                                                      double* __restrict__ work, double* __restrict__ S,
                                                      double* __restrict__ BinvD, double* __restrict__ C,
                                                      double* __restrict__ invD, int* bad) {
  const int e = blockIdx.x;
  const double* Ae = A + (size_t)e * nm * nm;
  double* W = work + (size_t)e * ni * 2 * ni;
  const int w2 = 2 * ni;
  for (int t = threadIdx.x; t < ni * w2; t += blockDim.x) {
    const int r = t / w2, c = t % w2;
    W[t] = c < ni ? Ae[im[r] * nm + im[c]] : (c - ni == r ? 1.0 : 0.0);
  }
  __syncthreads();
  __shared__ double piv;
  __shared__ double fac[kMaxInterior];  // column k before the elimination step
  for (int k = 0; k < ni; ++k) {
    if (threadIdx.x == 0) {
      piv = W[k * w2 + k];
      if (!(piv > 0.0)) {
        atomicExch(bad, 1);
        piv = 1.0;
      }
    }
    __syncthreads();
    const double inv = 1.0 / piv;
    for (int c = threadIdx.x; c < w2; c += blockDim.x) W[k * w2 + c] *= inv;
    for (int r = threadIdx.x; r < ni; r += blockDim.x) fac[r] = r == k ? 0.0 : W[r * w2 + k];
    __syncthreads();
    for (int t = threadIdx.x; t < ni * w2; t += blockDim.x) {
      const int r = t / w2, c = t % w2;
      if (r != k) W[t] -= fac[r] * W[k * w2 + c];
    }
    __syncthreads();
  }
  double* De = invD + (size_t)e * ni * ni;
  for (int t = threadIdx.x; t < ni * ni; t += blockDim.x) De[t] = W[(t / ni) * w2 + ni + t % ni];
  __syncthreads();
  double* Be = BinvD + (size_t)e * nb * ni;
  for (int t = threadIdx.x; t < nb * ni; t += blockDim.x) {
    const int r = t / ni, c = t % ni;
    double v = 0;
    for (int k = 0; k < ni; ++k) v = fma(Ae[bm[r] * nm + im[k]], De[k * ni + c], v);
    Be[t] = v;
  }
  double* Ce = C + (size_t)e * ni * nb;
  for (int t = threadIdx.x; t < ni * nb; t += blockDim.x) Ce[t] = Ae[im[t / nb] * nm + bm[t % nb]];
  __syncthreads();
  double* Se = S + (size_t)e * nb * nb;  // column-major: entry (r, c) at c * nb + r
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    double v = Ae[bm[r] * nm + bm[c]];
    for (int k = 0; k < ni; ++k) v = fma(-Be[r * ni + k], Ae[im[k] * nm + bm[c]], v);
    Se[c * nb + r] = v;
  }
}

// ---- solve kernels ------------------------------------------------------------------
// out[e*nb + k] = in[e*nm + modes[k]] (nk modes per element)
__global__ void pick_kernel(size_t n, int nm, int nk, const int* __restrict__ modes, const double* __restrict__ in,
                            double* __restrict__ out) {
  for (size_t t = (size_t)blockIdx.x * BT + threadIdx.x; t < n; t += (size_t)gridDim.x * BT)
    out[t] = in[(t / nk) * nm + modes[t % nk]];
}

// out[e*nm + modes[k]] = in[e*nk + k]
__global__ void place_kernel(size_t n, int nm, int nk, const int* __restrict__ modes, const double* __restrict__ in,
                             double* __restrict__ out) {
  for (size_t t = (size_t)blockIdx.x * BT + threadIdx.x; t < n; t += (size_t)gridDim.x * BT)
    out[(t / nk) * nm + modes[t % nk]] = in[t];
}

// One warp per element: y_e (+)= sgn * M_e x_e for an nr x nc block M_e, row-major, or
// column-major when colmajor (then consecutive lanes read consecutive entries), with x_e
// either local (xl[e*nc + j]) or gathered from a global boundary vector through the
// signed codes (global ids < ndir read as zero).
__global__ void __launch_bounds__(WPB * 32) block_mv_kernel(int E, int nr, int nc, int colmajor,
                                                            const double* __restrict__ M,
                                                            const double* __restrict__ xl,
                                                            const int* __restrict__ code,
                                                            const double* __restrict__ xg, int ndir,
                                                            double sgn, int accumulate, double* __restrict__ y) {
  extern __shared__ double xs[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * WPB + warp;
  double* x = xs + warp * nc;
  if (e < E) {
    for (int j = lane; j < nc; j += 32) {
      double v;
      if (code != nullptr) {
        const int c = code[(size_t)e * nc + j];
        const int g = c >= 0 ? c : ~c;
        v = g < ndir ? 0.0 : xg[g];
        v = c >= 0 ? v : -v;
      } else {
        v = xl[(size_t)e * nc + j];
      }
      x[j] = v;
    }
  }
  __syncwarp();
  if (e >= E) return;
  const double* Me = M + (size_t)e * nr * nc;
  for (int i = lane; i < nr; i += 32) {
    double acc = 0;
    if (colmajor)
      for (int j = 0; j < nc; ++j) acc = fma(Me[(size_t)j * nr + i], x[j], acc);
    else
      for (int j = 0; j < nc; ++j) acc = fma(Me[(size_t)i * nc + j], x[j], acc);
    double* yi = y + (size_t)e * nr + i;
    *yi = accumulate ? *yi + sgn * acc : sgn * acc;
  }
}

// Per-CTA partial sums written to part[slot * gridDim.x + cta] (fixed order).
template <int NS>
__device__ __forceinline__ void cta_sums(double (&v)[NS], double* part, const int (&slot)[NS]) {
  __shared__ double sh[NS][BT / 32];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    double t = v[k];
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < NS) {
    double t = 0;
    for (int w = 0; w < BT / 32; ++w) t += sh[threadIdx.x][w];
    part[slot[threadIdx.x] * gridDim.x + blockIdx.x] = t;
  }
}

// out[g] = sum over the row's local entries of sign * yl (CSR of signed local indices);
// rows g >= row0. With w != nullptr, partial out.w over g >= ndir into slot 2.
__global__ void __launch_bounds__(BT) assemble_kernel(int N, int row0, const int* __restrict__ rowptr,
                                                      const int* __restrict__ cols, const double* __restrict__ yl,
                                                      double* __restrict__ out, const double* __restrict__ w,
                                                      int ndir, double* part, const Scal* sc) {
  if (sc != nullptr && sc->done) return;
  double v[1] = {0};
  for (int g = row0 + blockIdx.x * BT + threadIdx.x; g < N; g += gridDim.x * BT) {
    double acc = 0;
    for (int j = rowptr[g]; j < rowptr[g + 1]; ++j) {
      const int c = cols[j];
      acc += c >= 0 ? yl[c] : -yl[~c];
    }
    out[g] = acc;
    if (w != nullptr && g >= ndir) v[0] = fma(acc, w[g], v[0]);
  }
  if (part != nullptr) {
    const int slot[1] = {2};
    cta_sums<1>(v, part, slot);
  }
}

// CG initial step: x = 0, r = b, w = dinv r on the free dofs; partials r.w, r.r.
__global__ void __launch_bounds__(BT) init_kernel(int N, int ndir, const double* __restrict__ b,
                                                  double* __restrict__ x, double* __restrict__ r,
                                                  double* __restrict__ w, const double* __restrict__ dinv,
                                                  double* part) {
  double v[2] = {0, 0};
  for (int g = blockIdx.x * BT + threadIdx.x; g < N; g += gridDim.x * BT) {
    x[g] = 0.0;
    if (g < ndir) {
      r[g] = w[g] = 0.0;
      continue;
    }
    const double rg = b[g], wg = dinv[g] * rg;
    r[g] = rg;
    w[g] = wg;
    v[0] = fma(rg, wg, v[0]);
    v[1] = fma(rg, rg, v[1]);
  }
  const int slot[2] = {0, 1};
  cta_sums<2>(v, part, slot);
}

// p = beta p + w; q = beta q + s; x += alpha p; r -= alpha q; w = dinv r; partials r.w, r.r.
__global__ void __launch_bounds__(BT) update_kernel(int N, int ndir, const Scal* sc, double* __restrict__ x,
                                                    double* __restrict__ r, double* __restrict__ w,
                                                    const double* __restrict__ s, double* __restrict__ p,
                                                    double* __restrict__ q, const double* __restrict__ dinv,
                                                    double* part) {
  if (sc->done) return;
  const double alpha = sc->alpha, beta = sc->beta;
  double v[2] = {0, 0};
  for (int g = ndir + blockIdx.x * BT + threadIdx.x; g < N; g += gridDim.x * BT) {
    const double pg = fma(beta, p[g], w[g]), qg = fma(beta, q[g], s[g]);
    p[g] = pg;
    q[g] = qg;
    x[g] = fma(alpha, pg, x[g]);
    const double rg = fma(-alpha, qg, r[g]), wg = dinv[g] * rg;
    r[g] = rg;
    w[g] = wg;
    v[0] = fma(rg, wg, v[0]);
    v[1] = fma(rg, rg, v[1]);
  }
  const int slot[2] = {0, 1};
  cta_sums<2>(v, part, slot);
}

__device__ double sum_slot(const double* part, int slot, int n) {
  __shared__ double sh[BT / 32];
  double t = 0;
  for (int i = threadIdx.x; i < n; i += BT) t += part[slot * n + i];
  for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  double s = 0;
  for (int w = 0; w < BT / 32; ++w) s += sh[w];
  __syncthreads();
  return s;
}

// The recurrence's scalars (NekLinSysIterCG.cpp:147-261). first: the initial step.
__global__ void __launch_bounds__(BT) scalars_kernel(const double* part, int n, Scal* sc, int first) {
  if (sc->done) return;
  const double rw = sum_slot(part, 0, n), rr = sum_slot(part, 1, n), sw = sum_slot(part, 2, n);
  if (threadIdx.x != 0) return;
  Scal o = *sc;
  if (!isfinite(rw) || !isfinite(rr) || !isfinite(sw)) {
    o.status = ITHACA_GPU_ERR_NUMERIC;
    o.done = 1;
  } else if (first) {
    o.eps = rr;
    if (rr < o.tol2 * o.rhs_mag) {
      o.done = 1;
      o.iters = 0;
    } else {
      o.rho = rw;
      o.mu = sw;
      o.beta = 0.0;
      o.alpha = rw / sw;
      o.iters = 1;
      o.k = 0;
      if (o.max_iter <= 0) {
        o.status = ITHACA_GPU_ERR_NOT_CONVERGED;
        o.done = 1;
      }
    }
  } else {
    o.eps = rr;
    o.mu = sw;
    o.iters += 1;
    if (rr < o.tol2 * o.rhs_mag) {
      o.done = 1;
    } else {
      const double bnew = rw / o.rho;
      o.alpha = rw / (sw - rw * bnew / o.alpha);
      o.beta = bnew;
      o.rho = rw;
      o.k += 1;
      if (o.k >= o.max_iter) {
        o.status = ITHACA_GPU_ERR_NOT_CONVERGED;
        o.done = 1;
      }
    }
  }
  *sc = o;
}

// sum of squares of b over [0, N) into part slot 0 (the rhs magnitude)
__global__ void __launch_bounds__(BT) sumsq_kernel(int N, const double* __restrict__ b, double* part) {
  double v[1] = {0};
  for (int g = blockIdx.x * BT + threadIdx.x; g < N; g += gridDim.x * BT) v[0] = fma(b[g], b[g], v[0]);
  const int slot[1] = {0};
  cta_sums<1>(v, part, slot);
}

__global__ void __launch_bounds__(BT) reduce_kernel(const double* part, int n, double* out) {
  const double s = sum_slot(part, 0, n);
  if (threadIdx.x == 0) *out = s;
}

// vb[e*nb + k] += sign * pert[g] (GlobalToLocalBnd of the perturbation; Dirichlet ids add 0)
__global__ void add_g2l_kernel(size_t n, const int* __restrict__ code, const double* __restrict__ pert, int ndir,
                               double* __restrict__ vb) {
  for (size_t t = (size_t)blockIdx.x * BT + threadIdx.x; t < n; t += (size_t)gridDim.x * BT) {
    const int c = code[t];
    const int g = c >= 0 ? c : ~c;
    if (g < ndir) continue;
    vb[t] += c >= 0 ? pert[g] : -pert[g];
  }
}

__global__ void diag_local_kernel(size_t n, int nb, const double* __restrict__ S, double* __restrict__ d) {
  for (size_t t = (size_t)blockIdx.x * BT + threadIdx.x; t < n; t += (size_t)gridDim.x * BT) {
    const size_t e = t / nb, k = t % nb;
    d[t] = S[(e * nb + k) * nb + k];
  }
}

// assembled diagonal -> inverse on the free ids (sign^2 = 1, so the sum is unsigned)
__global__ void inv_free_kernel(int N, int ndir, const double* __restrict__ d, double* __restrict__ dinv) {
  for (int g = blockIdx.x * BT + threadIdx.x; g < N; g += gridDim.x * BT) dinv[g] = g >= ndir ? 1.0 / d[g] : 0.0;
}

}  // namespace sc

struct Sc {
  Op* op = nullptr;
  int dim = 0, n = 0, nm = 0, nb = 0, ni = 0, E = 0;
  int Nb = 0, ndir = 0;
  int *bmodes = nullptr, *imodes = nullptr;
  int* bcode = nullptr;    // E*nb signed global boundary ids
  int* rowptr = nullptr;   // Nb + 1
  int* cols = nullptr;     // E*nb signed local boundary entries (e*nb + k or ~(...))
  int* rowptr_abs = nullptr;  // the same rows with unsigned entries (diagonal assembly)
  int* cols_abs = nullptr;
  double lambda = NAN;
  double *S = nullptr, *BinvD = nullptr, *C = nullptr, *invD = nullptr;
  double *x = nullptr, *r = nullptr, *w = nullptr, *s = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr,
         *b = nullptr;
  double *fb = nullptr, *vb = nullptr, *yl = nullptr, *fi = nullptr, *vi = nullptr;
  double *part = nullptr, *dmag = nullptr;
  int grid = 1;
  sc::Scal *scal = nullptr, *scal_host = nullptr;
  int* bad = nullptr;
  double rhs_mag = sc::kUnset;
  ~Sc();
};

Sc::~Sc() {
  for (void* p0 : {(void*)bmodes, (void*)imodes, (void*)bcode, (void*)rowptr, (void*)cols, (void*)rowptr_abs,
                   (void*)cols_abs, (void*)S, (void*)BinvD, (void*)C, (void*)invD, (void*)x, (void*)r, (void*)w,
                   (void*)s, (void*)p, (void*)q, (void*)dinv, (void*)b, (void*)fb, (void*)vb, (void*)yl, (void*)fi,
                   (void*)vi, (void*)part, (void*)dmag, (void*)scal, (void*)bad})
    cudaFree(p0);
  if (scal_host) cudaFreeHost(scal_host);
  if (op) release_op(op);
}

static int blocks_for(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + sc::BT - 1) / sc::BT, (size_t)device_sm_count() * 8));
}

// Builds the condensed element blocks for `lambda` (once per lambda).
static void sc_build(Sc* c, double lambda) {
  if (c->lambda == lambda) return;
  using namespace sc;
  Op* op = c->op;
  cudaStream_t s = op->ctx->stream;
  const int nm = c->nm, nb = c->nb, ni = c->ni;
  const size_t per_elem_jg = (size_t)n_jg(op->dim) * (op->deformed ? op->nq : 1);
  // element chunks sized so that the element matrices and the Gauss-Jordan work stay
  // within about 1 GB of scratch
  const size_t per_elem = (size_t)nm * nm + (size_t)ni * 2 * ni + 2 * (size_t)nm;
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(c->E, ((size_t)1 << 27) / per_elem));
  double *A = nullptr, *work = nullptr, *u = nullptr, *col = nullptr;
  ITHACA_CUDA(cudaMalloc(&A, sizeof(double) * chunk * nm * nm));
  ITHACA_CUDA(cudaMalloc(&work, sizeof(double) * chunk * std::max(1, ni * 2 * ni)));
  ITHACA_CUDA(cudaMalloc(&u, sizeof(double) * chunk * nm));
  ITHACA_CUDA(cudaMalloc(&col, sizeof(double) * chunk * nm));
  struct Free {
    std::vector<void*> v;
    ~Free() {
      for (void* p : v) cudaFree(p);
    }
  } fr{{A, work, u, col}};
  ITHACA_CUDA(cudaMemsetAsync(c->bad, 0, sizeof(int), s));
  for (int e0 = 0; e0 < c->E; e0 += chunk) {
    const int Ec = std::min(chunk, c->E - e0);
    const size_t nloc = (size_t)Ec * nm;
    for (int j = 0; j < nm; ++j) {
      unit_kernel<<<blocks_for(nloc), BT, 0, s>>>(nloc, nm, j, u);
      if (!launch_helmholtz<double>(op->kdim, op->n, op->Q, Ec, op->deformed, op->t64.base,
                                    op->jg64 + (size_t)e0 * per_elem_jg, lambda, u, col, nullptr, 0, s))
        fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz: (modes, points) combination not built");
      column_kernel<<<blocks_for(nloc), BT, 0, s>>>(nloc, nm, j, col, A);
    }
    condense_kernel<<<Ec, BT, 0, s>>>(nm, nb, ni, c->bmodes, c->imodes, A, work, c->S + (size_t)e0 * nb * nb,
                                      c->BinvD + (size_t)e0 * nb * ni, c->C + (size_t)e0 * ni * nb,
                                      c->invD + (size_t)e0 * ni * ni, c->bad);
    op->ctx->launches += 3LL * nm + 1;
  }
  // Jacobi preconditioner: assembled diagonal of the Schur complements
  const size_t nlb = (size_t)c->E * nb;
  diag_local_kernel<<<blocks_for(nlb), BT, 0, s>>>(nlb, nb, c->S, c->yl);
  assemble_kernel<<<blocks_for(c->Nb), BT, 0, s>>>(c->Nb, 0, c->rowptr_abs, c->cols_abs, c->yl, c->s, nullptr, 0,
                                                   nullptr, nullptr);
  inv_free_kernel<<<blocks_for(c->Nb), BT, 0, s>>>(c->Nb, c->ndir, c->s, c->dinv);
  op->ctx->launches += 3;
  int hbad = 0;
  ITHACA_CUDA(cudaMemcpyAsync(&hbad, c->bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  ITHACA_CUDA(cudaStreamSynchronize(s));
  if (hbad) fail(ITHACA_GPU_ERR_NUMERIC, "an element's interior block is not positive definite");
  c->lambda = lambda;
}

// GlobalLinSysStaticCond::v_Solve on device arrays: F (E*nm local forcing), V (E*nm: the
// boundary values already present -- Dirichlet data, initial guess -- in; solution out).
static void sc_solve_impl(Sc* c, double lambda, const double* F, double* V, const ithaca_gpu_cg_opts& o,
                          ithaca_gpu_cg_result* res) {
  using namespace sc;
  if (o.mode != ITHACA_GPU_SOLVE_FP64)
    fail(ITHACA_GPU_ERR_UNSUPPORTED, "the statically condensed solve runs in FP64 mode only");
  sc_build(c, lambda);
  Op* op = c->op;
  Ctx* ctx = op->ctx;
  cudaStream_t s = ctx->stream;
  const int nm = c->nm, nb = c->nb, ni = c->ni, E = c->E, Nb = c->Nb, nd = c->ndir;
  const size_t nlb = (size_t)E * nb, nli = (size_t)E * ni;
  const dim3 eg((E + WPB - 1) / WPB);
  const size_t smem_b = sizeof(double) * WPB * nb, smem_i = sizeof(double) * WPB * std::max(ni, 1);
  pick_kernel<<<blocks_for(nlb), BT, 0, s>>>(nlb, nm, nb, c->bmodes, F, c->fb);
  pick_kernel<<<blocks_for(nlb), BT, 0, s>>>(nlb, nm, nb, c->bmodes, V, c->vb);
  if (ni > 0) pick_kernel<<<blocks_for(nli), BT, 0, s>>>(nli, nm, ni, c->imodes, F, c->fi);
  // v_PreSolve: rhs magnitude from the assembled boundary forcing before condensation,
  // smoothed with the previous solve's (GlobalLinSysIterative::Set_Rhs_Magnitude)
  assemble_kernel<<<blocks_for(Nb), BT, 0, s>>>(Nb, 0, c->rowptr, c->cols, c->fb, c->b, nullptr, 0, nullptr, nullptr);
  sumsq_kernel<<<c->grid, BT, 0, s>>>(Nb, c->b, c->part);
  reduce_kernel<<<1, BT, 0, s>>>(c->part, c->grid, c->dmag);
  // F_bnd -= BinvD F_int; F_bnd -= S V_bnd; b = AssembleBnd(F_bnd)
  if (ni > 0)
    block_mv_kernel<<<eg, WPB * 32, smem_i, s>>>(E, nb, ni, 0, c->BinvD, c->fi, nullptr, nullptr, 0, -1.0, 1, c->fb);
  block_mv_kernel<<<eg, WPB * 32, smem_b, s>>>(E, nb, nb, 1, c->S, c->vb, nullptr, nullptr, 0, -1.0, 1, c->fb);
  assemble_kernel<<<blocks_for(Nb), BT, 0, s>>>(Nb, 0, c->rowptr, c->cols, c->fb, c->b, nullptr, 0, nullptr, nullptr);
  ctx->launches += 9;
  double mag = 0;
  ITHACA_CUDA(cudaMemcpyAsync(&mag, c->dmag, sizeof(double), cudaMemcpyDeviceToHost, s));
  ITHACA_CUDA(cudaStreamSynchronize(s));
  const double new_mag = mag > 1e-6 ? mag : 1.0;
  c->rhs_mag = c->rhs_mag == kUnset ? new_mag : 0.9 * c->rhs_mag + 0.1 * new_mag;
  // CG on the boundary system for the perturbation from V_bnd
  Scal init{};
  init.tol2 = std::max(o.tol, 1e-16) * std::max(o.tol, 1e-16);
  init.rhs_mag = c->rhs_mag;
  init.max_iter = o.max_iter;
  *c->scal_host = init;
  ITHACA_CUDA(cudaMemcpyAsync(c->scal, c->scal_host, sizeof(Scal), cudaMemcpyHostToDevice, s));
  auto op_apply = [&](const double* xin, double* yout, const double* wdot) {
    block_mv_kernel<<<eg, WPB * 32, smem_b, s>>>(E, nb, nb, 1, c->S, nullptr, c->bcode, xin, nd, 1.0, 0, c->yl);
    assemble_kernel<<<c->grid, BT, 0, s>>>(Nb, 0, c->rowptr, c->cols, c->yl, yout, wdot, nd, c->part,
                                           wdot ? c->scal : nullptr);
    ctx->launches += 2;
  };
  init_kernel<<<c->grid, BT, 0, s>>>(Nb, nd, c->b, c->x, c->r, c->w, c->dinv, c->part);
  op_apply(c->w, c->s, c->w);
  scalars_kernel<<<1, BT, 0, s>>>(c->part, c->grid, c->scal, 1);
  ctx->launches += 2;
  const int chunk = std::max(1, std::min(o.check_every, 64));
  const long long max_checks = (long long)o.max_iter / chunk + 2;
  for (long long it = 0;; ++it) {
    ITHACA_CUDA(cudaMemcpyAsync(c->scal_host, c->scal, sizeof(Scal), cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaStreamSynchronize(s));
    if (c->scal_host->done) break;
    if (it >= max_checks) fail(ITHACA_GPU_ERR_TIMEOUT, "CG did not flag completion within its iteration bound");
    for (int k = 0; k < chunk; ++k) {
      update_kernel<<<c->grid, BT, 0, s>>>(Nb, nd, c->scal, c->x, c->r, c->w, c->s, c->p, c->q, c->dinv, c->part);
      op_apply(c->w, c->s, c->w);
      scalars_kernel<<<1, BT, 0, s>>>(c->part, c->grid, c->scal, 0);
      ctx->launches += 2;
    }
  }
  const Scal fin = *c->scal_host;
  // V_bnd += GlobalToLocalBnd(pert); V_int = invD (F_int - C V_bnd)
  add_g2l_kernel<<<blocks_for(nlb), BT, 0, s>>>(nlb, c->bcode, c->x, nd, c->vb);
  place_kernel<<<blocks_for(nlb), BT, 0, s>>>(nlb, nm, nb, c->bmodes, c->vb, V);
  if (ni > 0) {
    block_mv_kernel<<<eg, WPB * 32, smem_b, s>>>(E, ni, nb, 0, c->C, c->vb, nullptr, nullptr, 0, -1.0, 1, c->fi);
    block_mv_kernel<<<eg, WPB * 32, smem_i, s>>>(E, ni, ni, 0, c->invD, c->fi, nullptr, nullptr, 0, 1.0, 0, c->vi);
    place_kernel<<<blocks_for(nli), BT, 0, s>>>(nli, nm, ni, c->imodes, c->vi, V);
  }
  ctx->launches += 5;
  ITHACA_CUDA(cudaGetLastError());
  ITHACA_CUDA(cudaStreamSynchronize(s));
  if (res) {
    ithaca_gpu_cg_result r{};
    r.iterations = fin.iters;
    r.eps = fin.eps;
    r.rhs_magnitude = fin.rhs_mag;
    r.rel_residual = std::sqrt(fin.eps / fin.rhs_mag);
    *res = r;
  }
  ctx->check_device_error();
  if (fin.status == ITHACA_GPU_ERR_NOT_CONVERGED)
    fail(fin.status, "Exceeded maximum number of iterations (" + std::to_string(fin.iters) + ")");
  if (fin.status != ITHACA_GPU_OK) fail(fin.status, "NaN or Inf in the CG recurrence");
}

}  // namespace ithaca

using namespace ithaca;

struct ithaca_gpu_sc : public Sc {};

template <typename F>
static int sc_guarded(F f) {
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

static void sreq(bool ok, const char* msg) {
  if (!ok) fail(ITHACA_GPU_ERR_ARG, msg);
}

extern "C" {

int ithaca_gpu_sc_create(ithaca_gpu_op* opp, const int* l2g, const double* sign, int nglobal, int ndir,
                         ithaca_gpu_sc** out) {
  return sc_guarded([&] {
    Op* op = reinterpret_cast<Op*>(opp);
    sreq(op && l2g && sign && out, "null argument");
    sreq(op->precision == ITHACA_GPU_FP64, "the global system needs an FP64 operator");
    sreq(op->deformed != 0, "the statically condensed solve takes a deformed (per-point) collection");
    sreq(nglobal > 0 && ndir >= 0 && ndir <= nglobal, "bad nglobal / ndir");
    const int dim = op->dim, n = op->n, nm = op->nm, E = op->E;
    std::vector<int> bm, im;
    for (int m = 0, tp = 0, tq = 0; m < nm; ++m) {
      if (op->shape == ITHACA_GPU_SHAPE_PYR) {
        // pyramid mode m(p, q, r): interior when p >= 2, q >= 2 and r >= 1
        int pp = 0, qq = 0, rest = m;
        while (rest >= n - std::max(pp, qq)) {
          rest -= n - std::max(pp, qq);
          if (++qq == n) {
            qq = 0;
            ++pp;
          }
        }
        (pp >= 2 && qq >= 2 && rest >= 1 ? im : bm).push_back(m);
        continue;
      }
      if (op->shape == ITHACA_GPU_SHAPE_PRISM) {
        // prism mode m(p, q, r): interior when p >= 2, q >= 2 and r >= 1
        int pp = 0, rest = m;
        while (rest >= n * (n - pp)) {
          rest -= n * (n - pp);
          ++pp;
        }
        const int qq = rest / (n - pp), rr = rest % (n - pp);
        (pp >= 2 && qq >= 2 && rr >= 1 ? im : bm).push_back(m);
        continue;
      }
      if (op->shape == ITHACA_GPU_SHAPE_TET) {
        // tetrahedron mode m(p, q, r): interior when p >= 2, q >= 1 and r >= 1
        int tp_ = 0, rest = m;
        while (rest >= (n - tp_) * (n - tp_ + 1) / 2) {
          rest -= (n - tp_) * (n - tp_ + 1) / 2;
          ++tp_;
        }
        int tq_ = 0;
        while (rest >= n - tp_ - tq_) {
          rest -= n - tp_ - tq_;
          ++tq_;
        }
        (tp_ >= 2 && tq_ >= 1 && rest >= 1 ? im : bm).push_back(m);
        continue;
      }
      if (op->shape == ITHACA_GPU_SHAPE_TRI) {
        // triangle mode m(tp, tq): vertices and edges are the rows tp <= 1 and the modes tq == 0
        (tp <= 1 || tq == 0 ? bm : im).push_back(m);
        if (++tq == n - tp) {
          tq = 0;
          ++tp;
        }
        continue;
      }
      const int p = m % n, q = (m / n) % n, r = dim == 3 ? m / (n * n) : n;
      (p < 2 || q < 2 || (dim == 3 && r < 2) ? bm : im).push_back(m);
    }
    const int nb = (int)bm.size(), ni = (int)im.size();
    sreq(ni <= sc::kMaxInterior, "too many interior modes per element");
    // compacted global boundary ids (the Dirichlet ids, numbered first, stay first)
    std::vector<int> bid(nglobal, -1);
    std::vector<char> isint(nglobal, 0), isbnd(nglobal, 0);
    for (int e = 0; e < E; ++e) {
      for (int k = 0; k < nb; ++k) {
        const size_t l = (size_t)e * nm + bm[k];
        sreq(l2g[l] >= 0 && l2g[l] < nglobal, "l2g entry out of range");
        sreq(sign[l] == 1.0 || sign[l] == -1.0, "sign entries must be +1 or -1");
        isbnd[l2g[l]] = 1;
      }
      for (int k = 0; k < ni; ++k) {
        const size_t l = (size_t)e * nm + im[k];
        sreq(l2g[l] >= 0 && l2g[l] < nglobal, "l2g entry out of range");
        isint[l2g[l]] = 1;
      }
    }
    int Nb = 0, nd = 0;
    for (int g = 0; g < nglobal; ++g) {
      sreq(!(isint[g] && isbnd[g]), "a global dof is both an interior and a boundary mode");
      if (isbnd[g]) {
        bid[g] = Nb++;
        nd += g < ndir;
      } else {
        sreq(g >= ndir, "a Dirichlet dof is not a boundary mode");
      }
    }
    std::vector<int> code((size_t)E * nb), cnt(Nb + 1, 0);
    for (int e = 0; e < E; ++e)
      for (int k = 0; k < nb; ++k) {
        const size_t l = (size_t)e * nm + bm[k];
        const int g = bid[l2g[l]];
        code[(size_t)e * nb + k] = sign[l] > 0 ? g : ~g;
        cnt[g + 1]++;
      }
    for (int g = 0; g < Nb; ++g) cnt[g + 1] += cnt[g];
    std::vector<int> cols((size_t)E * nb), cols_abs((size_t)E * nb), fill(cnt.begin(), cnt.end() - 1);
    for (size_t t = 0; t < (size_t)E * nb; ++t) {
      const int c = code[t], g = c >= 0 ? c : ~c;
      const int pos = fill[g]++;
      cols[pos] = c >= 0 ? (int)t : ~(int)t;
      cols_abs[pos] = (int)t;
    }
    auto c = std::make_unique<ithaca_gpu_sc>();
    retain_op(op);
    c->op = op;
    c->dim = dim;
    c->n = n;
    c->nm = nm;
    c->nb = nb;
    c->ni = ni;
    c->E = E;
    c->Nb = Nb;
    c->ndir = nd;
    c->grid = std::max(1, std::min(device_sm_count() * 4, (Nb + sc::BT - 1) / sc::BT));
    auto up = [&](int** dst, const std::vector<int>& src) {
      ITHACA_CUDA(cudaMalloc(dst, sizeof(int) * std::max<size_t>(1, src.size())));
      if (!src.empty())
        ITHACA_CUDA(cudaMemcpy(*dst, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice));
    };
    up(&c->bmodes, bm);
    up(&c->imodes, im);
    up(&c->bcode, code);
    up(&c->rowptr, cnt);
    up(&c->cols, cols);
    up(&c->rowptr_abs, cnt);
    up(&c->cols_abs, cols_abs);
    auto dal = [&](double** dst, size_t cntd) { ITHACA_CUDA(cudaMalloc(dst, sizeof(double) * std::max<size_t>(1, cntd))); };
    dal(&c->S, (size_t)E * nb * nb);
    dal(&c->BinvD, (size_t)E * nb * ni);
    dal(&c->C, (size_t)E * ni * nb);
    dal(&c->invD, (size_t)E * ni * ni);
    for (double** v : {&c->x, &c->r, &c->w, &c->s, &c->p, &c->q, &c->dinv, &c->b}) {
      dal(v, Nb);
      ITHACA_CUDA(cudaMemset(*v, 0, sizeof(double) * Nb));
    }
    dal(&c->fb, (size_t)E * nb);
    dal(&c->vb, (size_t)E * nb);
    dal(&c->yl, (size_t)E * nb);
    dal(&c->fi, (size_t)E * ni);
    dal(&c->vi, (size_t)E * ni);
    dal(&c->part, (size_t)3 * c->grid);
    dal(&c->dmag, 1);
    ITHACA_CUDA(cudaMalloc(&c->scal, sizeof(sc::Scal)));
    ITHACA_CUDA(cudaMallocHost(&c->scal_host, sizeof(sc::Scal)));
    ITHACA_CUDA(cudaMalloc(&c->bad, sizeof(int)));
    *out = c.release();
  });
}

int ithaca_gpu_sc_destroy(ithaca_gpu_sc* c) {
  return sc_guarded([&] {
    if (!c) return;
    cudaStreamSynchronize(c->op->ctx->stream);
    delete c;
  });
}

int ithaca_gpu_sc_info(ithaca_gpu_sc* c, int* nbnd_global, int* ndir_bnd, int* nbnd_local, int* nint_local) {
  return sc_guarded([&] {
    sreq(c != nullptr, "null solver");
    if (nbnd_global) *nbnd_global = c->Nb;
    if (ndir_bnd) *ndir_bnd = c->ndir;
    if (nbnd_local) *nbnd_local = c->nb;
    if (nint_local) *nint_local = c->ni;
  });
}

int ithaca_gpu_sc_solve(ithaca_gpu_sc* c, double lambda, const double* loc_rhs, double* loc_inout,
                        const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device) {
  return sc_guarded([&] {
    sreq(c && loc_rhs && loc_inout, "null argument");
    StreamOrder order_(c->op->ctx);
    ithaca_gpu_cg_opts o;
    ithaca_gpu_cg_default_opts(&o);
    if (opts) o = *opts;
    if (o.max_iter <= 0) o.max_iter = 5000;
    Ctx* ctx = c->op->ctx;
    cudaStream_t s = ctx->stream;
    const size_t bytes = sizeof(double) * (size_t)c->E * c->nm;
    const double* F = loc_rhs;
    double* V = loc_inout;
    if (!on_device) {
      double* dF = (double*)ctx->stage_ptr(0, bytes);
      double* dV = (double*)ctx->stage_ptr(1, bytes);
      ITHACA_CUDA(cudaMemcpyAsync(dF, loc_rhs, bytes, cudaMemcpyHostToDevice, s));
      ITHACA_CUDA(cudaMemcpyAsync(dV, loc_inout, bytes, cudaMemcpyHostToDevice, s));
      F = dF;
      V = dV;
    }
    sc_solve_impl(c, lambda, F, V, o, res);
    if (!on_device) {
      ITHACA_CUDA(cudaMemcpyAsync(loc_inout, V, bytes, cudaMemcpyDeviceToHost, s));
      ITHACA_CUDA(cudaStreamSynchronize(s));
    }
  });
}

}  // extern "C"
