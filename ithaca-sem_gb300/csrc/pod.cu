// POD offline / online on the GPU (FP64 throughout).
//
// Offline (CoupledLinearNS_ROM::ROM_offline_phase, solvers/IncNavierStokesSolver/
// EquationSystems/CoupledLinearNS_ROM.cpp:3916-4001): the reference takes a thin SVD of
// the snapshot matrix S with Eigen's BDCSVD. Here the method of snapshots gives the same
// subspace: C = S^T S (FP64 split-K GEMM with a fixed-order reduction), C = W L W^T
// (cuSOLVER's symmetric divide-and-conquer eigen-solver, ns x ns, on the device),
// V = S W_r L_r^{-1/2}, then two
// Cholesky-QR passes restore orthonormality (the modes are re-orthogonalised as
// VelocityCorrectionScheme_iROM.cpp:830-852 does with Gram-Schmidt). Eigenvalues of
// S^T S far below the largest are not resolved in FP64 (a pass keeps those above 1e-10
// of its largest), so further passes repeat the procedure on the deflated snapshots
// S - V (V^T S) to reach the smaller modes.
// Projection (:3661-3663, :3904-3911): A_L = V^T L V and A_M = V^T M V with L and M
// applied matrix-free to the modes (the affine split of gen_affine_mat_proj :4694-4703).
// Online (ROM_online_phase :4003-4100): for each lambda, (A_L + lambda A_M) x = V^T b by
// LU with partial pivoting, one CTA per system (the reference uses colPivHouseholderQr
// at :4053; both are direct dense solves of the same system).
#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cusolverDn.h>

#include "ithaca_internal.h"

namespace ithaca {

// ---- FP64 GEMM: C[m + n*ldc] = sum_k op(A)(m,k) op(B)(k,n), column-major operands ----
// TRANS_A: A stored K x M (A[k + m*lda]); otherwise M x K (A[m + k*lda]). B is K x N.
// Split-K: blockIdx.z takes rows [z*kchunk, (z+1)*kchunk) and writes its own partial.
constexpr int GT = 64, GK = 16;

template <bool TRANS_A>
__global__ void __launch_bounds__(256) dgemm_kernel(int M, int Nn, int K, int kchunk, const double* __restrict__ A,
                                                    int lda, const double* __restrict__ B, int ldb,
                                                    double* __restrict__ C, size_t part_stride, int ldc) {
  __shared__ double As[GK][GT + 1];
  __shared__ double Bs[GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
  const int k0 = blockIdx.z * kchunk, k1 = min(K, k0 + kchunk);
  double acc[4][4] = {};
  for (int kb = k0; kb < k1; kb += GK) {
    for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
      int kk, mm;
      if (TRANS_A) {  // consecutive threads walk k (contiguous in A)
        kk = idx % GK;
        mm = idx / GK;
      } else {  // consecutive threads walk m (contiguous in A)
        mm = idx % GT;
        kk = idx / GT;
      }
      const int k = kb + kk, m = m0 + mm;
      double v = 0;
      if (k < k1 && m < M) v = TRANS_A ? A[(size_t)m * lda + k] : A[(size_t)k * lda + m];
      As[kk][mm] = v;
      const int kk2 = idx % GK, nn = idx / GK;
      const int k2 = kb + kk2, n = n0 + nn;
      Bs[kk2][nn] = (k2 < k1 && n < Nn) ? B[(size_t)n * ldb + k2] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* Cp = C + blockIdx.z * part_stride;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < Nn) Cp[(size_t)n * ldc + m] = acc[i][j];
    }
}

// C[i] = sum_z part[z][i] in order z = 0, 1, ... (deterministic split-K reduction).
__global__ void sum_parts_kernel(size_t n, int nparts, const double* __restrict__ part, size_t stride,
                                 double* __restrict__ C) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int z = 0; z < nparts; ++z) s += part[z * stride + i];
    C[i] = s;
  }
}

// Split count and chunk for a K-long reduction.
static void split_k(int K, int tiles, int* nsplit, int* kchunk) {
  const int target = std::max(1, (device_sm_count() * 4) / std::max(1, tiles));
  int ns = std::max(1, std::min(target, (K + 255) / 256));
  int kc = (K + ns - 1) / ns;
  kc = (kc + GK - 1) / GK * GK;
  ns = (K + kc - 1) / kc;
  *nsplit = ns;
  *kchunk = kc;
}

// C (M x Nn, ldc = M) = A^T B with A: K x M, B: K x Nn (column-major, lda = ldb = K).
// `scratch` must hold nsplit * M * Nn doubles (see tn_scratch_doubles).
size_t tn_scratch_doubles(int M, int Nn, int K) {
  int ns, kc;
  split_k(K, ((M + GT - 1) / GT) * ((Nn + GT - 1) / GT), &ns, &kc);
  return (size_t)ns * M * Nn;
}

void dgemm_tn(int M, int Nn, int K, const double* A, const double* B, double* C, double* scratch, cudaStream_t s,
              long long* launches) {
  int ns, kc;
  const dim3 grid((M + GT - 1) / GT, (Nn + GT - 1) / GT, 1);
  split_k(K, grid.x * grid.y, &ns, &kc);
  const size_t stride = (size_t)M * Nn;
  dgemm_kernel<true><<<dim3(grid.x, grid.y, ns), 256, 0, s>>>(M, Nn, K, kc, A, K, B, K, scratch, stride, M);
  sum_parts_kernel<<<std::min<size_t>((stride + 255) / 256, 1024), 256, 0, s>>>(stride, ns, scratch, stride, C);
  if (launches) *launches += 2;
}

// C (M x Nn) = A (M x K, lda = M) * B (K x Nn, ldb = K); no split (K is small).
void dgemm_nn(int M, int Nn, int K, const double* A, const double* B, double* C, cudaStream_t s,
              long long* launches) {
  const dim3 grid((M + GT - 1) / GT, (Nn + GT - 1) / GT, 1);
  dgemm_kernel<false><<<grid, 256, 0, s>>>(M, Nn, K, K, A, M, B, K, C, 0, M);
  if (launches) *launches += 1;
}

// Device scratch owned by one call.
struct DevBuf {
  double* p = nullptr;
  explicit DevBuf(size_t n) { ITHACA_CUDA(cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1))); }
  ~DevBuf() { cudaFree(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// ---- dense symmetric eigen-decomposition on the device (cuSOLVER syevd) ----
static void free_solver(void* h) { cusolverDnDestroy(static_cast<cusolverDnHandle_t>(h)); }

static cusolverDnHandle_t ctx_solver(Ctx* ctx) {
  if (!ctx->solver) {
    cusolverDnHandle_t h = nullptr;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) fail(ITHACA_GPU_ERR_CUDA, "cusolverDnCreate failed");
    ctx->solver = h;
    ctx->solver_free = free_solver;
  }
  auto h = static_cast<cusolverDnHandle_t>(ctx->solver);
  if (cusolverDnSetStream(h, ctx->stream) != CUSOLVER_STATUS_SUCCESS)
    fail(ITHACA_GPU_ERR_CUDA, "cusolverDnSetStream failed");
  return h;
}

// A (n x n, column-major, symmetric, device) -> eigenvectors in place (column j for
// eigenvalue ev[j], ascending); ev is returned on the host.
static void sym_eigen(Ctx* ctx, int n, double* A, std::vector<double>& ev) {
  cusolverDnHandle_t h = ctx_solver(ctx);
  int lwork = 0;
  DevBuf dev_w((size_t)n);
  if (cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, dev_w.p, &lwork) !=
      CUSOLVER_STATUS_SUCCESS)
    fail(ITHACA_GPU_ERR_CUDA, "cusolverDnDsyevd_bufferSize failed");
  DevBuf work((size_t)std::max(lwork, 1) + 1);  // the last double holds the info word
  int* info = reinterpret_cast<int*>(work.p + std::max(lwork, 1));
  if (cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, dev_w.p, work.p, lwork, info) !=
      CUSOLVER_STATUS_SUCCESS)
    fail(ITHACA_GPU_ERR_CUDA, "cusolverDnDsyevd failed");
  int hinfo = 0;
  ev.resize(n);
  ITHACA_CUDA(cudaMemcpyAsync(ev.data(), dev_w.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  ITHACA_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hinfo != 0) fail(ITHACA_GPU_ERR_NUMERIC, "symmetric eigen-solver did not converge (info " +
                                                   std::to_string(hinfo) + ")");
}

// Cholesky of an SPD r x r (column-major, lower); returns false if not SPD.
static bool cholesky(int r, std::vector<double>& G) {
  for (int j = 0; j < r; ++j) {
    double d = G[(size_t)j * r + j];
    for (int k = 0; k < j; ++k) d -= G[(size_t)k * r + j] * G[(size_t)k * r + j];
    if (!(d > 0)) return false;
    d = std::sqrt(d);
    G[(size_t)j * r + j] = d;
    for (int i = j + 1; i < r; ++i) {
      double s = G[(size_t)j * r + i];
      for (int k = 0; k < j; ++k) s -= G[(size_t)k * r + i] * G[(size_t)k * r + j];
      G[(size_t)j * r + i] = s / d;
    }
  }
  return true;
}

// ---- batched LU with partial pivoting: one CTA per system ----
constexpr int LU_MAX = 64;

__global__ void __launch_bounds__(256) batched_lu_kernel(int r, const double* __restrict__ AL,
                                                         const double* __restrict__ AM, const double* __restrict__ f,
                                                         const double* __restrict__ lambdas, double* __restrict__ x,
                                                         int* __restrict__ singular) {
  __shared__ double A[LU_MAX][LU_MAX + 1];
  __shared__ double b[LU_MAX];
  __shared__ int piv;
  const int sys = blockIdx.x;
  const double lam = lambdas[sys];
  for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
    const int i = idx % r, j = idx / r;  // column-major input
    A[i][j] = AL[idx] + lam * AM[idx];
  }
  for (int i = threadIdx.x; i < r; i += blockDim.x) b[i] = f[i];
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (threadIdx.x == 0) {  // pivot search (r <= 64, serial is fine)
      int p = k;
      double best = fabs(A[k][k]);
      for (int i = k + 1; i < r; ++i)
        if (fabs(A[i][k]) > best) {
          best = fabs(A[i][k]);
          p = i;
        }
      piv = p;
      if (!(best > 0)) atomicOr(singular, 1);
    }
    __syncthreads();
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < r; j += blockDim.x) {
        const double t = A[k][j];
        A[k][j] = A[p][j];
        A[p][j] = t;
      }
      if (threadIdx.x == 0) {
        const double t = b[k];
        b[k] = b[p];
        b[p] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / A[k][k];
    const int rows = r - k - 1;
    for (int idx = threadIdx.x; idx < rows * (r - k); idx += blockDim.x) {
      const int i = k + 1 + idx / (r - k), j = k + idx % (r - k);
      const double l = A[i][k] * inv;
      if (j > k) A[i][j] -= l * A[k][j];
    }
    for (int i = k + 1 + threadIdx.x; i < r; i += blockDim.x) b[i] -= A[i][k] * inv * b[k];
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < r; i += blockDim.x) A[i][k] = 0.0;
    __syncthreads();
  }
  if (threadIdx.x == 0) {  // back substitution
    for (int i = r - 1; i >= 0; --i) {
      double s = b[i];
      for (int j = i + 1; j < r; ++j) s -= A[i][j] * b[j];
      b[i] = s / A[i][i];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < r; i += blockDim.x) x[(size_t)sys * r + i] = b[i];
}

// r = s - r elementwise (deflation of the snapshot matrix).
__global__ void sub_from_kernel(size_t n, const double* __restrict__ s, double* __restrict__ r) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    r[i] = s[i] - r[i];
}

}  // namespace ithaca

using namespace ithaca;

struct ithaca_gpu_ctx : public Ctx {};
struct ithaca_gpu_cg;  // defined in cg.cu

namespace ithaca {
// implemented in cg.cu: L (lambda = 0) and M applications of the global operator to
// `ncols` global vectors (columns of X, nglobal rows), results assembled into Y.
void cg_apply_LM(ithaca_gpu_cg* cg, int ncols, const double* X, double* LX, double* MX);
int cg_sizes(ithaca_gpu_cg* cg, int* nglobal, int* ndir, Ctx** ctx);
}  // namespace ithaca

template <typename F>
static int pod_guarded(F f) {
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

static void preq(bool ok, const char* msg) {
  if (!ok) fail(ITHACA_GPU_ERR_ARG, msg);
}

// Copies n doubles from a host or device source into a fresh device buffer.
static std::unique_ptr<DevBuf> upload(const double* src, size_t n, int on_device, cudaStream_t s) {
  auto b = std::make_unique<DevBuf>(n);
  ITHACA_CUDA(cudaMemcpyAsync(b->p, src, sizeof(double) * n, on_device ? cudaMemcpyDeviceToDevice
                                                                       : cudaMemcpyHostToDevice, s));
  return b;
}

static void download(double* dst, const double* src, size_t n, int on_device, cudaStream_t s) {
  ITHACA_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, on_device ? cudaMemcpyDeviceToDevice
                                                                      : cudaMemcpyDeviceToHost, s));
}

extern "C" {

int ithaca_gpu_pod_gram(ithaca_gpu_ctx* ctx, int N, int ns, const double* S, double* C, int on_device) {
  return pod_guarded([&] {
    preq(ctx && S && C && N > 0 && ns > 0, "bad argument");
    StreamOrder order_(ctx);
    cudaStream_t s = ctx->stream;
    auto dS = upload(S, (size_t)N * ns, on_device, s);
    DevBuf dC((size_t)ns * ns), scratch(tn_scratch_doubles(ns, ns, N));
    dgemm_tn(ns, ns, N, dS->p, dS->p, dC.p, scratch.p, s, &ctx->launches);
    download(C, dC.p, (size_t)ns * ns, on_device, s);
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_pod_offline(ithaca_gpu_ctx* ctx, int N, int ns, const double* S, int nmodes, double* V,
                           double* sigma, int* nmodes_out, int on_device) {
  return pod_guarded([&] {
    preq(ctx && S && V && N > 0 && ns > 0 && nmodes > 0 && nmodes <= ns, "bad argument");
    StreamOrder order_(ctx);
    cudaStream_t s = ctx->stream;
    auto dS = upload(S, (size_t)N * ns, on_device, s);
    DevBuf dR((size_t)N * ns), dC((size_t)ns * ns), dV((size_t)N * nmodes), dT((size_t)N * nmodes),
        dG((size_t)nmodes * nmodes), dRinv((size_t)nmodes * nmodes), dP((size_t)nmodes * ns), dW((size_t)ns * nmodes),
        scratch(std::max(tn_scratch_doubles(ns, ns, N), tn_scratch_doubles(nmodes, ns, N)));
    ITHACA_CUDA(cudaMemcpyAsync(dR.p, dS->p, sizeof(double) * N * ns, cudaMemcpyDeviceToDevice, s));
    std::vector<double> sig(ns, 0.0);
    int r = 0;
    double l1 = 0;
    // Method of snapshots with deflation: each pass takes the eigenpairs of R^T R that
    // FP64 resolves (eigenvalue > 1e-10 of the pass maximum, so that sigma has ~6 digits), appends R W L^{-1/2} to V,
    // re-orthonormalises V (two Cholesky-QR passes) and deflates R = S - V (V^T S).
    for (int pass = 0; pass < 8 && r < nmodes; ++pass) {
      dgemm_tn(ns, ns, N, dR.p, dR.p, dC.p, scratch.p, s, &ctx->launches);
      std::vector<double> W((size_t)ns * ns), ev;
      sym_eigen(ctx, ns, dC.p, ev);  // dC now holds the eigenvectors
      ITHACA_CUDA(cudaMemcpyAsync(W.data(), dC.p, sizeof(double) * W.size(), cudaMemcpyDeviceToHost, s));
      ITHACA_CUDA(cudaStreamSynchronize(s));
      std::vector<int> order(ns);
      for (int i = 0; i < ns; ++i) order[i] = i;
      std::sort(order.begin(), order.end(), [&](int a, int b) { return ev[a] > ev[b]; });
      const double lmax = std::max(ev[order[0]], 0.0);
      if (pass == 0) l1 = lmax;
      if (!(lmax > 1e-28 * l1) || lmax <= 0) break;  // the rest is below FP64 noise of S
      std::vector<double> Wr;
      int taken = 0;
      for (int j = 0; j < ns && r + taken < nmodes; ++j) {
        const double l = ev[order[j]];
        if (!(l > 1e-10 * lmax)) break;
        const double sc = 1.0 / std::sqrt(l);
        for (int i = 0; i < ns; ++i) Wr.push_back(W[(size_t)order[j] * ns + i] * sc);
        sig[r + taken] = std::sqrt(l);
        ++taken;
      }
      for (int j = taken; j < ns && r + j < ns; ++j) sig[r + j] = std::sqrt(std::max(ev[order[j]], 0.0));
      if (taken == 0) break;
      ITHACA_CUDA(cudaMemcpyAsync(dW.p, Wr.data(), sizeof(double) * Wr.size(), cudaMemcpyHostToDevice, s));
      dgemm_nn(N, taken, ns, dR.p, dW.p, dV.p + (size_t)r * N, s, &ctx->launches);
      r += taken;
      for (int q = 0; q < 2; ++q) {  // Cholesky-QR: G = V^T V = L L^T, V <- V L^{-T}
        dgemm_tn(r, r, N, dV.p, dV.p, dG.p, scratch.p, s, &ctx->launches);
        std::vector<double> G((size_t)r * r);
        ITHACA_CUDA(cudaMemcpyAsync(G.data(), dG.p, sizeof(double) * G.size(), cudaMemcpyDeviceToHost, s));
        ITHACA_CUDA(cudaStreamSynchronize(s));
        if (!cholesky(r, G)) fail(ITHACA_GPU_ERR_NUMERIC, "POD modes are numerically dependent (Cholesky-QR failed)");
        std::vector<double> Rinv((size_t)r * r, 0.0);  // inverse of R = L^T (upper triangular)
        for (int j = 0; j < r; ++j) {
          Rinv[(size_t)j * r + j] = 1.0 / G[(size_t)j * r + j];
          for (int i = j - 1; i >= 0; --i) {
            double sum = 0;
            for (int k = i + 1; k <= j; ++k) sum += G[(size_t)i * r + k] * Rinv[(size_t)j * r + k];
            Rinv[(size_t)j * r + i] = -sum / G[(size_t)i * r + i];
          }
        }
        ITHACA_CUDA(cudaMemcpyAsync(dRinv.p, Rinv.data(), sizeof(double) * Rinv.size(), cudaMemcpyHostToDevice, s));
        dgemm_nn(N, r, r, dV.p, dRinv.p, dT.p, s, &ctx->launches);
        ITHACA_CUDA(cudaMemcpyAsync(dV.p, dT.p, sizeof(double) * N * r, cudaMemcpyDeviceToDevice, s));
      }
      if (r >= nmodes) break;
      // R = S - V (V^T S)
      dgemm_tn(r, ns, N, dV.p, dS->p, dP.p, scratch.p, s, &ctx->launches);
      dgemm_nn(N, ns, r, dV.p, dP.p, dR.p, s, &ctx->launches);
      sub_from_kernel<<<1024, 256, 0, s>>>((size_t)N * ns, dS->p, dR.p);
      ctx->launches++;
    }
    preq(r > 0, "snapshot matrix is zero");
    download(V, dV.p, (size_t)N * r, on_device, s);
    if (sigma) std::copy(sig.begin(), sig.end(), sigma);
    if (nmodes_out) *nmodes_out = r;
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_pod_project(ithaca_gpu_cg* cg, int nmodes, const double* V, double* A_L, double* A_M,
                           int on_device) {
  return pod_guarded([&] {
    preq(cg && V && A_L && A_M && nmodes > 0, "bad argument");
    int N = 0, ndir = 0;
    Ctx* ctx = nullptr;
    cg_sizes(cg, &N, &ndir, &ctx);
    StreamOrder order_(ctx);
    cudaStream_t s = ctx->stream;
    const int nnd = N - ndir;
    auto dV = upload(V, (size_t)nnd * nmodes, on_device, s);
    DevBuf X((size_t)N * nmodes), LX((size_t)N * nmodes), MX((size_t)N * nmodes);
    ITHACA_CUDA(cudaMemsetAsync(X.p, 0, sizeof(double) * N * nmodes, s));
    ITHACA_CUDA(cudaMemcpy2DAsync(X.p + ndir, sizeof(double) * N, dV->p, sizeof(double) * nnd, sizeof(double) * nnd,
                                  nmodes, cudaMemcpyDeviceToDevice, s));
    cg_apply_LM(cg, nmodes, X.p, LX.p, MX.p);
    // compact the non-Dirichlet rows, then A_X = V^T X
    DevBuf cL((size_t)nnd * nmodes), cM((size_t)nnd * nmodes), dAL((size_t)nmodes * nmodes),
        dAM((size_t)nmodes * nmodes), scratch(tn_scratch_doubles(nmodes, nmodes, nnd));
    ITHACA_CUDA(cudaMemcpy2DAsync(cL.p, sizeof(double) * nnd, LX.p + ndir, sizeof(double) * N, sizeof(double) * nnd,
                                  nmodes, cudaMemcpyDeviceToDevice, s));
    ITHACA_CUDA(cudaMemcpy2DAsync(cM.p, sizeof(double) * nnd, MX.p + ndir, sizeof(double) * N, sizeof(double) * nnd,
                                  nmodes, cudaMemcpyDeviceToDevice, s));
    dgemm_tn(nmodes, nmodes, nnd, dV->p, cL.p, dAL.p, scratch.p, s, &ctx->launches);
    dgemm_tn(nmodes, nmodes, nnd, dV->p, cM.p, dAM.p, scratch.p, s, &ctx->launches);
    download(A_L, dAL.p, (size_t)nmodes * nmodes, on_device, s);
    download(A_M, dAM.p, (size_t)nmodes * nmodes, on_device, s);
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_pod_online(ithaca_gpu_ctx* ctx, int r, const double* A_L, const double* A_M, const double* f_r,
                          int nlambda, const double* lambdas, double* x_r, int on_device) {
  return pod_guarded([&] {
    preq(ctx && A_L && A_M && f_r && lambdas && x_r, "null argument");
    StreamOrder order_(ctx);
    preq(r > 0 && r <= LU_MAX && nlambda > 0, "need 0 < r <= 64 and nlambda > 0");
    cudaStream_t s = ctx->stream;
    auto dL = upload(A_L, (size_t)r * r, on_device, s);
    auto dM = upload(A_M, (size_t)r * r, on_device, s);
    auto df = upload(f_r, r, on_device, s);
    auto dl = upload(lambdas, nlambda, on_device, s);
    DevBuf dx((size_t)r * nlambda);
    int* dsing = nullptr;
    ITHACA_CUDA(cudaMalloc(&dsing, sizeof(int)));
    std::unique_ptr<int, decltype(&cudaFree)> g(dsing, cudaFree);
    ITHACA_CUDA(cudaMemsetAsync(dsing, 0, sizeof(int), s));
    batched_lu_kernel<<<nlambda, 128, 0, s>>>(r, dL->p, dM->p, df->p, dl->p, dx.p, dsing);
    ctx->launches++;
    download(x_r, dx.p, (size_t)r * nlambda, on_device, s);
    int hs = 0;
    ITHACA_CUDA(cudaMemcpyAsync(&hs, dsing, sizeof(int), cudaMemcpyDeviceToHost, s));
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
    if (hs) fail(ITHACA_GPU_ERR_NUMERIC, "a reduced system is singular");
  });
}

int ithaca_gpu_pod_reconstruct(ithaca_gpu_ctx* ctx, int N, int r, const double* V, int nsol, const double* x_r,
                               double* u, int on_device) {
  return pod_guarded([&] {
    preq(ctx && V && x_r && u && N > 0 && r > 0 && nsol > 0, "bad argument");
    StreamOrder order_(ctx);
    cudaStream_t s = ctx->stream;
    auto dV = upload(V, (size_t)N * r, on_device, s);
    auto dx = upload(x_r, (size_t)r * nsol, on_device, s);
    DevBuf du((size_t)N * nsol);
    dgemm_nn(N, nsol, r, dV->p, dx->p, du.p, s, &ctx->launches);
    download(u, du.p, (size_t)N * nsol, on_device, s);
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(s));
  });
}

int ithaca_gpu_pod_rb_size(int ns, const double* sigma, double pod_tolerance, int* size) {
  return pod_guarded([&] {
    preq(sigma && size && ns > 0, "bad argument");
    double total = 0;
    for (int i = 0; i < ns; ++i) total += sigma[i];
    int rb = 1;
    double cum = 0;
    for (int i = 0; i < ns; ++i) {
      cum += sigma[i];
      if (cum / total < pod_tolerance) rb = i + 2;
    }
    *size = rb;
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Gram matrix without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need S^T S: a host
// that reserves all device memory up front for a fixed-budget pool and forbids further
// allocations in its solve loop, or a time-stepping loop that must not stall on the
// device-wide synchronisation cudaFree implies. ithaca_gpu_pod_gram allocates its split-K
// partial sums per call; this variant keeps them in a fixed, file-scope device array.
//
// The array holds kNoAllocGramDoubles doubles (2 MiB), allocated when the library is
// loaded on a device and held until the process exits. It bounds the problem: ns <= 128
// snapshots (the split-K reduction is capped so that splits * ns * ns fits). Every call
// shares the array and leaves the last call's partial sums in it; each partial is fully
// written before it is read, so nothing needs clearing, but calls whose work overlaps on
// the GPU (different streams, or other devices' host threads racing on one device) race
// on the array and must be serialised by the caller.
namespace ithaca {

constexpr int kNoAllocMaxSnapshots = 128;
constexpr int kNoAllocMaxSplits = 16;
constexpr size_t kNoAllocGramDoubles = (size_t)kNoAllocMaxSplits * kNoAllocMaxSnapshots * kNoAllocMaxSnapshots;

static __device__ __align__(256) double g_gram_scratch[kNoAllocGramDoubles];

// Device address of g_gram_scratch on the current device, looked up once per device
// (the host-side name of a __device__ array is only a stand-in, not a device address)
// and kept for the life of the process: a cudaDeviceReset of that device is not supported.
static double* gram_scratch_on_current_device() {
  constexpr int kMaxDevices = 64;
  static double* cache[kMaxDevices] = {};
  static std::mutex m;
  int dev = 0;
  ITHACA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) fail(ITHACA_GPU_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(m);
  if (!cache[dev]) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_gram_scratch);
    if (rc != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fail(ITHACA_GPU_ERR_CUDA, std::string("cudaGetSymbolAddress(g_gram_scratch): ") + cudaGetErrorString(rc));
    }
    cache[dev] = static_cast<double*>(p);
  }
  return cache[dev];
}

}  // namespace ithaca

extern "C" int ithaca_gpu_pod_gram_noalloc(int N, int ns, const double* S, double* C, void* stream) {
  return pod_guarded([&] {
    preq(S && C && N > 0 && ns > 0, "bad argument");
    if (ns > kNoAllocMaxSnapshots)
      fail(ITHACA_GPU_ERR_ARG, "ithaca_gpu_pod_gram_noalloc: ns = " + std::to_string(ns) + " exceeds the " +
                                   std::to_string(kNoAllocMaxSnapshots) +
                                   " snapshots its fixed scratch holds (use ithaca_gpu_pod_gram)");
    // an error left by the caller's earlier work is reported as such and stays pending
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
      fail(ITHACA_GPU_ERR_CUDA, std::string("ithaca_gpu_pod_gram_noalloc: a CUDA error from earlier work is pending (") +
                                    cudaGetErrorString(pending) + "); nothing was queued");
    double* scratch = gram_scratch_on_current_device();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const dim3 grid((ns + GT - 1) / GT, (ns + GT - 1) / GT, 1);
    int nsplit, kc;
    split_k(N, grid.x * grid.y, &nsplit, &kc);
    if (nsplit > kNoAllocMaxSplits) {  // fewer, longer splits so that the partials fit
      kc = (N + kNoAllocMaxSplits - 1) / kNoAllocMaxSplits;
      kc = (kc + GK - 1) / GK * GK;
      nsplit = (N + kc - 1) / kc;
    }
    const size_t stride = (size_t)ns * ns;
    if ((size_t)nsplit * stride > kNoAllocGramDoubles) fail(ITHACA_GPU_ERR_ARG, "noalloc Gram scratch too small");
    dgemm_kernel<true><<<dim3(grid.x, grid.y, nsplit), 256, 0, s>>>(ns, ns, N, kc, S, N, S, N, scratch, stride, ns);
    sum_parts_kernel<<<std::min<size_t>((stride + 255) / 256, 1024), 256, 0, s>>>(stride, nsplit, scratch, stride, C);
    ITHACA_CUDA(cudaGetLastError());
  });
}
