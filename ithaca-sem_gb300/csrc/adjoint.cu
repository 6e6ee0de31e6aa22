// Variable-coefficient Helmholtz and the adjoint gradient of a misfit.
//
// A(kappa) = lambda M + L_kappa with an isotropic coefficient kappa at the quadrature
// points: the reference's LaplacianMatrixOp_MatFree with eVarCoeffD00 = eVarCoeffD11
// [= D22] = kappa (StdRegions/StdExpansion.cpp:664-717). On the GPU it is the same element
// kernel fed a geometry whose metric fields G_ab = Jw g^{ab} are scaled by kappa_q
// (scale_metric_kernel), so the solver, the Jacobi diagonal and the FP32 copy all see it.
//
// The misfit J = sum_q Jw_q (u_q - t_q)^2 and the gradient
//   dJ/dkappa_q = -Jw_q grad psi(x_q) . grad u(x_q),   A(kappa) psi = dJ/du,
// have no counterpart in the reference; they are new here (the adjoint of the
// symmetric Helmholtz system is the same solver).
#include <memory>

#include "ithaca_internal.h"

namespace ithaca {

constexpr int AT = 256, AB = 608;

// dst = src with fields 1.. (the metric) multiplied by kappa at each point (deformed layout).
__global__ void scale_metric_kernel(int E, int ng, int nq, const double* __restrict__ src,
                                    const double* __restrict__ kappa, double* __restrict__ dst) {
  const size_t total = (size_t)E * ng * nq;
  for (size_t i = (size_t)blockIdx.x * AT + threadIdx.x; i < total; i += (size_t)AB * AT) {
    const size_t e = i / ((size_t)ng * nq);
    const int c = (int)((i / nq) % ng);
    const int p = (int)(i % nq);
    dst[i] = c == 0 ? src[i] : kappa[e * nq + p] * src[i];
  }
}

// diff_q = 2 (u_q - t_q) in place of u; partial sums of Jw (u - t)^2 per CTA.
__global__ void misfit_kernel(int E, int ng, int nq, const double* __restrict__ jg, double* __restrict__ u,
                              const double* __restrict__ t, double* __restrict__ partial) {
  __shared__ double sm[AT];
  double acc = 0;
  const size_t total = (size_t)E * nq;
  for (size_t i = (size_t)blockIdx.x * AT + threadIdx.x; i < total; i += (size_t)AB * AT) {
    const size_t e = i / nq;
    const int p = (int)(i % nq);
    const double d = u[i] - t[i];
    acc += jg[e * ng * nq + p] * d * d;
    u[i] = 2.0 * d;
  }
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int w = AT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

__global__ void sum_fixed_kernel(const double* __restrict__ partial, int n, double* out) {
  __shared__ double sm[AT];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += AT) s += partial[i];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = AT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

// grad_q = -Jw_q sum_k du_k dpsi_k.
__global__ void kappa_grad_kernel(int E, int ng, int nq, int dim, const double* __restrict__ jg,
                                  const double* __restrict__ du, const double* __restrict__ dp,
                                  double* __restrict__ grad) {
  const size_t total = (size_t)E * nq;
  for (size_t i = (size_t)blockIdx.x * AT + threadIdx.x; i < total; i += (size_t)AB * AT) {
    const size_t e = i / nq;
    const int p = (int)(i % nq);
    double s = 0;
    for (int k = 0; k < dim; ++k) s += du[k * total + i] * dp[k * total + i];
    grad[i] = -jg[e * ng * nq + p] * s;
  }
}

__global__ void zero_head_kernel(int n, double* __restrict__ a) {
  for (int i = blockIdx.x * AT + threadIdx.x; i < n; i += AB * AT) a[i] = 0.0;
}

// Anisotropic coefficient: the metric of the Laplacian term becomes
// J w sum_{k,l} (dxi_a/dx_k) K_kl (dxi_b/dx_l), with K the symmetric tensor at each point
// (K components in the order D00, D01, (D02,) D11, (D12, D22), each E*nq values; df per
// element dfe[e][k*d+a][p] = dxi_a/dx_k). dst keeps J w in field 0 and the d(d+1)/2 metric
// terms (upper triangle, row-major) after it.
__global__ void tensor_metric_kernel(int E, int dim, int nq, const double* __restrict__ jg,
                                     const double* __restrict__ dfe, const double* __restrict__ K,
                                     double* __restrict__ dst) {
  const size_t total = (size_t)E * nq;
  const int ng = 1 + dim * (dim + 1) / 2, nd = dim * dim;
  for (size_t i = (size_t)blockIdx.x * AT + threadIdx.x; i < total; i += (size_t)AB * AT) {
    const size_t e = i / nq;
    const int p = (int)(i % nq);
    const double jw = jg[e * ng * nq + p];
    double f[9], k[3][3];
    for (int c = 0; c < nd; ++c) f[c] = dfe[(e * nd + c) * nq + p];
    int t = 0;
    for (int a = 0; a < dim; ++a)
      for (int b = a; b < dim; ++b) {
        k[a][b] = k[b][a] = K[(size_t)t * total + i];
        ++t;
      }
    double* out = dst + e * ng * nq + p;
    out[0] = jw;
    int cnt = 1;
    for (int a = 0; a < dim; ++a)
      for (int b = a; b < dim; ++b) {
        double s = 0;
        for (int kk = 0; kk < dim; ++kk)
          for (int l = 0; l < dim; ++l) s += f[kk * dim + a] * k[kk][l] * f[l * dim + b];
        out[(size_t)cnt * nq] = jw * s;
        ++cnt;
      }
  }
}

}  // namespace ithaca

namespace ithaca {

void launch_tensor_metric(int E, int dim, int nq, const double* jg, const double* dfe, const double* K, double* dst,
                          cudaStream_t s) {
  tensor_metric_kernel<<<AB, AT, 0, s>>>(E, dim, nq, jg, dfe, K, dst);
}

void launch_scale_metric(int E, int ng, int nq, const double* src, const double* kappa, double* dst,
                         cudaStream_t s) {
  scale_metric_kernel<<<AB, AT, 0, s>>>(E, ng, nq, src, kappa, dst);
}

void launch_misfit(int E, int ng, int nq, const double* jg, double* u, const double* t, double* partial,
                   double* out, cudaStream_t s) {
  misfit_kernel<<<AB, AT, 0, s>>>(E, ng, nq, jg, u, t, partial);
  sum_fixed_kernel<<<1, AT, 0, s>>>(partial, AB, out);
}

void launch_kappa_grad(int E, int ng, int nq, int dim, const double* jg, const double* du, const double* dp,
                       double* grad, cudaStream_t s) {
  kappa_grad_kernel<<<AB, AT, 0, s>>>(E, ng, nq, dim, jg, du, dp, grad);
}

void launch_zero_head(int n, double* a, cudaStream_t s) {
  if (n > 0) zero_head_kernel<<<AB, AT, 0, s>>>(n, a);
}

}  // namespace ithaca
