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

}  // namespace ithaca

namespace ithaca {

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
