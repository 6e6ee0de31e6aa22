// Geometric factors on the GPU.
//
// geom_factors_kernel restates SpatialDomains/GeomFactors.cpp for coordinate
// dimension == shape dimension: collocation derivatives of the coordinates
// (ComputeDeriv :168-239, map points == target points), g_ij, its adjugate,
// J = sqrt(det g) (ComputeJac :252-308) and df[k*d+j] = sum_i dx_k/dxi_i (g^-1)_ij
// = dxi_j/dx_k (ComputeDerivFactors :399-475), written in the CoalescedGeomData
// layouts (Collections/CoalescedGeomData.cpp:53-313).
//
// build_jg_kernel turns (jac, df) into what the element kernels read per point:
// Jw = J w_i w_j [w_k] and G_ab = Jw g^{ab}, g^{ab} = sum_k df[k*d+a] df[k*d+b]
// (the metric of MatrixFreeOps/Helmholtz.h:193-205, 794-833), laid out
// [e][field][point] so that a CTA reads one contiguous slab per element.
#include "ithaca_internal.h"

namespace ithaca {

__global__ void geom_factors_kernel(int dim, int Q, int E, const double* __restrict__ D,
                                    const double* __restrict__ X, double* __restrict__ jac,
                                    double* __restrict__ df, int* bad) {
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  const size_t total = (size_t)E * nq;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q, j = (p / Q) % Q, k = p / (Q * Q);
    double dr[3][3];  // dr[a][c] = dx_c / dxi_a
    for (int c = 0; c < dim; ++c) {
      const double* x = X + (size_t)c * total + (size_t)e * nq;
      double s0 = 0, s1 = 0, s2 = 0;
      for (int a = 0; a < Q; ++a) {
        s0 += D[a * Q + i] * x[p + (a - i)];
        s1 += D[a * Q + j] * x[p + (a - j) * Q];
        if (dim == 3) s2 += D[a * Q + k] * x[p + (a - k) * Q * Q];
      }
      dr[0][c] = s0;
      dr[1][c] = s1;
      dr[2][c] = s2;
    }
    double g[3][3], adj[3][3], det;
    for (int a = 0; a < dim; ++a)
      for (int b = 0; b < dim; ++b) {
        double s = 0;
        for (int c = 0; c < dim; ++c) s += dr[a][c] * dr[b][c];
        g[a][b] = s;
      }
    if (dim == 2) {
      adj[0][0] = g[1][1];
      adj[0][1] = -g[0][1];
      adj[1][0] = -g[1][0];
      adj[1][1] = g[0][0];
    } else {
      adj[0][0] = g[1][1] * g[2][2] - g[1][2] * g[2][1];
      adj[0][1] = g[0][2] * g[2][1] - g[0][1] * g[2][2];
      adj[0][2] = g[0][1] * g[1][2] - g[0][2] * g[1][1];
      adj[1][0] = g[1][2] * g[2][0] - g[1][0] * g[2][2];
      adj[1][1] = g[0][0] * g[2][2] - g[0][2] * g[2][0];
      adj[1][2] = g[0][2] * g[1][0] - g[0][0] * g[1][2];
      adj[2][0] = g[1][0] * g[2][1] - g[1][1] * g[2][0];
      adj[2][1] = g[0][1] * g[2][0] - g[0][0] * g[2][1];
      adj[2][2] = g[0][0] * g[1][1] - g[0][1] * g[1][0];
    }
    det = 0;
    for (int a = 0; a < dim; ++a) det += g[0][a] * adj[a][0];
    if (!(det > 0.0)) atomicOr(bad, 1);
    jac[gid] = sqrt(det);
    for (int c = 0; c < dim; ++c)
      for (int b = 0; b < dim; ++b) {
        double s = 0;
        for (int a = 0; a < dim; ++a) s += dr[a][c] * adj[a][b] / det;
        df[(size_t)(c * dim + b) * total + gid] = s;
      }
  }
}

void launch_geom_factors(int dim, int Q, int E, const double* D, const double* coords, double* jac, double* df,
                         int* bad, cudaStream_t s) {
  const size_t total = (size_t)E * (dim == 2 ? Q * Q : Q * Q * Q);
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  geom_factors_kernel<<<blocks, threads, 0, s>>>(dim, Q, E, D, coords, jac, df, bad);
}

template <typename T>
__global__ void build_jg_kernel(int dim, int Q, int E, int deformed, const double* __restrict__ w,
                                const double* __restrict__ jac, const double* __restrict__ df,
                                T* __restrict__ jg, T* __restrict__ dfo) {
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  const int npt = deformed ? nq : 1;
  const int ng = n_jg(dim), nd = dim * dim;
  const size_t total = (size_t)E * npt;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / npt), p = (int)(gid % npt);
    double wp = 1.0;  // regular elements: the kernels multiply the weights in per point
    if (deformed) {
      wp = w[p % Q] * w[(p / Q) % Q];
      if (dim == 3) wp *= w[p / (Q * Q)];
    }
    const double jw = jac[gid] * wp;
    double f[9];
    for (int c = 0; c < nd; ++c) f[c] = df[(size_t)c * total + gid];
    T* out = jg + (size_t)e * ng * npt + p;
    out[0] = (T)jw;
    int cnt = 1;
    for (int a = 0; a < dim; ++a)
      for (int b = a; b < dim; ++b) {
        double s = 0;
        for (int k = 0; k < dim; ++k) s += f[k * dim + a] * f[k * dim + b];
        out[(size_t)cnt * npt] = (T)(jw * s);
        ++cnt;
      }
    T* o2 = dfo + (size_t)e * nd * npt + p;
    for (int c = 0; c < nd; ++c) o2[(size_t)c * npt] = (T)f[c];
  }
}

template <typename T>
void launch_build_jg(int dim, int Q, int E, int deformed, const double* w, const double* jac, const double* df,
                     T* jg, T* dfo, cudaStream_t s) {
  const size_t total = (size_t)E * (deformed ? (dim == 2 ? Q * Q : Q * Q * Q) : 1);
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  build_jg_kernel<T><<<blocks, threads, 0, s>>>(dim, Q, E, deformed, w, jac, df, jg, dfo);
}

template void launch_build_jg<double>(int, int, int, int, const double*, const double*, const double*, double*,
                                      double*, cudaStream_t);
template void launch_build_jg<float>(int, int, int, int, const double*, const double*, const double*, float*,
                                     float*, cudaStream_t);

}  // namespace ithaca
