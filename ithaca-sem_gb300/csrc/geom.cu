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

// ---- triangles ----
// Coordinates at the Q0 x Q1 collapsed points -> J and df per point: the collapsed
// derivatives mapped by d/dxi0 = h1 d/deta0, d/dxi1 = h0 h1 d/deta0 + d/deta1 (the chain
// rule of StdRegions/StdTriExp.cpp v_PhysDeriv), J = det(dx/dxi), df = its inverse
// (df[k*2 + j] = dxi_j / dx_k). Flags non-positive Jacobians (inverted triangles).
__global__ void geom_factors_tri_kernel(int n, int E, const double* __restrict__ tab, const double* __restrict__ X,
                                        double* __restrict__ jac, double* __restrict__ df, int* bad) {
  const TriOff o = tri_off(n);
  const int Q0 = n + 1, Q1 = n, nq = Q0 * Q1;
  const size_t total = (size_t)E * nq;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int j = p / Q0, i = p - j * Q0;
    double dx[2][2];  // dx[c][a] = dx_c / dxi_a
    for (int c = 0; c < 2; ++c) {
      const double* x = X + (size_t)c * total + (size_t)e * nq;
      double d0 = 0, d1 = 0;
      for (int a = 0; a < Q0; ++a) d0 += tab[o.D0 + a * Q0 + i] * x[j * Q0 + a];
      for (int a = 0; a < Q1; ++a) d1 += tab[o.D1 + a * Q1 + j] * x[a * Q0 + i];
      const double x0 = tab[o.h1 + j] * d0;
      dx[c][0] = x0;
      dx[c][1] = d1 + tab[o.h0 + i] * x0;
    }
    const double det = dx[0][0] * dx[1][1] - dx[0][1] * dx[1][0];
    if (!(det > 0.0)) atomicOr(bad, 1);
    jac[gid] = det;
    df[0 * total + gid] = dx[1][1] / det;
    df[1 * total + gid] = -dx[1][0] / det;
    df[2 * total + gid] = -dx[0][1] / det;
    df[3 * total + gid] = dx[0][0] / det;
  }
}

void launch_geom_factors_tri(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                             int* bad, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  geom_factors_tri_kernel<<<blocks, threads, 0, s>>>(n, E, tab, coords, jac, df, bad);
}

// Deformed triangles: per point Jw = J w0_i w1_j (w1 with its factor 1/2) and Jw m^{ab}
// with the collapsed metric of HelmholtzTriImpl (MatrixFreeOps/Helmholtz.h:581-605):
//   a = h1 (df0 + h0 df1), b = h1 (df2 + h0 df3),
//   m00 = a^2 + b^2, m01 = a df1 + b df3, m11 = df1^2 + df3^2.
// Regular triangles: per element J and J g^{ab} as for quads.
template <typename T>
__global__ void build_jg_tri_kernel(int n, int E, int deformed, const double* __restrict__ tab,
                                    const double* __restrict__ jac, const double* __restrict__ df,
                                    T* __restrict__ jg, T* __restrict__ dfo) {
  const TriOff o = tri_off(n);
  const int Q0 = n + 1, nq = (n + 1) * n;
  const int npt = deformed ? nq : 1;
  const size_t total = (size_t)E * npt;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / npt), p = (int)(gid % npt);
    double f[4];
    for (int c = 0; c < 4; ++c) f[c] = df[(size_t)c * total + gid];
    T* out = jg + (size_t)e * 4 * npt + p;
    if (deformed) {
      const int j = p / Q0, i = p - j * Q0;
      const double h0 = tab[o.h0 + i], h1 = tab[o.h1 + j];
      const double jw = jac[gid] * tab[o.w0 + i] * tab[o.w1 + j];
      const double a = h1 * (f[0] + h0 * f[1]);
      const double b = h1 * (f[2] + h0 * f[3]);
      out[0] = (T)jw;
      out[(size_t)npt] = (T)(jw * (a * a + b * b));
      out[(size_t)2 * npt] = (T)(jw * (a * f[1] + b * f[3]));
      out[(size_t)3 * npt] = (T)(jw * (f[1] * f[1] + f[3] * f[3]));
    } else {
      const double J = jac[gid];
      out[0] = (T)J;
      out[1] = (T)(J * (f[0] * f[0] + f[2] * f[2]));
      out[2] = (T)(J * (f[0] * f[1] + f[2] * f[3]));
      out[3] = (T)(J * (f[1] * f[1] + f[3] * f[3]));
    }
    T* o2 = dfo + (size_t)e * 4 * npt + p;
    for (int c = 0; c < 4; ++c) o2[(size_t)c * npt] = (T)f[c];
  }
}

template <typename T>
void launch_build_jg_tri(int n, int E, int deformed, const double* tab, const double* jac, const double* df, T* jg,
                         T* dfo, cudaStream_t s) {
  const size_t total = (size_t)E * (deformed ? (n + 1) * n : 1);
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  build_jg_tri_kernel<T><<<blocks, threads, 0, s>>>(n, E, deformed, tab, jac, df, jg, dfo);
}

template void launch_build_jg_tri<double>(int, int, int, const double*, const double*, const double*, double*,
                                          double*, cudaStream_t);
template void launch_build_jg_tri<float>(int, int, int, const double*, const double*, const double*, float*,
                                         float*, cudaStream_t);

// ---- tetrahedra ----
// xi derivatives from the collapsed ones: d/dxi0 = h2 h3 d0, d/dxi1 = h0 d/dxi0 + h3 d1,
// d/dxi2 = h0 d/dxi0 + h1 h3 d1 + d2 (the chain rule of StdTetExp::v_PhysDeriv).
__device__ __forceinline__ void tet_xi(const TetOff& o, const double* __restrict__ tab, int i, int j, int k,
                                       double d0, double d1, double d2, double& x0, double& x1, double& x2) {
  const double h0 = tab[o.h0 + i], h1 = tab[o.h1 + j], h2 = tab[o.h2 + j], h3 = tab[o.h3 + k];
  x0 = h2 * h3 * d0;
  x1 = h0 * x0 + h3 * d1;
  x2 = h0 * x0 + h1 * h3 * d1 + d2;
}

// Coordinates at the (n+1) n n collapsed points -> J = det(dx/dxi) and df = its inverse
// (df[c*3 + j] = dxi_j / dx_c) per point; flags non-positive Jacobians.
__global__ void geom_factors_tet_kernel(int n, int E, const double* __restrict__ tab, const double* __restrict__ X,
                                        double* __restrict__ jac, double* __restrict__ df, int* bad) {
  const TetOff o = tet_off(n);
  const int Q0 = n + 1, Q = n, nq = Q0 * Q * Q;
  const size_t total = (size_t)E * nq;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
    double M[3][3];  // M[c][a] = dx_c / dxi_a
    for (int c = 0; c < 3; ++c) {
      const double* x = X + (size_t)c * total + (size_t)e * nq;
      double d0 = 0, d1 = 0, d2 = 0;
      for (int a = 0; a < Q0; ++a) d0 += tab[o.D0 + a * Q0 + i] * x[(k * Q + j) * Q0 + a];
      for (int a = 0; a < Q; ++a) d1 += tab[o.D1 + a * Q + j] * x[(k * Q + a) * Q0 + i];
      for (int a = 0; a < Q; ++a) d2 += tab[o.D2 + a * Q + k] * x[(a * Q + j) * Q0 + i];
      tet_xi(o, tab, i, j, k, d0, d1, d2, M[c][0], M[c][1], M[c][2]);
    }
    const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    if (!(det > 0.0)) atomicOr(bad, 1);
    jac[gid] = det;
    // inverse: inv[a][c] = cofactor(c, a) / det
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[1][0] = c01 / det;
    inv[2][0] = c02 / det;
    inv[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
    inv[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
    inv[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
    inv[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
    inv[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
    inv[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) df[(size_t)(c * 3 + a) * total + gid] = inv[a][c];
  }
}

void launch_geom_factors_tet(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                             int* bad, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * n * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  geom_factors_tet_kernel<<<blocks, threads, 0, s>>>(n, E, tab, coords, jac, df, bad);
}

// Per point Jw = J w0 w1/2 w2/4 and Jw m^{ab} (fields 00, 01, 02, 11, 12, 22) with the
// collapsed metric of HelmholtzTetImpl (MatrixFreeOps/Helmholtz.h:2336-2420): for each
// physical direction c, a_c = h2 h3 (df_c0 + h0 (df_c1 + df_c2)), b_c = h3 (df_c1 + h1 df_c2),
// e_c = df_c2; m00 = a.a, m01 = a.b, m02 = a.e, m11 = b.b, m12 = b.e, m22 = e.e. The input
// geometry may be per point or per element; the output is always per point.
template <typename T>
__global__ void build_jg_tet_kernel(int n, int E, int deformed, const double* __restrict__ tab,
                                    const double* __restrict__ jac, const double* __restrict__ df,
                                    T* __restrict__ jg, T* __restrict__ dfo) {
  const TetOff o = tet_off(n);
  const int Q0 = n + 1, Q = n, nq = Q0 * Q * Q;
  const size_t total = (size_t)E * nq, tin = (size_t)E * (deformed ? nq : 1);
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q, k = p / (Q0 * Q);
    const size_t src = deformed ? gid : (size_t)e;
    double f[9];
    for (int c = 0; c < 9; ++c) f[c] = df[(size_t)c * tin + src];
    const double h0 = tab[o.h0 + i], h1 = tab[o.h1 + j], h2 = tab[o.h2 + j], h3 = tab[o.h3 + k];
    const double jw = jac[src] * tab[o.w0 + i] * tab[o.w1 + j] * tab[o.w2 + k];
    double a[3], b[3], c3[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = h2 * h3 * (f[3 * c] + h0 * (f[3 * c + 1] + f[3 * c + 2]));
      b[c] = h3 * (f[3 * c + 1] + h1 * f[3 * c + 2]);
      c3[c] = f[3 * c + 2];
    }
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    T* out = jg + (size_t)e * 7 * nq + p;
    out[0] = (T)jw;
    out[(size_t)1 * nq] = (T)(jw * dot(a, a));
    out[(size_t)2 * nq] = (T)(jw * dot(a, b));
    out[(size_t)3 * nq] = (T)(jw * dot(a, c3));
    out[(size_t)4 * nq] = (T)(jw * dot(b, b));
    out[(size_t)5 * nq] = (T)(jw * dot(b, c3));
    out[(size_t)6 * nq] = (T)(jw * dot(c3, c3));
    T* o2 = dfo + (size_t)e * 9 * nq + p;
    for (int c = 0; c < 9; ++c) o2[(size_t)c * nq] = (T)f[c];
  }
}

template <typename T>
void launch_build_jg_tet(int n, int E, int deformed, const double* tab, const double* jac, const double* df, T* jg,
                         T* dfo, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * n * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  build_jg_tet_kernel<T><<<blocks, threads, 0, s>>>(n, E, deformed, tab, jac, df, jg, dfo);
}

template void launch_build_jg_tet<double>(int, int, int, const double*, const double*, const double*, double*,
                                          double*, cudaStream_t);
template void launch_build_jg_tet<float>(int, int, int, const double*, const double*, const double*, float*,
                                         float*, cudaStream_t);

// ---- prisms ----
// xi derivatives: d/dxi0 = h1 d0, d/dxi1 = d1, d/dxi2 = h0 d/dxi0 + d2 (StdPrismExp).
__global__ void geom_factors_prism_kernel(int n, int E, const double* __restrict__ tab,
                                          const double* __restrict__ X, double* __restrict__ jac,
                                          double* __restrict__ df, int* bad) {
  const PrismOff o = prism_off(n);
  const int Q0 = n + 1, Q2 = n, nq = Q0 * Q0 * Q2;
  const size_t total = (size_t)E * nq;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q0, k = p / (Q0 * Q0);
    double M[3][3];
    for (int c = 0; c < 3; ++c) {
      const double* x = X + (size_t)c * total + (size_t)e * nq;
      double d0 = 0, d1 = 0, d2 = 0;
      for (int a = 0; a < Q0; ++a) d0 += tab[o.D0 + a * Q0 + i] * x[(k * Q0 + j) * Q0 + a];
      for (int a = 0; a < Q0; ++a) d1 += tab[o.D0 + a * Q0 + j] * x[(k * Q0 + a) * Q0 + i];
      for (int a = 0; a < Q2; ++a) d2 += tab[o.D2 + a * Q2 + k] * x[(a * Q0 + j) * Q0 + i];
      M[c][0] = tab[o.h1 + k] * d0;
      M[c][1] = d1;
      M[c][2] = tab[o.h0 + i] * M[c][0] + d2;
    }
    const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    if (!(det > 0.0)) atomicOr(bad, 1);
    jac[gid] = det;
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[1][0] = c01 / det;
    inv[2][0] = c02 / det;
    inv[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
    inv[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
    inv[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
    inv[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
    inv[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
    inv[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) df[(size_t)(c * 3 + a) * total + gid] = inv[a][c];
  }
}

void launch_geom_factors_prism(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                               int* bad, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * (n + 1) * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  geom_factors_prism_kernel<<<blocks, threads, 0, s>>>(n, E, tab, coords, jac, df, bad);
}

// Per point Jw = J w0_i w0_j w2_k/2 and Jw m^{ab} with the collapsed metric of
// HelmholtzPrismImpl (MatrixFreeOps/Helmholtz.h:1340-1400): a_c = h1 (df_c0 + h0 df_c2),
// b_c = df_c1, e_c = df_c2.
template <typename T>
__global__ void build_jg_prism_kernel(int n, int E, int deformed, const double* __restrict__ tab,
                                      const double* __restrict__ jac, const double* __restrict__ df,
                                      T* __restrict__ jg, T* __restrict__ dfo) {
  const PrismOff o = prism_off(n);
  const int Q0 = n + 1, Q2 = n, nq = Q0 * Q0 * Q2;
  const size_t total = (size_t)E * nq, tin = (size_t)E * (deformed ? nq : 1);
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q0, k = p / (Q0 * Q0);
    const size_t src = deformed ? gid : (size_t)e;
    double f[9];
    for (int c = 0; c < 9; ++c) f[c] = df[(size_t)c * tin + src];
    const double h0 = tab[o.h0 + i], h1 = tab[o.h1 + k];
    const double jw = jac[src] * tab[o.w0 + i] * tab[o.w0 + j] * tab[o.w2 + k];
    double a[3], b[3], c3[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = h1 * (f[3 * c] + h0 * f[3 * c + 2]);
      b[c] = f[3 * c + 1];
      c3[c] = f[3 * c + 2];
    }
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    T* out = jg + (size_t)e * 7 * nq + p;
    out[0] = (T)jw;
    out[(size_t)1 * nq] = (T)(jw * dot(a, a));
    out[(size_t)2 * nq] = (T)(jw * dot(a, b));
    out[(size_t)3 * nq] = (T)(jw * dot(a, c3));
    out[(size_t)4 * nq] = (T)(jw * dot(b, b));
    out[(size_t)5 * nq] = (T)(jw * dot(b, c3));
    out[(size_t)6 * nq] = (T)(jw * dot(c3, c3));
    T* o2 = dfo + (size_t)e * 9 * nq + p;
    for (int c = 0; c < 9; ++c) o2[(size_t)c * nq] = (T)f[c];
  }
}

template <typename T>
void launch_build_jg_prism(int n, int E, int deformed, const double* tab, const double* jac, const double* df,
                           T* jg, T* dfo, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * (n + 1) * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  build_jg_prism_kernel<T><<<blocks, threads, 0, s>>>(n, E, deformed, tab, jac, df, jg, dfo);
}

template void launch_build_jg_prism<double>(int, int, int, const double*, const double*, const double*, double*,
                                            double*, cudaStream_t);
template void launch_build_jg_prism<float>(int, int, int, const double*, const double*, const double*, float*,
                                           float*, cudaStream_t);

// ---- pyramids ----
// xi derivatives: d/dxi0 = h2 d0, d/dxi1 = h2 d1, d/dxi2 = h0 d/dxi0 + h1 d/dxi1 + d2
// (StdPyrExp; h1 = (1 + z0_j)/2).
__global__ void geom_factors_pyr_kernel(int n, int E, const double* __restrict__ tab,
                                          const double* __restrict__ X, double* __restrict__ jac,
                                          double* __restrict__ df, int* bad) {
  const PyrOff o = pyr_off(n);
  const int Q0 = n + 1, Q2 = n, nq = Q0 * Q0 * Q2;
  const size_t total = (size_t)E * nq;
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q0, k = p / (Q0 * Q0);
    double M[3][3];
    for (int c = 0; c < 3; ++c) {
      const double* x = X + (size_t)c * total + (size_t)e * nq;
      double d0 = 0, d1 = 0, d2 = 0;
      for (int a = 0; a < Q0; ++a) d0 += tab[o.D0 + a * Q0 + i] * x[(k * Q0 + j) * Q0 + a];
      for (int a = 0; a < Q0; ++a) d1 += tab[o.D0 + a * Q0 + j] * x[(k * Q0 + a) * Q0 + i];
      for (int a = 0; a < Q2; ++a) d2 += tab[o.D2 + a * Q2 + k] * x[(a * Q0 + j) * Q0 + i];
      M[c][0] = tab[o.h2 + k] * d0;
      M[c][1] = tab[o.h2 + k] * d1;
      M[c][2] = tab[o.h0 + i] * M[c][0] + tab[o.h0 + j] * M[c][1] + d2;
    }
    const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    if (!(det > 0.0)) atomicOr(bad, 1);
    jac[gid] = det;
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[1][0] = c01 / det;
    inv[2][0] = c02 / det;
    inv[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
    inv[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
    inv[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
    inv[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
    inv[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
    inv[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) df[(size_t)(c * 3 + a) * total + gid] = inv[a][c];
  }
}

void launch_geom_factors_pyr(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                               int* bad, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * (n + 1) * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  geom_factors_pyr_kernel<<<blocks, threads, 0, s>>>(n, E, tab, coords, jac, df, bad);
}

// Per point Jw = J w0_i w0_j w2_k/2 and Jw m^{ab} with the collapsed metric of
// HelmholtzPrismImpl (MatrixFreeOps/Helmholtz.h:1340-1400): a_c = h1 (df_c0 + h0 df_c2),
// b_c = df_c1, e_c = df_c2.
template <typename T>
__global__ void build_jg_pyr_kernel(int n, int E, int deformed, const double* __restrict__ tab,
                                      const double* __restrict__ jac, const double* __restrict__ df,
                                      T* __restrict__ jg, T* __restrict__ dfo) {
  const PyrOff o = pyr_off(n);
  const int Q0 = n + 1, Q2 = n, nq = Q0 * Q0 * Q2;
  const size_t total = (size_t)E * nq, tin = (size_t)E * (deformed ? nq : 1);
  for (size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(gid / nq), p = (int)(gid % nq);
    const int i = p % Q0, j = (p / Q0) % Q0, k = p / (Q0 * Q0);
    const size_t src = deformed ? gid : (size_t)e;
    double f[9];
    for (int c = 0; c < 9; ++c) f[c] = df[(size_t)c * tin + src];
    const double h0 = tab[o.h0 + i], h1 = tab[o.h0 + j], h2 = tab[o.h2 + k];
    const double jw = jac[src] * tab[o.w0 + i] * tab[o.w0 + j] * tab[o.w2 + k];
    double a[3], b[3], c3[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = h2 * (f[3 * c] + h0 * f[3 * c + 2]);
      b[c] = h2 * (f[3 * c + 1] + h1 * f[3 * c + 2]);
      c3[c] = f[3 * c + 2];
    }
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    T* out = jg + (size_t)e * 7 * nq + p;
    out[0] = (T)jw;
    out[(size_t)1 * nq] = (T)(jw * dot(a, a));
    out[(size_t)2 * nq] = (T)(jw * dot(a, b));
    out[(size_t)3 * nq] = (T)(jw * dot(a, c3));
    out[(size_t)4 * nq] = (T)(jw * dot(b, b));
    out[(size_t)5 * nq] = (T)(jw * dot(b, c3));
    out[(size_t)6 * nq] = (T)(jw * dot(c3, c3));
    T* o2 = dfo + (size_t)e * 9 * nq + p;
    for (int c = 0; c < 9; ++c) o2[(size_t)c * nq] = (T)f[c];
  }
}

template <typename T>
void launch_build_jg_pyr(int n, int E, int deformed, const double* tab, const double* jac, const double* df,
                           T* jg, T* dfo, cudaStream_t s) {
  const size_t total = (size_t)E * (n + 1) * (n + 1) * n;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, (size_t)device_sm_count() * 32);
  build_jg_pyr_kernel<T><<<blocks, threads, 0, s>>>(n, E, deformed, tab, jac, df, jg, dfo);
}

template void launch_build_jg_pyr<double>(int, int, int, const double*, const double*, const double*, double*,
                                            double*, cudaStream_t);
template void launch_build_jg_pyr<float>(int, int, int, const double*, const double*, const double*, float*,
                                           float*, cudaStream_t);

}  // namespace ithaca
