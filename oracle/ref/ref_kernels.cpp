// Oracle driver around the reference's OWN arithmetic (test infrastructure only).
//
// Compiled by oracle/ref/Makefile against the unmodified reference sources
//   library/LibUtilities/Polylib/Polylib.cpp            (GLL points, weights, D)
//   library/MatrixFreeOps/{BwdTrans,IProduct,PhysDeriv}Kernels.hpp
//   library/LibUtilities/SimdLib/*.hpp                  (tinysimd; scalar width 1)
// into oracle/_ref/libithaca_ref.so. This file only drives those kernels the way the
// reference operators do; every driver cites the reference routine it restates.
// It also provides the reference-path CPU baseline (multi-threaded element loop and
// the reference CG recurrence around it).

#include <LibUtilities/BasicConst/NektarUnivTypeDefs.hpp>
#include <LibUtilities/Polylib/Polylib.h>
#include <boost/core/ignore_unused.hpp>
#include <MatrixFreeOps/BwdTransKernels.hpp>
#include <MatrixFreeOps/IProductKernels.hpp>
#include <MatrixFreeOps/PhysDerivKernels.hpp>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

using namespace Nektar;
using namespace Nektar::MatrixFree;
using vvec = std::vector<vec_t, tinysimd::allocator<vec_t>>;
static constexpr int W = vec_t::width;

namespace {

// ---- basis -----------------------------------------------------------------
// GaussPoints::CalculatePoints / CalculateDerivMatrix for eGaussLobattoLegendre
// (LibUtilities/Foundations/GaussPoints.cpp:91-92,178-179,235).
void gll_tables(int Q, double* z, double* w, double* D) {
  Polylib::zwglj(z, w, Q, 0.0, 0.0);
  Polylib::Dglj(D, z, Q, 0.0, 0.0);  // raw storage copied as-is into the column-major matrix
}

// Basis::GenBasis eModified_A (LibUtilities/Foundations/Basis.cpp:392-421).
void modA_tables(int n, int Q, const double* z, const double* D, double* B, double* DB) {
  for (int i = 0; i < Q; ++i) {
    B[i] = 0.5 * (1 - z[i]);
    B[Q + i] = 0.5 * (1 + z[i]);
  }
  for (int p = 2; p < n; ++p) {
    double* mode = B + p * Q;
    Polylib::jacobfd(Q, z, mode, nullptr, p - 2, 1.0, 1.0);
    for (int i = 0; i < Q; ++i) mode[i] *= B[i] * B[Q + i];
  }
  // DB = D * B with D column-major (Q x Q) and B column-major (Q x n)
  for (int p = 0; p < n; ++p)
    for (int i = 0; i < Q; ++i) {
      double s = 0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * B[p * Q + k];
      DB[p * Q + i] = s;
    }
}

struct Tables {
  vvec b, db, D, w;
};

Tables make_tables(int n, int Q) {
  std::vector<double> z(Q), w(Q), D(Q * Q), B(n * Q), DB(n * Q);
  gll_tables(Q, z.data(), w.data(), D.data());
  modA_tables(n, Q, z.data(), D.data(), B.data(), DB.data());
  Tables t;
  t.b.assign(B.begin(), B.end());
  t.db.assign(DB.begin(), DB.end());
  t.D.assign(D.begin(), D.end());
  t.w.assign(w.begin(), w.end());
  return t;
}

// ---- geometry interleave (Collections/CoalescedGeomData.cpp:115-198, 315-403) ----
// Reference layouts in: jac[e*nq + q] (deformed) or jac[e]; df[dir][e*nq + q] or df[dir][e].
struct Geo {
  vvec jac, df;
};

Geo interleave(int dim, int nq, int E, int Epad, const double* jac, const double* df, bool deformed) {
  const int ndf = dim * dim;
  const int nb = Epad / W;
  Geo g;
  alignas(64) double tmp[16];
  if (deformed) {
    g.jac.resize((size_t)nb * nq);
    g.df.resize((size_t)nb * nq * ndf);
    for (int b = 0; b < nb; ++b)
      for (int q = 0; q < nq; ++q) {
        for (int j = 0; j < W; ++j) {
          int e = b * W + j;
          tmp[j] = e < E ? jac[(size_t)e * nq + q] : 0.0;
        }
        g.jac[(size_t)b * nq + q].load(tmp);
        for (int dir = 0; dir < ndf; ++dir) {
          for (int j = 0; j < W; ++j) {
            int e = b * W + j;
            tmp[j] = e < E ? df[(size_t)dir * E * nq + (size_t)e * nq + q] : 0.0;
          }
          g.df[((size_t)b * nq + q) * ndf + dir].load(tmp);
        }
      }
  } else {
    g.jac.resize(nb);
    g.df.resize((size_t)nb * ndf);
    for (int b = 0; b < nb; ++b) {
      for (int j = 0; j < W; ++j) tmp[j] = b * W + j < E ? jac[b * W + j] : 0.0;
      g.jac[b].load(tmp);
      for (int dir = 0; dir < ndf; ++dir) {
        for (int j = 0; j < W; ++j) tmp[j] = b * W + j < E ? df[(size_t)dir * E + b * W + j] : 0.0;
        g.df[(size_t)b * ndf + dir].load(tmp);
      }
    }
  }
  return g;
}

template <class F>
void parallel_blocks(int nb, int nthreads, F f) {
  nthreads = std::max(1, std::min(nthreads, nb));
  if (nthreads == 1) {
    f(0, nb);
    return;
  }
  std::vector<std::thread> th;
  int chunk = (nb + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    int b0 = t * chunk, b1 = std::min(nb, b0 + chunk);
    if (b0 >= b1) break;
    th.emplace_back([=] { f(b0, b1); });
  }
  for (auto& x : th) x.join();
}

// ---- Helmholtz: HelmholtzQuadImpl (MatrixFreeOps/Helmholtz.h:137-275) ----
template <int N, int Q, bool DEF>
void helm_quad(const Tables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int nm = N * N, nq = Q * Q, ndf = 4;
  constexpr int wspSize = (Q > Q * N) ? Q : Q * N;
  vec_t wsp[wspSize];
  vvec tmpIn(nm), tmpOut(nm), bwd(nq), d0v(nq), d1v(nq);
  const int dfSize = DEF ? ndf * nq : ndf;
  vec_t df0, df1, df2, df3, m00, m01, m11;
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * dfSize];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nm * W, nm, tmpIn);
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2]; df3 = df_ptr[3];
      m00 = df0 * df0; m00.fma(df2, df2);
      m01 = df0 * df1; m01.fma(df2, df3);
      m11 = df1 * df1; m11.fma(df3, df3);
    }
    BwdTransQuadKernel<N, N, Q, Q>(tmpIn, t.b, t.b, wsp, bwd);
    IProductQuadKernel<N, N, Q, Q, true, false, DEF>(bwd, t.b, t.b, t.w, t.w, jac_ptr, wsp, tmpOut, lambda);
    PhysDerivTensor2DKernel<Q, Q>(bwd, t.D, t.D, d0v, d1v);
    for (int c = 0; c < nq; ++c) {
      if (DEF) {
        df0 = df_ptr[c * ndf]; df1 = df_ptr[c * ndf + 1]; df2 = df_ptr[c * ndf + 2]; df3 = df_ptr[c * ndf + 3];
        m00 = df0 * df0; m00.fma(df2, df2);
        m01 = df0 * df1; m01.fma(df2, df3);
        m11 = df1 * df1; m11.fma(df3, df3);
      }
      vec_t a = d0v[c], b = d1v[c];
      vec_t t0 = m00 * a; t0.fma(m01, b);
      vec_t t1 = m01 * a; t1.fma(m11, b);
      bwd[c] = t0;
      d0v[c] = t1;
    }
    IProductQuadKernel<N, N, Q, Q, false, true, DEF>(bwd, t.db, t.b, t.w, t.w, jac_ptr, wsp, tmpOut);
    IProductQuadKernel<N, N, Q, Q, false, true, DEF>(d0v, t.b, t.db, t.w, t.w, jac_ptr, wsp, tmpOut);
    deinterleave_store(tmpOut, nm, out + (size_t)e * nm * W);
  }
}

// ---- Helmholtz: HelmholtzHexImpl (MatrixFreeOps/Helmholtz.h:763-993) ----
template <int N, int Q, bool DEF>
void helm_hex(const Tables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int nm = N * N * N, nq = Q * Q * Q, ndf = 9;
  std::vector<vec_t> w1(nq), w2(nq);
  vvec tmpIn(nm), tmpOut(nm), bwd(nq), d0v(nq), d1v(nq), d2v(nq);
  const int dfSize = DEF ? ndf * nq : ndf;
  vec_t df[9], m00, m01, m02, m11, m12, m22;
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * dfSize];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nm * W, nm, tmpIn);
    auto metrics = [&](const vec_t* d) {
      m00 = d[0] * d[0]; m00.fma(d[3], d[3]); m00.fma(d[6], d[6]);
      m01 = d[0] * d[1]; m01.fma(d[3], d[4]); m01.fma(d[6], d[7]);
      m02 = d[0] * d[2]; m02.fma(d[3], d[5]); m02.fma(d[6], d[8]);
      m11 = d[1] * d[1]; m11.fma(d[4], d[4]); m11.fma(d[7], d[7]);
      m12 = d[1] * d[2]; m12.fma(d[4], d[5]); m12.fma(d[7], d[8]);
      m22 = d[2] * d[2]; m22.fma(d[5], d[5]); m22.fma(d[8], d[8]);
    };
    if (!DEF) {
      for (int k = 0; k < 9; ++k) df[k] = df_ptr[k];
      metrics(df);
    }
    // The reference passes the direction-0 tables for all three directions
    // (Helmholtz.h:843-856); for homogeneous n and Q this is the same data.
    BwdTransHexKernel<N, N, N, Q, Q, Q>(tmpIn, t.b, t.b, t.b, w1.data(), w2.data(), bwd);
    IProductHexKernel<N, N, N, Q, Q, Q, true, false, DEF>(bwd, t.b, t.b, t.b, t.w, t.w, t.w, jac_ptr, w1.data(),
                                                          w2.data(), tmpOut, lambda);
    PhysDerivTensor3DKernel<Q, Q, Q>(bwd, t.D, t.D, t.D, d0v, d1v, d2v);
    for (int c = 0; c < nq; ++c) {
      if (DEF) {
        for (int k = 0; k < 9; ++k) df[k] = df_ptr[c * ndf + k];
        metrics(df);
      }
      vec_t a = d0v[c], b = d1v[c], cc = d2v[c];
      vec_t t0 = m00 * a; t0.fma(m01, b); t0.fma(m02, cc);
      vec_t t1 = m01 * a; t1.fma(m11, b); t1.fma(m12, cc);
      vec_t t2 = m02 * a; t2.fma(m12, b); t2.fma(m22, cc);
      d0v[c] = t0; d1v[c] = t1; d2v[c] = t2;
    }
    IProductHexKernel<N, N, N, Q, Q, Q, false, true, DEF>(d0v, t.db, t.b, t.b, t.w, t.w, t.w, jac_ptr, w1.data(),
                                                          w2.data(), tmpOut);
    IProductHexKernel<N, N, N, Q, Q, Q, false, true, DEF>(d1v, t.b, t.db, t.b, t.w, t.w, t.w, jac_ptr, w1.data(),
                                                          w2.data(), tmpOut);
    IProductHexKernel<N, N, N, Q, Q, Q, false, true, DEF>(d2v, t.b, t.b, t.db, t.w, t.w, t.w, jac_ptr, w1.data(),
                                                          w2.data(), tmpOut);
    deinterleave_store(tmpOut, nm, out + (size_t)e * nm * W);
  }
}

// ---- BwdTrans / IProduct / PhysDeriv operators (MatrixFreeOps/BwdTrans.h:172-331,576-734;
//      IProduct.h:178-347,604-786; PhysDeriv.h:255-380,508-644) ----
template <int N, int Q>
void bwd_op(int dim, const Tables& t, const double* in, double* out, int b0, int b1) {
  const int nm = dim == 2 ? N * N : N * N * N, nq = dim == 2 ? Q * Q : Q * Q * Q;
  vvec tin(nm), tout(nq);
  std::vector<vec_t> w1(Q * Q * Q), w2(Q * Q * Q);
  for (int e = b0; e < b1; ++e) {
    load_interleave(in + (size_t)e * nm * W, nm, tin);
    if (dim == 2)
      BwdTransQuadKernel<N, N, Q, Q>(tin, t.b, t.b, w1.data(), tout);
    else
      BwdTransHexKernel<N, N, N, Q, Q, Q>(tin, t.b, t.b, t.b, w1.data(), w2.data(), tout);
    deinterleave_store(tout, nq, out + (size_t)e * nq * W);
  }
}

template <int N, int Q, bool DEF>
void iprod_op(int dim, const Tables& t, const Geo& g, const double* in, double* out, int b0, int b1) {
  const int nm = dim == 2 ? N * N : N * N * N, nq = dim == 2 ? Q * Q : Q * Q * Q;
  vvec tin(nq), tout(nm);
  std::vector<vec_t> w1(Q * Q * Q), w2(Q * Q * Q);
  for (int e = b0; e < b1; ++e) {
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    if (dim == 2)
      IProductQuadKernel<N, N, Q, Q, false, false, DEF>(tin, t.b, t.b, t.w, t.w, jac_ptr, w1.data(), tout);
    else
      IProductHexKernel<N, N, N, Q, Q, Q, false, false, DEF>(tin, t.b, t.b, t.b, t.w, t.w, t.w, jac_ptr, w1.data(),
                                                             w2.data(), tout);
    deinterleave_store(tout, nm, out + (size_t)e * nm * W);
  }
}

template <int N, int Q, bool DEF>
void deriv_op(int dim, const Tables& t, const Geo& g, const double* in, double* o0, double* o1, double* o2, int b0,
              int b1) {
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  const int ndf = dim * dim;
  vvec tin(nq), a(nq), b(nq), c(nq);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nq : ndf)];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    if (dim == 2) {
      PhysDerivQuadKernel<Q, Q, DEF>(tin, t.w, t.w, t.D, t.D, df_ptr, a, b);
    } else {
      PhysDerivHexKernel<Q, Q, Q, DEF>(tin, t.w, t.w, t.w, t.D, t.D, t.D, df_ptr, a, b, c);
      deinterleave_store(c, nq, o2 + (size_t)e * nq * W);
    }
    deinterleave_store(a, nq, o0 + (size_t)e * nq * W);
    deinterleave_store(b, nq, o1 + (size_t)e * nq * W);
  }
}

// ---- triangles: eModified_A on Q0 = n + 1 GLL points in direction 0, eModified_B on
//      Q1 = n Gauss-Radau-Jacobi (alpha 1, beta 0) points in direction 1, the default
//      keys of SpatialDomains/MeshGraph.cpp:1665-1681 ----
// GaussPoints::CalculatePoints / CalculateDerivMatrix for eGaussRadauMAlpha1Beta0
// (LibUtilities/Foundations/GaussPoints.cpp:119-121, 206-208, 235).
void radau_tables(int Q, double* z, double* w, double* D) {
  Polylib::zwgrjm(z, w, Q, 1.0, 0.0);
  Polylib::Dgrjm(D, z, Q, 1.0, 0.0);
}

// Basis::GenBasis eModified_B (LibUtilities/Foundations/Basis.cpp:423-507): the
// triangular mode index m(p, q), q fastest, 0 <= p < n, 0 <= q < n - p.
void modB_tables(int n, int Q, const double* z, const double* D, double* B, double* DB) {
  for (int i = 0; i < Q; ++i) {
    B[i] = 0.5 * (1 - z[i]);
    B[Q + i] = 0.5 * (1 + z[i]);
  }
  double* mode = B + 2 * Q;
  for (int q = 2; q < n; ++q, mode += Q) {  // p = 0, q >= 2
    Polylib::jacobfd(Q, z, mode, nullptr, q - 2, 1.0, 1.0);
    for (int i = 0; i < Q; ++i) mode[i] *= B[i] * B[Q + i];
  }
  for (int i = 0; i < Q; ++i) mode[i] = 0.5 * (1 - z[i]);  // p = 1, q = 0
  mode += Q;
  for (int q = 2; q < n; ++q, mode += Q) {  // p = 1, q >= 1
    Polylib::jacobfd(Q, z, mode, nullptr, q - 2, 1.0, 1.0);
    for (int i = 0; i < Q; ++i) mode[i] *= B[i] * B[Q + i];
  }
  const double* one_m_z_pow = B;
  const double* one_p_z = B + Q;
  for (int p = 2; p < n; ++p) {
    for (int i = 0; i < Q; ++i) mode[i] = B[i] * one_m_z_pow[i];
    one_m_z_pow = mode;
    mode += Q;
    for (int q = 1; q < n - p; ++q, mode += Q) {
      Polylib::jacobfd(Q, z, mode, nullptr, q - 1, 2 * p - 1, 1.0);
      for (int i = 0; i < Q; ++i) mode[i] *= one_m_z_pow[i] * one_p_z[i];
    }
  }
  const int nc = n * (n + 1) / 2;
  for (int m = 0; m < nc; ++m)
    for (int i = 0; i < Q; ++i) {
      double s = 0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * B[m * Q + k];
      DB[m * Q + i] = s;
    }
}

struct TriTables {
  vvec b0, db0, D0, w0, z0, b1, db1, D1, w1, z1;
};

// The tables the MatrixFree Helper holds (MatrixFreeOps/Operator.hpp:206-275): the
// Gauss-Radau weights carry the factor 0.5 of the collapsed map (:245-248).
TriTables make_tri_tables(int n) {
  const int Q0 = n + 1, Q1 = n, nc = n * (n + 1) / 2;
  std::vector<double> z0(Q0), w0(Q0), D0(Q0 * Q0), B0(n * Q0), DB0(n * Q0);
  std::vector<double> z1(Q1), w1(Q1), D1(Q1 * Q1), B1(nc * Q1), DB1(nc * Q1);
  gll_tables(Q0, z0.data(), w0.data(), D0.data());
  modA_tables(n, Q0, z0.data(), D0.data(), B0.data(), DB0.data());
  radau_tables(Q1, z1.data(), w1.data(), D1.data());
  modB_tables(n, Q1, z1.data(), D1.data(), B1.data(), DB1.data());
  TriTables t;
  t.b0.assign(B0.begin(), B0.end());
  t.db0.assign(DB0.begin(), DB0.end());
  t.D0.assign(D0.begin(), D0.end());
  t.w0.assign(w0.begin(), w0.end());
  t.z0.assign(z0.begin(), z0.end());
  t.b1.assign(B1.begin(), B1.end());
  t.db1.assign(DB1.begin(), DB1.end());
  t.D1.assign(D1.begin(), D1.end());
  for (double& v : w1) v *= 0.5;
  t.w1.assign(w1.begin(), w1.end());
  t.z1.assign(z1.begin(), z1.end());
  return t;
}

// BwdTrans / IProduct / PhysDeriv for triangles (MatrixFreeOps/BwdTrans.h:540-570,
// IProduct.h:560-590, PhysDeriv.h:470-500), CORRECT = true (eModified_A).
template <int N>
void tri_bwd(const TriTables& t, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) / 2, nq = (N + 1) * N;
  vvec tin(nc), tout(nq);
  vec_t wsp[N];
  for (int e = b0; e < b1; ++e) {
    load_interleave(in + (size_t)e * nc * W, nc, tin);
    BwdTransTriKernel<N, N, N + 1, N, true>(tin, t.b0, t.b1, wsp, tout);
    deinterleave_store(tout, nq, out + (size_t)e * nq * W);
  }
}

template <int N, bool DEF>
void tri_iprod(const TriTables& t, const Geo& g, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) / 2, nq = (N + 1) * N;
  vvec tin(nq), tout(nc);
  vec_t wsp[N];
  for (int e = b0; e < b1; ++e) {
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    IProductTriKernel<N, N, N + 1, N, true, false, false, DEF>(tin, t.b0, t.b1, t.w0, t.w1, jac_ptr, wsp, tout);
    deinterleave_store(tout, nc, out + (size_t)e * nc * W);
  }
}

template <int N, bool DEF>
void tri_deriv(const TriTables& t, const Geo& g, const double* in, double* o0, double* o1, int b0, int b1) {
  constexpr int nq = (N + 1) * N, ndf = 4;
  vvec tin(nq), a(nq), b(nq);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nq : ndf)];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    PhysDerivTriKernel<N + 1, N, DEF>(tin, t.z0, t.z1, t.D0, t.D1, df_ptr, a, b);
    deinterleave_store(a, nq, o0 + (size_t)e * nq * W);
    deinterleave_store(b, nq, o1 + (size_t)e * nq * W);
  }
}

// ---- Helmholtz: HelmholtzTriImpl (MatrixFreeOps/Helmholtz.h:290-330, 505-635) ----
template <int N, bool DEF>
void helm_tri(const TriTables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N, nc = N * (N + 1) / 2, nqTot = NQ0 * NQ1, ndf = 4;
  std::vector<double> h0(NQ0), h1(NQ1);
  for (int i = 0; i < NQ0; ++i) h0[i] = 0.5 * (1 + t.z0[i][0]);
  for (int j = 0; j < NQ1; ++j) h1[j] = 2.0 / (1 - t.z1[j][0]);
  vec_t wsp[NQ1 > N ? NQ1 : N];
  vvec tmpIn(nc), tmpOut(nc), bwd(nqTot), deriv0(nqTot), deriv1(nqTot);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in + (size_t)e * nc * W, nc, tmpIn);
    vec_t df0, df1, df2, df3, metric00, metric01, metric11;
    if (!DEF) {
      df0 = df_ptr[0];
      df1 = df_ptr[1];
      df2 = df_ptr[2];
      df3 = df_ptr[3];
    }
    BwdTransTriKernel<N, N, NQ0, NQ1, true>(tmpIn, t.b0, t.b1, wsp, bwd);
    IProductTriKernel<N, N, NQ0, NQ1, true, true, false, DEF>(bwd, t.b0, t.b1, t.w0, t.w1, jac_ptr, wsp, tmpOut,
                                                              lambda);
    PhysDerivTensor2DKernel<NQ0, NQ1>(bwd, t.D0, t.D1, deriv0, deriv1);
    for (int j = 0, cnt = 0; j < NQ1; ++j) {
      vec_t h1j = h1[j];
      for (int i = 0; i < NQ0; ++i, ++cnt) {
        if (DEF) {
          df0 = df_ptr[cnt * ndf];
          df1 = df_ptr[cnt * ndf + 1];
          df2 = df_ptr[cnt * ndf + 2];
          df3 = df_ptr[cnt * ndf + 3];
        }
        vec_t h0i = h0[i];
        metric00 = h1j * (df0 + h0i * df1);
        metric01 = metric00 * df1;
        metric00 = metric00 * metric00;
        vec_t tmp = h1j * (df2 + h0i * df3);
        metric01.fma(tmp, df3);
        metric00.fma(tmp, tmp);
        metric11 = df1 * df1;
        metric11.fma(df3, df3);
        vec_t d0 = deriv0[cnt];
        vec_t d1 = deriv1[cnt];
        tmp = metric00 * d0;
        tmp.fma(metric01, d1);
        bwd[cnt] = tmp;
        tmp = metric01 * d0;
        tmp.fma(metric11, d1);
        deriv0[cnt] = tmp;
      }
    }
    IProductTriKernel<N, N, NQ0, NQ1, true, false, true, DEF>(bwd, t.db0, t.b1, t.w0, t.w1, jac_ptr, wsp, tmpOut);
    IProductTriKernel<N, N, NQ0, NQ1, true, false, true, DEF>(deriv0, t.b0, t.db1, t.w0, t.w1, jac_ptr, wsp, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- IProductWRTDerivBaseTriImpl (MatrixFreeOps/IProductWRTDerivBase.h:671-1060), 2-D input ----
template <int N, bool DEF>
void iprd_tri(const TriTables& t, const Geo& g, const double* in0, const double* in1, double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N, nc = N * (N + 1) / 2, nqTot = NQ0 * NQ1, ndf = 4;
  vec_t sums_j[NQ1];
  vvec tmpIn0(nqTot), tmpIn1(nqTot), tmp0(nqTot), tmp1(nqTot), tmpOut(nc);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in0 + (size_t)e * nqTot * W, nqTot, tmpIn0);
    load_interleave(in1 + (size_t)e * nqTot * W, nqTot, tmpIn1);
    vec_t df0, df1, df2, df3;
    if (!DEF) {
      df0 = df_ptr[0];
      df1 = df_ptr[1];
      df2 = df_ptr[2];
      df3 = df_ptr[3];
    }
    for (int j = 0, cnt = 0; j < NQ1; ++j) {
      vec_t f0 = 2.0 / (1.0 - t.z1[j]);
      for (int i = 0; i < NQ0; ++i, ++cnt) {
        if (DEF) {
          df0 = df_ptr[cnt * ndf];
          df1 = df_ptr[cnt * ndf + 1];
          df2 = df_ptr[cnt * ndf + 2];
          df3 = df_ptr[cnt * ndf + 3];
        }
        vec_t tI0 = tmpIn0[cnt], tI1 = tmpIn1[cnt];
        vec_t t0 = df0 * tI0 + df2 * tI1;
        vec_t t1 = df1 * tI0 + df3 * tI1;
        vec_t hf1 = 0.5 * (1.0 + t.z0[i]);
        t0 *= f0;
        vec_t c1 = hf1 * t1;
        t0.fma(c1, f0);
        tmp0[cnt] = t0;
        tmp1[cnt] = t1;
      }
    }
    IProductTriKernel<N, N, NQ0, NQ1, true, false, false, DEF>(tmp0, t.db0, t.b1, t.w0, t.w1, jac_ptr, sums_j,
                                                               tmpOut);
    IProductTriKernel<N, N, NQ0, NQ1, true, false, true, DEF>(tmp1, t.b0, t.db1, t.w0, t.w1, jac_ptr, sums_j,
                                                              tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- tetrahedra: eModified_A (Q0 = n + 1 GLL), eModified_B (Q1 = n Gauss-Radau alpha 1),
//      eModified_C (Q2 = n Gauss-Radau alpha 2): the default keys of
//      SpatialDomains/MeshGraph.cpp:1683-1716 ----
// Basis::GenBasis eModified_C (Basis.cpp:512-566): phi^c_{pqr} = phi^b_{p+q,r}, i.e. for
// each p the ModifiedB rows from (p, 0) on, (n - p)(n - p + 1)/2 of them.
void modC_tables(int n, int Q, const double* z, const double* D, double* C, double* DC) {
  const int ncb = n * (n + 1) / 2;
  std::vector<double> B((size_t)ncb * Q), DB((size_t)ncb * Q);
  modB_tables(n, Q, z, D, B.data(), DB.data());
  int boff = 0, off = 0;
  for (int p = 0; p < n; ++p) {
    const int rows = (n - p) * (n - p + 1) / 2;
    std::copy(B.begin() + (size_t)boff * Q, B.begin() + (size_t)(boff + rows) * Q, C + (size_t)off * Q);
    boff += n - p;
    off += rows;
  }
  const int nct = n * (n + 1) * (n + 2) / 6;
  for (int m = 0; m < nct; ++m)
    for (int i = 0; i < Q; ++i) {
      double s = 0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * C[m * Q + k];
      DC[m * Q + i] = s;
    }
}

struct TetTables {
  vvec b0, db0, D0, w0, z0, b1, db1, D1, w1, z1, b2, db2, D2, w2, z2;
};

// The MatrixFree Helper's tables (Operator.hpp:206-275): Gauss-Radau weights times 0.5
// (alpha 1) and 0.25 (alpha 2).
TetTables make_tet_tables(int n) {
  const int Q0 = n + 1, Q = n, ncb = n * (n + 1) / 2, nct = n * (n + 1) * (n + 2) / 6;
  std::vector<double> z0(Q0), w0(Q0), D0(Q0 * Q0), B0(n * Q0), DB0(n * Q0);
  std::vector<double> z1(Q), w1(Q), D1(Q * Q), B1(ncb * Q), DB1(ncb * Q);
  std::vector<double> z2(Q), w2(Q), D2(Q * Q), B2((size_t)nct * Q), DB2((size_t)nct * Q);
  gll_tables(Q0, z0.data(), w0.data(), D0.data());
  modA_tables(n, Q0, z0.data(), D0.data(), B0.data(), DB0.data());
  radau_tables(Q, z1.data(), w1.data(), D1.data());
  modB_tables(n, Q, z1.data(), D1.data(), B1.data(), DB1.data());
  Polylib::zwgrjm(z2.data(), w2.data(), Q, 2.0, 0.0);  // GaussPoints.cpp eGaussRadauMAlpha2Beta0
  Polylib::Dgrjm(D2.data(), z2.data(), Q, 2.0, 0.0);
  modC_tables(n, Q, z2.data(), D2.data(), B2.data(), DB2.data());
  for (double& v : w1) v *= 0.5;
  for (double& v : w2) v *= 0.25;
  TetTables t;
  auto put = [](vvec& dst, const std::vector<double>& src) { dst.assign(src.begin(), src.end()); };
  put(t.b0, B0); put(t.db0, DB0); put(t.D0, D0); put(t.w0, w0); put(t.z0, z0);
  put(t.b1, B1); put(t.db1, DB1); put(t.D1, D1); put(t.w1, w1); put(t.z1, z1);
  put(t.b2, B2); put(t.db2, DB2); put(t.D2, D2); put(t.w2, w2); put(t.z2, z2);
  return t;
}

// BwdTrans / IProduct / PhysDeriv for tetrahedra (MatrixFreeOps/BwdTrans.h:1010-1045,
// IProduct.h:1730-1770, PhysDeriv.h:990-1030), CORRECT = true.
template <int N>
void tet_bwd(const TetTables& t, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) * (N + 2) / 6, nq = (N + 1) * N * N;
  vvec tin(nc), tout(nq);
  vec_t fpq[N * N], fp[N];
  for (int e = b0; e < b1; ++e) {
    load_interleave(in + (size_t)e * nc * W, nc, tin);
    BwdTransTetKernel<N, N, N, N + 1, N, N, true>(tin, t.b0, t.b1, t.b2, fpq, fp, tout);
    deinterleave_store(tout, nq, out + (size_t)e * nq * W);
  }
}

template <int N, bool DEF>
void tet_iprod(const TetTables& t, const Geo& g, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) * (N + 2) / 6, nq = (N + 1) * N * N;
  vvec tin(nq), tout(nc);
  vec_t wsp[N * N + N];
  for (int e = b0; e < b1; ++e) {
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    IProductTetKernel<N, N, N, N + 1, N, N, true, false, false, DEF>(tin, t.b0, t.b1, t.b2, t.w0, t.w1, t.w2, jac_ptr,
                                                                     wsp, tout);
    deinterleave_store(tout, nc, out + (size_t)e * nc * W);
  }
}

template <int N, bool DEF>
void tet_deriv(const TetTables& t, const Geo& g, const double* in, double* o0, double* o1, double* o2, int b0,
               int b1) {
  constexpr int nq = (N + 1) * N * N, ndf = 9;
  vvec tin(nq), d0(nq), d1(nq), d2(nq), a(nq), b(nq), c(nq);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nq : ndf)];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    PhysDerivTetKernel<N + 1, N, N, DEF>(tin, t.z0, t.z1, t.z2, t.D0, t.D1, t.D2, df_ptr, d0, d1, d2, a, b, c);
    deinterleave_store(a, nq, o0 + (size_t)e * nq * W);
    deinterleave_store(b, nq, o1 + (size_t)e * nq * W);
    deinterleave_store(c, nq, o2 + (size_t)e * nq * W);
  }
}

// ---- Helmholtz: HelmholtzTetImpl (MatrixFreeOps/Helmholtz.h:1970-2010, 2266-2448) ----
template <int N, bool DEF>
void helm_tet(const TetTables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N, NQ2 = N, nc = N * (N + 1) * (N + 2) / 6, nqTot = NQ0 * NQ1 * NQ2, ndf = 9;
  std::vector<double> h0(NQ0), h1(NQ1), h2(NQ1), h3(NQ2);
  for (int i = 0; i < NQ0; ++i) h0[i] = 0.5 * (1 + t.z0[i][0]);
  for (int j = 0; j < NQ1; ++j) {
    h1[j] = 0.5 * (1 + t.z1[j][0]);
    h2[j] = 2.0 / (1 - t.z1[j][0]);
  }
  for (int k = 0; k < NQ2; ++k) h3[k] = 2.0 / (1 - t.z2[k][0]);
  vec_t wsp1[NQ1 * NQ2 + NQ2], wsp2[N];
  vvec tmpIn(nc), tmpOut(nc), bwd(nqTot), deriv0(nqTot), deriv1(nqTot), deriv2(nqTot);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in + (size_t)e * nc * W, nc, tmpIn);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    BwdTransTetKernel<N, N, N, NQ0, NQ1, NQ2, true>(tmpIn, t.b0, t.b1, t.b2, wsp1, wsp2, bwd);
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, true, false, DEF>(bwd, t.b0, t.b1, t.b2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp1, tmpOut, lambda);
    PhysDerivTensor3DKernel<NQ0, NQ1, NQ2>(bwd, t.D0, t.D1, t.D2, deriv0, deriv1, deriv2);
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t vh3 = h3[k];
      for (int j = 0; j < NQ1; ++j) {
        vec_t vh1 = h1[j], vh2 = h2[j];
        vec_t h2h3 = vh2 * vh3, h1h3 = vh1 * vh3;
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t h0h2h3 = vec_t(h0[i]) * h2h3;
          vec_t tmp1 = h0h2h3 * (df1 + df2);
          tmp1.fma(df0, h2h3);
          vec_t tmp2 = h0h2h3 * (df4 + df5);
          tmp2.fma(df3, h2h3);
          vec_t tmp3 = h0h2h3 * (df7 + df8);
          tmp3.fma(df6, h2h3);
          vec_t g0 = tmp1 * tmp1;
          g0.fma(tmp2, tmp2);
          g0.fma(tmp3, tmp3);
          vec_t g4 = df2 * tmp1;
          g4.fma(df5, tmp2);
          g4.fma(df8, tmp3);
          vec_t tmp4 = df1 * vh3;
          tmp4.fma(df2, h1h3);
          vec_t tmp5 = df4 * vh3;
          tmp5.fma(df5, h1h3);
          vec_t tmp6 = df7 * vh3;
          tmp6.fma(df8, h1h3);
          vec_t g3 = tmp1 * tmp4;
          g3.fma(tmp2, tmp5);
          g3.fma(tmp3, tmp6);
          vec_t g1 = tmp4 * tmp4;
          g1.fma(tmp5, tmp5);
          g1.fma(tmp6, tmp6);
          vec_t g5 = df2 * tmp4;
          g5.fma(df5, tmp5);
          g5.fma(df8, tmp6);
          vec_t g2 = df2 * df2;
          g2.fma(df5, df5);
          g2.fma(df8, df8);
          vec_t d0 = deriv0[cnt], d1 = deriv1[cnt], d2 = deriv2[cnt];
          tmp1 = g0 * d0;
          tmp1.fma(g3, d1);
          tmp1.fma(g4, d2);
          deriv0[cnt] = tmp1;
          tmp2 = g3 * d0;
          tmp2.fma(g1, d1);
          tmp2.fma(g5, d2);
          deriv1[cnt] = tmp2;
          tmp3 = g4 * d0;
          tmp3.fma(g5, d1);
          tmp3.fma(g2, d2);
          deriv2[cnt] = tmp3;
        }
      }
    }
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv0, t.db0, t.b1, t.b2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp1, tmpOut);
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv1, t.b0, t.db1, t.b2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp1, tmpOut);
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv2, t.b0, t.b1, t.db2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp1, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- IProductWRTDerivBaseTetImpl (MatrixFreeOps/IProductWRTDerivBase.h:2212-2630) ----
template <int N, bool DEF>
void iprd_tet(const TetTables& t, const Geo& g, const double* in0, const double* in1, const double* in2, double* out,
              int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N, NQ2 = N, nc = N * (N + 1) * (N + 2) / 6, nqTot = NQ0 * NQ1 * NQ2, ndf = 9;
  vec_t wsp[NQ1 * NQ2 + NQ2];
  vvec tI0v(nqTot), tI1v(nqTot), tI2v(nqTot), tmp0(nqTot), tmp1(nqTot), tmp2(nqTot), tmpOut(nc);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in0 + (size_t)e * nqTot * W, nqTot, tI0v);
    load_interleave(in1 + (size_t)e * nqTot * W, nqTot, tI1v);
    load_interleave(in2 + (size_t)e * nqTot * W, nqTot, tI2v);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t f2 = 2.0 / (1.0 - t.z2[k]);
      for (int j = 0; j < NQ1; ++j) {
        vec_t z1l = t.z1[j];
        vec_t f3 = 0.5 * (1.0 + z1l);
        vec_t f0 = 2.0 * f2 / (1.0 - z1l);
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t a = tI0v[cnt], b = tI1v[cnt], c = tI2v[cnt];
          vec_t t0 = df0 * a + df3 * b + df6 * c;
          vec_t t1 = df1 * a + df4 * b + df7 * c;
          vec_t t2 = df2 * a + df5 * b + df8 * c;
          vec_t f1 = 0.5 * (1.0 + t.z0[i]);
          t0.fma(t1 + t2, f1);
          t0 *= f0;
          t1.fma(t2, f3);
          t1 *= f2;
          tmp0[cnt] = t0;
          tmp1[cnt] = t1;
          tmp2[cnt] = t2;
        }
      }
    }
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, false, DEF>(tmp0, t.db0, t.b1, t.b2, t.w0, t.w1, t.w2,
                                                                      jac_ptr, wsp, tmpOut);
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp1, t.b0, t.db1, t.b2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp, tmpOut);
    IProductTetKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp2, t.b0, t.b1, t.db2, t.w0, t.w1, t.w2,
                                                                     jac_ptr, wsp, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- prisms: eModified_A on Q0 = Q1 = n + 1 GLL points (directions 0, 1), eModified_B on
//      Q2 = n Gauss-Radau (alpha 1) points (direction 2, rows (p, r)): the default keys of
//      SpatialDomains/MeshGraph.cpp:1011-1045; modes (p, q, r), r fastest, r < n - p ----
struct PrismTables {
  vvec b0, db0, D0, w0, z0, b2, db2, D2, w2, z2;
};

PrismTables make_prism_tables(int n) {
  const int Q0 = n + 1, Q = n, npr = n * (n + 1) / 2;
  std::vector<double> z0(Q0), w0(Q0), D0(Q0 * Q0), B0(n * Q0), DB0(n * Q0);
  std::vector<double> z2(Q), w2(Q), D2(Q * Q), B2(npr * Q), DB2(npr * Q);
  gll_tables(Q0, z0.data(), w0.data(), D0.data());
  modA_tables(n, Q0, z0.data(), D0.data(), B0.data(), DB0.data());
  radau_tables(Q, z2.data(), w2.data(), D2.data());
  modB_tables(n, Q, z2.data(), D2.data(), B2.data(), DB2.data());
  for (double& v : w2) v *= 0.5;  // MatrixFreeOps/Operator.hpp:245-248
  PrismTables t;
  auto put = [](vvec& dst, const std::vector<double>& src) { dst.assign(src.begin(), src.end()); };
  put(t.b0, B0); put(t.db0, DB0); put(t.D0, D0); put(t.w0, w0); put(t.z0, z0);
  put(t.b2, B2); put(t.db2, DB2); put(t.D2, D2); put(t.w2, w2); put(t.z2, z2);
  return t;
}

// BwdTrans / IProduct / PhysDeriv for prisms (MatrixFreeOps/BwdTrans.h, IProduct.h:1070-1110,
// PhysDeriv.h), CORRECT = true; direction 1 uses the direction-0 tables.
template <int N>
void prism_bwd(const PrismTables& t, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * N * (N + 1) / 2, nq = (N + 1) * (N + 1) * N;
  vvec tin(nc), tout(nq);
  vec_t fpq[N * N], fp[N];
  for (int e = b0; e < b1; ++e) {
    load_interleave(in + (size_t)e * nc * W, nc, tin);
    BwdTransPrismKernel<N, N, N, N + 1, N + 1, N, true>(tin, t.b0, t.b0, t.b2, fpq, fp, tout);
    deinterleave_store(tout, nq, out + (size_t)e * nq * W);
  }
}

template <int N, bool DEF>
void prism_iprod(const PrismTables& t, const Geo& g, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * N * (N + 1) / 2, nq = (N + 1) * (N + 1) * N;
  vvec tin(nq), tout(nc);
  vec_t skj[(N + 1) * N], sk[N], cq[N];
  for (int e = b0; e < b1; ++e) {
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    IProductPrismKernel<N, N, N, N + 1, N + 1, N, true, false, false, DEF>(tin, t.b0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                           jac_ptr, skj, sk, cq, tout);
    deinterleave_store(tout, nc, out + (size_t)e * nc * W);
  }
}

template <int N, bool DEF>
void prism_deriv(const PrismTables& t, const Geo& g, const double* in, double* o0, double* o1, double* o2, int b0,
                 int b1) {
  constexpr int nq = (N + 1) * (N + 1) * N, ndf = 9;
  vvec tin(nq), a(nq), b(nq), c(nq);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nq : ndf)];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    PhysDerivPrismKernel<N + 1, N + 1, N, DEF>(tin, t.z0, t.z0, t.z2, t.D0, t.D0, t.D2, df_ptr, a, b, c);
    deinterleave_store(a, nq, o0 + (size_t)e * nq * W);
    deinterleave_store(b, nq, o1 + (size_t)e * nq * W);
    deinterleave_store(c, nq, o2 + (size_t)e * nq * W);
  }
}

// ---- Helmholtz: HelmholtzPrismImpl (MatrixFreeOps/Helmholtz.h:1003-1030, 1291-1440) ----
template <int N, bool DEF>
void helm_prism(const PrismTables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N + 1, NQ2 = N, nc = N * N * (N + 1) / 2, nqTot = NQ0 * NQ1 * NQ2, ndf = 9;
  std::vector<double> h0(NQ0), h1(NQ2);
  for (int i = 0; i < NQ0; ++i) h0[i] = 0.5 * (1 + t.z0[i][0]);
  for (int k = 0; k < NQ2; ++k) h1[k] = 2.0 / (1 - t.z2[k][0]);
  vec_t wsp1[NQ1 * NQ2], wsp2[NQ2], wsp3[N];
  vvec tmpIn(nc), tmpOut(nc), bwd(nqTot), deriv0(nqTot), deriv1(nqTot), deriv2(nqTot);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in + (size_t)e * nc * W, nc, tmpIn);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    BwdTransPrismKernel<N, N, N, NQ0, NQ1, NQ2, true>(tmpIn, t.b0, t.b0, t.b2, wsp1, wsp2, bwd);
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, true, false, DEF>(bwd, t.b0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, wsp1, wsp2, wsp3, tmpOut, lambda);
    PhysDerivTensor3DKernel<NQ0, NQ1, NQ2>(bwd, t.D0, t.D0, t.D2, deriv0, deriv1, deriv2);
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t vh1 = h1[k];
      for (int j = 0; j < NQ1; ++j) {
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          vec_t vh0 = h0[i];
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t tmp1 = vh1 * (vh0 * df2 + df0);
          vec_t tmp2 = vh1 * (vh0 * df5 + df3);
          vec_t tmp3 = vh1 * (vh0 * df8 + df6);
          vec_t g0 = tmp1 * tmp1;
          g0.fma(tmp2, tmp2);
          g0.fma(tmp3, tmp3);
          vec_t g3 = df1 * tmp1;
          g3.fma(df4, tmp2);
          g3.fma(df7, tmp3);
          vec_t g4 = df2 * tmp1;
          g4.fma(df5, tmp2);
          g4.fma(df8, tmp3);
          vec_t g1 = df1 * df1;
          g1.fma(df4, df4);
          g1.fma(df7, df7);
          vec_t g2 = df2 * df2;
          g2.fma(df5, df5);
          g2.fma(df8, df8);
          vec_t g5 = df1 * df2;
          g5.fma(df4, df5);
          g5.fma(df7, df8);
          vec_t d0 = deriv0[cnt], d1 = deriv1[cnt], d2 = deriv2[cnt];
          tmp1 = g0 * d0;
          tmp1.fma(g3, d1);
          tmp1.fma(g4, d2);
          deriv0[cnt] = tmp1;
          tmp2 = g3 * d0;
          tmp2.fma(g1, d1);
          tmp2.fma(g5, d2);
          deriv1[cnt] = tmp2;
          tmp3 = g4 * d0;
          tmp3.fma(g5, d1);
          tmp3.fma(g2, d2);
          deriv2[cnt] = tmp3;
        }
      }
    }
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv0, t.db0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, wsp1, wsp2, wsp3, tmpOut);
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv1, t.b0, t.db0, t.b2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, wsp1, wsp2, wsp3, tmpOut);
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv2, t.b0, t.b0, t.db2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, wsp1, wsp2, wsp3, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- IProductWRTDerivBasePrismImpl (MatrixFreeOps/IProductWRTDerivBase.h:1660-1760) ----
template <int N, bool DEF>
void iprd_prism(const PrismTables& t, const Geo& g, const double* in0, const double* in1, const double* in2,
                double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N + 1, NQ2 = N, nc = N * N * (N + 1) / 2, nqTot = NQ0 * NQ1 * NQ2, ndf = 9;
  vec_t skj[NQ1 * NQ2], sk[NQ2], cq[N];
  vvec a0(nqTot), a1(nqTot), a2(nqTot), tmp0(nqTot), tmp1(nqTot), tmp2(nqTot), tmpOut(nc);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in0 + (size_t)e * nqTot * W, nqTot, a0);
    load_interleave(in1 + (size_t)e * nqTot * W, nqTot, a1);
    load_interleave(in2 + (size_t)e * nqTot * W, nqTot, a2);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t f0 = 2.0 / (1.0 - t.z2[k]);
      for (int j = 0; j < NQ1; ++j) {
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t tI0 = a0[cnt], tI1 = a1[cnt], tI2 = a2[cnt];
          vec_t t0 = df0 * tI0 + df3 * tI1 + df6 * tI2;
          vec_t t1 = df1 * tI0 + df4 * tI1 + df7 * tI2;
          vec_t t2 = df2 * tI0 + df5 * tI1 + df8 * tI2;
          vec_t hf1 = 0.5 * (1.0 + t.z0[i]);
          t0 *= f0;
          vec_t f1t2 = hf1 * t2;
          t0.fma(f1t2, f0);
          tmp0[cnt] = t0;
          tmp1[cnt] = t1;
          tmp2[cnt] = t2;
        }
      }
    }
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, false, DEF>(tmp0, t.db0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                        jac_ptr, skj, sk, cq, tmpOut);
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp1, t.b0, t.db0, t.b2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, skj, sk, cq, tmpOut);
    IProductPrismKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp2, t.b0, t.b0, t.db2, t.w0, t.w0, t.w2,
                                                                       jac_ptr, skj, sk, cq, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- pyramids: eModified_A on Q0 = Q1 = n + 1 GLL points (directions 0, 1),
//      eModifiedPyr_C on Q2 = n Gauss-Radau (alpha 2) points (direction 2): the default keys
//      of SpatialDomains/MeshGraph.cpp:1719-1745; modes (p, q, r), r fastest,
//      r < n - max(p, q) ----
// Basis::GenBasis eModifiedPyr_C (LibUtilities/Foundations/Basis.cpp:568-672): rows of the
// ModifiedB table for p <= 1 and for q <= 1, the face-0 rows ((1-z)/2)^(p+q-2) and the
// interior rows ((1-z)/2)^(p+q-2) (1+z)/2 P_{r-1}^{(2p+2q-3,1)} for p, q >= 2.
void modPyrC_tables(int n, int Q, const double* z, const double* D, double* C, double* DC) {
  const int ncb = n * (n + 1) / 2, ncp = n * (n + 1) * (2 * n + 1) / 6;
  std::vector<double> B((size_t)ncb * Q), DB((size_t)ncb * Q);
  modB_tables(n, Q, z, D, B.data(), DB.data());
  size_t off = 0, boff = 0;
  auto copy_rows = [&](size_t rows) {
    std::copy(B.begin() + boff * Q, B.begin() + (boff + rows) * Q, C + off * Q);
    off += rows;
  };
  copy_rows((size_t)n * (n + 1) / 2);  // p = 0: all (q, r)
  boff += n;
  copy_rows(n - 1);                    // p = 1, q = 0
  copy_rows((size_t)(n - 1) * n / 2);  // p = 1, q >= 1
  boff += n - 1;
  for (int p = 2; p < n; ++p) {
    copy_rows(n - p);  // q = 0
    boff -= 0;
    std::copy(B.begin() + boff * Q, B.begin() + (boff + n - p) * Q, C + off * Q);  // q = 1: same rows
    off += n - p;
    boff += n - p;
    for (int q = 2; q < n; ++q) {
      double* mode = C + off * Q;
      for (int i = 0; i < Q; ++i) mode[i] = std::pow(B[i], p + q - 2);
      const double* one_m_z_pow = mode;
      ++off;
      for (int r = 1; r < n - std::max(p, q); ++r, ++off) {
        double* md = C + off * Q;
        Polylib::jacobfd(Q, z, md, nullptr, r - 1, 2 * p + 2 * q - 3, 1.0);
        for (int i = 0; i < Q; ++i) md[i] *= one_m_z_pow[i] * B[Q + i];
      }
    }
  }
  for (int m = 0; m < ncp; ++m)
    for (int i = 0; i < Q; ++i) {
      double s = 0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * C[m * Q + k];
      DC[m * Q + i] = s;
    }
}

struct PyrTables {
  vvec b0, db0, D0, w0, z0, b2, db2, D2, w2, z2;
};

PyrTables make_pyr_tables(int n) {
  const int Q0 = n + 1, Q = n, ncp = n * (n + 1) * (2 * n + 1) / 6;
  std::vector<double> z0(Q0), w0(Q0), D0(Q0 * Q0), B0(n * Q0), DB0(n * Q0);
  std::vector<double> z2(Q), w2(Q), D2(Q * Q), B2((size_t)ncp * Q), DB2((size_t)ncp * Q);
  gll_tables(Q0, z0.data(), w0.data(), D0.data());
  modA_tables(n, Q0, z0.data(), D0.data(), B0.data(), DB0.data());
  Polylib::zwgrjm(z2.data(), w2.data(), Q, 2.0, 0.0);
  Polylib::Dgrjm(D2.data(), z2.data(), Q, 2.0, 0.0);
  modPyrC_tables(n, Q, z2.data(), D2.data(), B2.data(), DB2.data());
  for (double& v : w2) v *= 0.25;  // MatrixFreeOps/Operator.hpp:249-251
  PyrTables t;
  auto put = [](vvec& dst, const std::vector<double>& src) { dst.assign(src.begin(), src.end()); };
  put(t.b0, B0); put(t.db0, DB0); put(t.D0, D0); put(t.w0, w0); put(t.z0, z0);
  put(t.b2, B2); put(t.db2, DB2); put(t.D2, D2); put(t.w2, w2); put(t.z2, z2);
  return t;
}

template <int N>
void pyr_bwd(const PyrTables& t, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) * (2 * N + 1) / 6, nq = (N + 1) * (N + 1) * N;
  vvec tin(nc), tout(nq);
  vec_t fpq[(N + 1) * N], fp[N];
  for (int e = b0; e < b1; ++e) {
    load_interleave(in + (size_t)e * nc * W, nc, tin);
    BwdTransPyrKernel<N, N, N, N + 1, N + 1, N, true>(tin, t.b0, t.b0, t.b2, fpq, fp, tout);
    deinterleave_store(tout, nq, out + (size_t)e * nq * W);
  }
}

template <int N, bool DEF>
void pyr_iprod(const PyrTables& t, const Geo& g, const double* in, double* out, int b0, int b1) {
  constexpr int nc = N * (N + 1) * (2 * N + 1) / 6, nq = (N + 1) * (N + 1) * N;
  vvec tin(nq), tout(nc);
  vec_t skj[(N + 1) * N], sk[N];
  for (int e = b0; e < b1; ++e) {
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nq] : &g.jac[e];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    IProductPyrKernel<N, N, N, N + 1, N + 1, N, true, false, false, DEF>(tin, t.b0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                         jac_ptr, skj, sk, tout);
    deinterleave_store(tout, nc, out + (size_t)e * nc * W);
  }
}

template <int N, bool DEF>
void pyr_deriv(const PyrTables& t, const Geo& g, const double* in, double* o0, double* o1, double* o2, int b0,
               int b1) {
  constexpr int nq = (N + 1) * (N + 1) * N, ndf = 9;
  vvec tin(nq), a(nq), b(nq), c(nq);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nq : ndf)];
    load_interleave(in + (size_t)e * nq * W, nq, tin);
    PhysDerivPyrKernel<N + 1, N + 1, N, DEF>(tin, t.z0, t.z0, t.z2, t.D0, t.D0, t.D2, df_ptr, a, b, c);
    deinterleave_store(a, nq, o0 + (size_t)e * nq * W);
    deinterleave_store(b, nq, o1 + (size_t)e * nq * W);
    deinterleave_store(c, nq, o2 + (size_t)e * nq * W);
  }
}

// ---- Helmholtz: HelmholtzPyrImpl (MatrixFreeOps/Helmholtz.h:1480-1510, 1770-1960) ----
template <int N, bool DEF>
void helm_pyr(const PyrTables& t, const Geo& g, double lambda, const double* in, double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N + 1, NQ2 = N, nc = N * (N + 1) * (2 * N + 1) / 6, nqTot = NQ0 * NQ1 * NQ2,
                ndf = 9;
  std::vector<double> h0(NQ0), h2(NQ2);
  for (int i = 0; i < NQ0; ++i) h0[i] = 0.5 * (1 + t.z0[i][0]);
  for (int k = 0; k < NQ2; ++k) h2[k] = 2.0 / (1 - t.z2[k][0]);
  vec_t wsp1[NQ1 * NQ2], wsp2[NQ2];
  vvec tmpIn(nc), tmpOut(nc), bwd(nqTot), deriv0(nqTot), deriv1(nqTot), deriv2(nqTot);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in + (size_t)e * nc * W, nc, tmpIn);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    BwdTransPyrKernel<N, N, N, NQ0, NQ1, NQ2, true>(tmpIn, t.b0, t.b0, t.b2, wsp1, wsp2, bwd);
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, true, false, DEF>(bwd, t.b0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, wsp1, wsp2, tmpOut, lambda);
    PhysDerivTensor3DKernel<NQ0, NQ1, NQ2>(bwd, t.D0, t.D0, t.D2, deriv0, deriv1, deriv2);
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t vh2 = h2[k];
      for (int j = 0; j < NQ1; ++j) {
        vec_t vh1 = 0.5 * (1 + t.z0[j][0]);
        vec_t h1h2 = vh1 * vh2;
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          vec_t h0h2 = vec_t(h0[i]) * vh2;
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t tmp0 = vh2 * df0;
          tmp0.fma(h0h2, df2);
          vec_t tmp1 = vh2 * df3;
          tmp1.fma(h0h2, df5);
          vec_t tmp2 = vh2 * df6;
          tmp2.fma(h0h2, df8);
          vec_t tmp3 = vh2 * df1;
          tmp3.fma(h1h2, df2);
          vec_t tmp4 = vh2 * df4;
          tmp4.fma(h1h2, df5);
          vec_t tmp5 = vh2 * df7;
          tmp5.fma(h1h2, df8);
          vec_t g0 = tmp0 * tmp0;
          g0.fma(tmp1, tmp1);
          g0.fma(tmp2, tmp2);
          vec_t g1 = tmp3 * tmp3;
          g1.fma(tmp4, tmp4);
          g1.fma(tmp5, tmp5);
          vec_t g2 = df2 * df2;
          g2.fma(df5, df5);
          g2.fma(df8, df8);
          vec_t g3 = tmp0 * tmp3;
          g3.fma(tmp1, tmp4);
          g3.fma(tmp2, tmp5);
          vec_t g4 = df2 * tmp0;
          g4.fma(df5, tmp1);
          g4.fma(df8, tmp2);
          vec_t g5 = df2 * tmp3;
          g5.fma(df5, tmp4);
          g5.fma(df8, tmp5);
          vec_t d0 = deriv0[cnt], d1 = deriv1[cnt], d2 = deriv2[cnt];
          tmp1 = g0 * d0;
          tmp1.fma(g3, d1);
          tmp1.fma(g4, d2);
          deriv0[cnt] = tmp1;
          tmp2 = g3 * d0;
          tmp2.fma(g1, d1);
          tmp2.fma(g5, d2);
          deriv1[cnt] = tmp2;
          tmp3 = g4 * d0;
          tmp3.fma(g5, d1);
          tmp3.fma(g2, d2);
          deriv2[cnt] = tmp3;
        }
      }
    }
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv0, t.db0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, wsp1, wsp2, tmpOut);
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv1, t.b0, t.db0, t.b2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, wsp1, wsp2, tmpOut);
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(deriv2, t.b0, t.b0, t.db2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, wsp1, wsp2, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// ---- IProductWRTDerivBasePyrImpl (MatrixFreeOps/IProductWRTDerivBase.h:2070-2200) ----
template <int N, bool DEF>
void iprd_pyr(const PyrTables& t, const Geo& g, const double* in0, const double* in1, const double* in2,
              double* out, int b0, int b1) {
  constexpr int NQ0 = N + 1, NQ1 = N + 1, NQ2 = N, nc = N * (N + 1) * (2 * N + 1) / 6, nqTot = NQ0 * NQ1 * NQ2,
                ndf = 9;
  vec_t skj[NQ1 * NQ2], sk[NQ2];
  vvec a0(nqTot), a1(nqTot), a2(nqTot), tmp0(nqTot), tmp1(nqTot), tmp2(nqTot), tmpOut(nc);
  for (int e = b0; e < b1; ++e) {
    const vec_t* df_ptr = &g.df[(size_t)e * (DEF ? ndf * nqTot : ndf)];
    const vec_t* jac_ptr = DEF ? &g.jac[(size_t)e * nqTot] : &g.jac[e];
    load_interleave(in0 + (size_t)e * nqTot * W, nqTot, a0);
    load_interleave(in1 + (size_t)e * nqTot * W, nqTot, a1);
    load_interleave(in2 + (size_t)e * nqTot * W, nqTot, a2);
    vec_t df0, df1, df2, df3, df4, df5, df6, df7, df8;
    if (!DEF) {
      df0 = df_ptr[0]; df1 = df_ptr[1]; df2 = df_ptr[2];
      df3 = df_ptr[3]; df4 = df_ptr[4]; df5 = df_ptr[5];
      df6 = df_ptr[6]; df7 = df_ptr[7]; df8 = df_ptr[8];
    }
    for (int k = 0, cnt = 0; k < NQ2; ++k) {
      vec_t f0 = 2.0 / (1.0 - t.z2[k]);
      for (int j = 0; j < NQ1; ++j) {
        vec_t hf2 = 0.5 * (1.0 + t.z0[j]);
        for (int i = 0; i < NQ0; ++i, ++cnt) {
          if (DEF) {
            df0 = df_ptr[cnt * ndf]; df1 = df_ptr[cnt * ndf + 1]; df2 = df_ptr[cnt * ndf + 2];
            df3 = df_ptr[cnt * ndf + 3]; df4 = df_ptr[cnt * ndf + 4]; df5 = df_ptr[cnt * ndf + 5];
            df6 = df_ptr[cnt * ndf + 6]; df7 = df_ptr[cnt * ndf + 7]; df8 = df_ptr[cnt * ndf + 8];
          }
          vec_t tI0 = a0[cnt], tI1 = a1[cnt], tI2 = a2[cnt];
          vec_t t0 = df0 * tI0 + df3 * tI1 + df6 * tI2;
          vec_t t1 = df1 * tI0 + df4 * tI1 + df7 * tI2;
          vec_t t2 = df2 * tI0 + df5 * tI1 + df8 * tI2;
          t0 *= f0;
          vec_t hf1 = 0.5 * (1.0 + t.z0[i]);
          vec_t f1t2 = hf1 * t2;
          t0.fma(f1t2, f0);
          t1 *= f0;
          f1t2 = hf2 * t2;
          t1.fma(f1t2, f0);
          tmp0[cnt] = t0;
          tmp1[cnt] = t1;
          tmp2[cnt] = t2;
        }
      }
    }
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, false, DEF>(tmp0, t.db0, t.b0, t.b2, t.w0, t.w0, t.w2,
                                                                      jac_ptr, skj, sk, tmpOut);
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp1, t.b0, t.db0, t.b2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, skj, sk, tmpOut);
    IProductPyrKernel<N, N, N, NQ0, NQ1, NQ2, true, false, true, DEF>(tmp2, t.b0, t.b0, t.db2, t.w0, t.w0, t.w2,
                                                                     jac_ptr, skj, sk, tmpOut);
    deinterleave_store(tmpOut, nc, out + (size_t)e * nc * W);
  }
}

// Runs CALL(N) for N in 2..12 (triangles: Q0 = N + 1, Q1 = N).
#define TRI12_DISPATCH(n, CALL) \
  switch (n) {                  \
    case 2: CALL(2); return 0;  \
    case 3: CALL(3); return 0;  \
    case 4: CALL(4); return 0;  \
    case 5: CALL(5); return 0;  \
    case 6: CALL(6); return 0;  \
    case 7: CALL(7); return 0;  \
    case 8: CALL(8); return 0;  \
    case 9: CALL(9); return 0;  \
    case 10: CALL(10); return 0; \
    case 11: CALL(11); return 0; \
    case 12: CALL(12); return 0; \
    default: break;             \
  }                             \
  return 1;

// Runs CALL(N) for N in 2..10 (tetrahedra, prisms, pyramids).
#define TRI_DISPATCH(n, CALL)   \
  switch (n) {                  \
    case 2: CALL(2); return 0;  \
    case 3: CALL(3); return 0;  \
    case 4: CALL(4); return 0;  \
    case 5: CALL(5); return 0;  \
    case 6: CALL(6); return 0;  \
    case 7: CALL(7); return 0;  \
    case 8: CALL(8); return 0;  \
    case 9: CALL(9); return 0;  \
    case 10: CALL(10); return 0; \
    default: break;             \
  }                             \
  return 1;

// Runs fn<N, Q=N+1>(args...) for N in 2..10 (P = 1..9, Q = P + 2).
#define ORACLE_DISPATCH(n, Q, CALL)                                    \
  switch (n) {                                                         \
    case 2: if (Q == 3) { CALL(2, 3); return 0; } break;               \
    case 3: if (Q == 4) { CALL(3, 4); return 0; } break;               \
    case 4: if (Q == 5) { CALL(4, 5); return 0; } break;               \
    case 5: if (Q == 6) { CALL(5, 6); return 0; } break;               \
    case 6: if (Q == 7) { CALL(6, 7); return 0; } break;               \
    case 7: if (Q == 8) { CALL(7, 8); return 0; } break;               \
    case 8: if (Q == 9) { CALL(8, 9); return 0; } break;               \
    case 9: if (Q == 10) { CALL(9, 10); return 0; } break;             \
    case 10: if (Q == 11) { CALL(10, 11); return 0; } break;           \
    default: break;                                                    \
  }                                                                    \
  return 1;

}  // namespace

extern "C" {

int ref_simd_width() { return W; }

int ref_gll(int Q, double* z, double* w, double* D) {
  gll_tables(Q, z, w, D);
  return 0;
}

int ref_modA(int n, int Q, double* B, double* DB) {
  std::vector<double> z(Q), w(Q), D(Q * Q);
  gll_tables(Q, z.data(), w.data(), D.data());
  modA_tables(n, Q, z.data(), D.data(), B, DB);
  return 0;
}

// Element-local Helmholtz apply, reference layouts; E must be a multiple of W.
int ref_helmholtz(int dim, int n, int Q, int E, const double* jac, const double* df, int deformed, double lambda,
                  const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  Tables t = make_tables(n, Q);
  Geo g = interleave(dim, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define HCALL(NN, QQ)                                                                             \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                                             \
    if (dim == 2) {                                                                               \
      if (deformed) helm_quad<NN, QQ, true>(t, g, lambda, in, out, b0, b1);                       \
      else helm_quad<NN, QQ, false>(t, g, lambda, in, out, b0, b1);                               \
    } else {                                                                                      \
      if (deformed) helm_hex<NN, QQ, true>(t, g, lambda, in, out, b0, b1);                        \
      else helm_hex<NN, QQ, false>(t, g, lambda, in, out, b0, b1);                                \
    }                                                                                             \
  })
  ORACLE_DISPATCH(n, Q, HCALL)
#undef HCALL
}

int ref_bwdtrans(int dim, int n, int Q, int E, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  Tables t = make_tables(n, Q);
  const int nb = E / W;
#define BCALL(NN, QQ) parallel_blocks(nb, nthreads, [&](int b0, int b1) { bwd_op<NN, QQ>(dim, t, in, out, b0, b1); })
  ORACLE_DISPATCH(n, Q, BCALL)
#undef BCALL
}

int ref_iproduct(int dim, int n, int Q, int E, const double* jac, int deformed, const double* in, double* out,
                 int nthreads) {
  if (E % W) return 2;
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  Tables t = make_tables(n, Q);
  std::vector<double> dfz((size_t)dim * dim * E * (deformed ? nq : 1), 0.0);
  Geo g = interleave(dim, nq, E, E, jac, dfz.data(), deformed != 0);
  const int nb = E / W;
#define ICALL(NN, QQ)                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                 \
    if (deformed) iprod_op<NN, QQ, true>(dim, t, g, in, out, b0, b1); \
    else iprod_op<NN, QQ, false>(dim, t, g, in, out, b0, b1);         \
  })
  ORACLE_DISPATCH(n, Q, ICALL)
#undef ICALL
}

int ref_physderiv(int dim, int n, int Q, int E, const double* df, int deformed, const double* in, double* o0,
                  double* o1, double* o2, int nthreads) {
  if (E % W) return 2;
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  Tables t = make_tables(n, Q);
  std::vector<double> jz((size_t)E * (deformed ? nq : 1), 1.0);
  Geo g = interleave(dim, nq, E, E, jz.data(), df, deformed != 0);
  const int nb = E / W;
#define DCALL(NN, QQ)                                                                  \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                                  \
    if (deformed) deriv_op<NN, QQ, true>(dim, t, g, in, o0, o1, o2, b0, b1);           \
    else deriv_op<NN, QQ, false>(dim, t, g, in, o0, o1, o2, b0, b1);                   \
  })
  ORACLE_DISPATCH(n, Q, DCALL)
#undef DCALL
}

// Reference CG solve for the CPU baseline: the single-reduction PCG of
// LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp:104-263 with Jacobi preconditioning
// (MultiRegions/PreconditionerDiagonal.cpp:191-206), the matrix-free operator of
// GlobalLinSysIterativeFull::v_DoMatrixMultiply (:215-257) = GlobalToLocal, element
// Helmholtz, Assemble (AssemblyMapCG.cpp:2853-2910). x holds the solution on return.
// Returns the iteration count (>=0), or -1 if max_iter was reached.
int ref_cg_solve(int dim, int n, int Q, int E, const double* jac, const double* df, int deformed, double lambda,
                 const int* l2g, const double* sign, int nglobal, int ndir, const double* dinv, const double* rhs,
                 double* x, double tol, int max_iter, int nthreads, double* final_eps) {
  if (E % W) return -2;
  const int nm = dim == 2 ? n * n : n * n * n;
  const int nq = dim == 2 ? Q * Q : Q * Q * Q;
  const size_t nloc = (size_t)E * nm;
  Tables t = make_tables(n, Q);
  Geo g = interleave(dim, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
  const int nnd = nglobal - ndir;
  std::vector<double> wA(nglobal, 0.0), sA(nglobal, 0.0), p(nnd, 0.0), r(nnd), q(nnd, 0.0);
  std::vector<double> loc_in(nloc), loc_out(nloc);

  auto apply = [&](const std::vector<double>& gin, std::vector<double>& gout) -> int {
    for (size_t i = 0; i < nloc; ++i) loc_in[i] = sign[i] * gin[l2g[i]];
    int rc = 1;
#define CGCALL(NN, QQ)                                                                                  \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                                                   \
    if (dim == 2) {                                                                                     \
      if (deformed) helm_quad<NN, QQ, true>(t, g, lambda, loc_in.data(), loc_out.data(), b0, b1);       \
      else helm_quad<NN, QQ, false>(t, g, lambda, loc_in.data(), loc_out.data(), b0, b1);               \
    } else {                                                                                            \
      if (deformed) helm_hex<NN, QQ, true>(t, g, lambda, loc_in.data(), loc_out.data(), b0, b1);        \
      else helm_hex<NN, QQ, false>(t, g, lambda, loc_in.data(), loc_out.data(), b0, b1);                \
    }                                                                                                   \
  });                                                                                                   \
  rc = 0;
    [&]() -> int { ORACLE_DISPATCH(n, Q, CGCALL) }();
#undef CGCALL
    rc = 0;
    std::fill(gout.begin(), gout.end(), 0.0);
    for (size_t i = 0; i < nloc; ++i) gout[l2g[i]] += sign[i] * loc_out[i];
    return rc;
  };
  auto dot = [&](const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i < nnd; ++i) s += a[i] * b[i];
    return s;
  };
  for (int i = 0; i < nnd; ++i) r[i] = rhs[ndir + i];
  for (int i = 0; i < nnd; ++i) x[ndir + i] = 0.0;
  double eps = dot(r.data(), r.data());
  double rhs_mag = 0;
  for (int i = 0; i < nglobal; ++i) rhs_mag += rhs[i] * rhs[i];
  rhs_mag = rhs_mag > 1e-6 ? rhs_mag : 1.0;
  if (eps < tol * tol * rhs_mag) {
    if (final_eps) *final_eps = eps;
    return 0;
  }
  for (int i = 0; i < nnd; ++i) wA[ndir + i] = r[i] * dinv[i];
  apply(wA, sA);
  double rho = dot(r.data(), wA.data() + ndir), mu = dot(sA.data() + ndir, wA.data() + ndir);
  double beta = 0.0, alpha = rho / mu;
  int iters = 1, k = 0;
  while (true) {
    if (k >= max_iter) {
      if (final_eps) *final_eps = eps;
      return -1;
    }
    for (int i = 0; i < nnd; ++i) {
      p[i] = beta * p[i] + wA[ndir + i];
      q[i] = beta * q[i] + sA[ndir + i];
      x[ndir + i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    for (int i = 0; i < nnd; ++i) wA[ndir + i] = r[i] * dinv[i];
    apply(wA, sA);
    double rho_new = dot(r.data(), wA.data() + ndir);
    mu = dot(sA.data() + ndir, wA.data() + ndir);
    eps = dot(r.data(), r.data());
    iters++;
    if (eps < tol * tol * rhs_mag) break;
    beta = rho_new / rho;
    alpha = rho_new / (mu - rho_new * beta / alpha);
    rho = rho_new;
    k++;
  }
  if (final_eps) *final_eps = eps;
  return iters;
}

// ---- triangles ----
// Tables as the reference's Basis objects hold them (GetZ/GetW/GetD/GetBdata/GetDbdata):
// direction 0 GLL + eModified_A (n modes, Q0 = n + 1), direction 1 Gauss-Radau (alpha 1,
// beta 0) + eModified_B (n (n + 1) / 2 modes, Q1 = n); w1 without the factor 0.5.
int ref_tri_tables(int n, double* z0, double* w0, double* D0, double* B0, double* DB0, double* z1, double* w1,
                   double* D1, double* B1, double* DB1) {
  const int Q0 = n + 1, Q1 = n;
  gll_tables(Q0, z0, w0, D0);
  modA_tables(n, Q0, z0, D0, B0, DB0);
  radau_tables(Q1, z1, w1, D1);
  modB_tables(n, Q1, z1, D1, B1, DB1);
  return 0;
}

int ref_tri_bwdtrans(int n, int E, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  TriTables t = make_tri_tables(n);
  const int nb = E / W;
#define TB(NN) parallel_blocks(nb, nthreads, [&](int b0, int b1) { tri_bwd<NN>(t, in, out, b0, b1); })
  TRI12_DISPATCH(n, TB)
#undef TB
}

int ref_tri_iproduct(int n, int E, const double* jac, int deformed, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n;
  TriTables t = make_tri_tables(n);
  std::vector<double> dfz((size_t)4 * E * (deformed ? nq : 1), 0.0);
  Geo g = interleave(2, nq, E, E, jac, dfz.data(), deformed != 0);
  const int nb = E / W;
#define TI(NN)                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {            \
    if (deformed) tri_iprod<NN, true>(t, g, in, out, b0, b1);    \
    else tri_iprod<NN, false>(t, g, in, out, b0, b1);            \
  })
  TRI12_DISPATCH(n, TI)
#undef TI
}

int ref_tri_physderiv(int n, int E, const double* df, int deformed, const double* in, double* o0, double* o1,
                      int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n;
  TriTables t = make_tri_tables(n);
  std::vector<double> jz((size_t)E * (deformed ? nq : 1), 1.0);
  Geo g = interleave(2, nq, E, E, jz.data(), df, deformed != 0);
  const int nb = E / W;
#define TD(NN)                                                          \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                   \
    if (deformed) tri_deriv<NN, true>(t, g, in, o0, o1, b0, b1);        \
    else tri_deriv<NN, false>(t, g, in, o0, o1, b0, b1);                \
  })
  TRI12_DISPATCH(n, TD)
#undef TD
}

int ref_tri_helmholtz(int n, int E, const double* jac, const double* df, int deformed, double lambda,
                      const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n;
  TriTables t = make_tri_tables(n);
  Geo g = interleave(2, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define TH(NN)                                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                          \
    if (deformed) helm_tri<NN, true>(t, g, lambda, in, out, b0, b1);           \
    else helm_tri<NN, false>(t, g, lambda, in, out, b0, b1);                   \
  })
  TRI12_DISPATCH(n, TH)
#undef TH
}

int ref_tri_iproduct_deriv(int n, int E, const double* jac, const double* df, int deformed, const double* in0,
                           const double* in1, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n;
  TriTables t = make_tri_tables(n);
  Geo g = interleave(2, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define TP(NN)                                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                          \
    if (deformed) iprd_tri<NN, true>(t, g, in0, in1, out, b0, b1);             \
    else iprd_tri<NN, false>(t, g, in0, in1, out, b0, b1);                     \
  })
  TRI12_DISPATCH(n, TP)
#undef TP
}

// ---- tetrahedra ----
// Tables as the reference's Basis objects hold them (weights without the collapsed factors).
int ref_tet_tables(int n, double* z0, double* w0, double* D0, double* B0, double* DB0, double* z1, double* w1,
                   double* D1, double* B1, double* DB1, double* z2, double* w2, double* D2, double* B2, double* DB2) {
  const int Q0 = n + 1, Q = n;
  gll_tables(Q0, z0, w0, D0);
  modA_tables(n, Q0, z0, D0, B0, DB0);
  radau_tables(Q, z1, w1, D1);
  modB_tables(n, Q, z1, D1, B1, DB1);
  Polylib::zwgrjm(z2, w2, Q, 2.0, 0.0);
  Polylib::Dgrjm(D2, z2, Q, 2.0, 0.0);
  modC_tables(n, Q, z2, D2, B2, DB2);
  return 0;
}

int ref_tet_bwdtrans(int n, int E, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  TetTables t = make_tet_tables(n);
  const int nb = E / W;
#define TB(NN) parallel_blocks(nb, nthreads, [&](int b0, int b1) { tet_bwd<NN>(t, in, out, b0, b1); })
  TRI_DISPATCH(n, TB)
#undef TB
}

int ref_tet_iproduct(int n, int E, const double* jac, int deformed, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n * n;
  TetTables t = make_tet_tables(n);
  std::vector<double> dfz((size_t)9 * E * (deformed ? nq : 1), 0.0);
  Geo g = interleave(3, nq, E, E, jac, dfz.data(), deformed != 0);
  const int nb = E / W;
#define TI(NN)                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {            \
    if (deformed) tet_iprod<NN, true>(t, g, in, out, b0, b1);    \
    else tet_iprod<NN, false>(t, g, in, out, b0, b1);            \
  })
  TRI_DISPATCH(n, TI)
#undef TI
}

int ref_tet_physderiv(int n, int E, const double* df, int deformed, const double* in, double* o0, double* o1,
                      double* o2, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n * n;
  TetTables t = make_tet_tables(n);
  std::vector<double> jz((size_t)E * (deformed ? nq : 1), 1.0);
  Geo g = interleave(3, nq, E, E, jz.data(), df, deformed != 0);
  const int nb = E / W;
#define TD(NN)                                                            \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                     \
    if (deformed) tet_deriv<NN, true>(t, g, in, o0, o1, o2, b0, b1);      \
    else tet_deriv<NN, false>(t, g, in, o0, o1, o2, b0, b1);              \
  })
  TRI_DISPATCH(n, TD)
#undef TD
}

int ref_tet_helmholtz(int n, int E, const double* jac, const double* df, int deformed, double lambda,
                      const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n * n;
  TetTables t = make_tet_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define TH(NN)                                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                          \
    if (deformed) helm_tet<NN, true>(t, g, lambda, in, out, b0, b1);           \
    else helm_tet<NN, false>(t, g, lambda, in, out, b0, b1);                   \
  })
  TRI_DISPATCH(n, TH)
#undef TH
}

int ref_tet_iproduct_deriv(int n, int E, const double* jac, const double* df, int deformed, const double* in0,
                           const double* in1, const double* in2, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * n * n;
  TetTables t = make_tet_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define TP(NN)                                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                            \
    if (deformed) iprd_tet<NN, true>(t, g, in0, in1, in2, out, b0, b1);          \
    else iprd_tet<NN, false>(t, g, in0, in1, in2, out, b0, b1);                  \
  })
  TRI_DISPATCH(n, TP)
#undef TP
}

// ---- prisms ----
int ref_prism_bwdtrans(int n, int E, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  PrismTables t = make_prism_tables(n);
  const int nb = E / W;
#define PB(NN) parallel_blocks(nb, nthreads, [&](int b0, int b1) { prism_bwd<NN>(t, in, out, b0, b1); })
  TRI_DISPATCH(n, PB)
#undef PB
}

int ref_prism_iproduct(int n, int E, const double* jac, int deformed, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PrismTables t = make_prism_tables(n);
  std::vector<double> dfz((size_t)9 * E * (deformed ? nq : 1), 0.0);
  Geo g = interleave(3, nq, E, E, jac, dfz.data(), deformed != 0);
  const int nb = E / W;
#define PI(NN)                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {            \
    if (deformed) prism_iprod<NN, true>(t, g, in, out, b0, b1);  \
    else prism_iprod<NN, false>(t, g, in, out, b0, b1);          \
  })
  TRI_DISPATCH(n, PI)
#undef PI
}

int ref_prism_physderiv(int n, int E, const double* df, int deformed, const double* in, double* o0, double* o1,
                        double* o2, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PrismTables t = make_prism_tables(n);
  std::vector<double> jz((size_t)E * (deformed ? nq : 1), 1.0);
  Geo g = interleave(3, nq, E, E, jz.data(), df, deformed != 0);
  const int nb = E / W;
#define PD(NN)                                                            \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                     \
    if (deformed) prism_deriv<NN, true>(t, g, in, o0, o1, o2, b0, b1);    \
    else prism_deriv<NN, false>(t, g, in, o0, o1, o2, b0, b1);            \
  })
  TRI_DISPATCH(n, PD)
#undef PD
}

int ref_prism_helmholtz(int n, int E, const double* jac, const double* df, int deformed, double lambda,
                        const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PrismTables t = make_prism_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define PH(NN)                                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                          \
    if (deformed) helm_prism<NN, true>(t, g, lambda, in, out, b0, b1);         \
    else helm_prism<NN, false>(t, g, lambda, in, out, b0, b1);                 \
  })
  TRI_DISPATCH(n, PH)
#undef PH
}

int ref_prism_iproduct_deriv(int n, int E, const double* jac, const double* df, int deformed, const double* in0,
                             const double* in1, const double* in2, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PrismTables t = make_prism_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define PP(NN)                                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                            \
    if (deformed) iprd_prism<NN, true>(t, g, in0, in1, in2, out, b0, b1);        \
    else iprd_prism<NN, false>(t, g, in0, in1, in2, out, b0, b1);                \
  })
  TRI_DISPATCH(n, PP)
#undef PP
}

// ---- pyramids ----
int ref_pyr_tables(int n, double* z2, double* w2, double* D2, double* B2, double* DB2) {
  Polylib::zwgrjm(z2, w2, n, 2.0, 0.0);
  Polylib::Dgrjm(D2, z2, n, 2.0, 0.0);
  modPyrC_tables(n, n, z2, D2, B2, DB2);
  return 0;
}

int ref_pyr_bwdtrans(int n, int E, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  PyrTables t = make_pyr_tables(n);
  const int nb = E / W;
#define YB(NN) parallel_blocks(nb, nthreads, [&](int b0, int b1) { pyr_bwd<NN>(t, in, out, b0, b1); })
  TRI_DISPATCH(n, YB)
#undef YB
}

int ref_pyr_iproduct(int n, int E, const double* jac, int deformed, const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PyrTables t = make_pyr_tables(n);
  std::vector<double> dfz((size_t)9 * E * (deformed ? nq : 1), 0.0);
  Geo g = interleave(3, nq, E, E, jac, dfz.data(), deformed != 0);
  const int nb = E / W;
#define YI(NN)                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {            \
    if (deformed) pyr_iprod<NN, true>(t, g, in, out, b0, b1);    \
    else pyr_iprod<NN, false>(t, g, in, out, b0, b1);            \
  })
  TRI_DISPATCH(n, YI)
#undef YI
}

int ref_pyr_physderiv(int n, int E, const double* df, int deformed, const double* in, double* o0, double* o1,
                      double* o2, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PyrTables t = make_pyr_tables(n);
  std::vector<double> jz((size_t)E * (deformed ? nq : 1), 1.0);
  Geo g = interleave(3, nq, E, E, jz.data(), df, deformed != 0);
  const int nb = E / W;
#define YD(NN)                                                            \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                     \
    if (deformed) pyr_deriv<NN, true>(t, g, in, o0, o1, o2, b0, b1);      \
    else pyr_deriv<NN, false>(t, g, in, o0, o1, o2, b0, b1);              \
  })
  TRI_DISPATCH(n, YD)
#undef YD
}

int ref_pyr_helmholtz(int n, int E, const double* jac, const double* df, int deformed, double lambda,
                      const double* in, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PyrTables t = make_pyr_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define YH(NN)                                                                 \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                          \
    if (deformed) helm_pyr<NN, true>(t, g, lambda, in, out, b0, b1);           \
    else helm_pyr<NN, false>(t, g, lambda, in, out, b0, b1);                   \
  })
  TRI_DISPATCH(n, YH)
#undef YH
}

int ref_pyr_iproduct_deriv(int n, int E, const double* jac, const double* df, int deformed, const double* in0,
                           const double* in1, const double* in2, double* out, int nthreads) {
  if (E % W) return 2;
  const int nq = (n + 1) * (n + 1) * n;
  PyrTables t = make_pyr_tables(n);
  Geo g = interleave(3, nq, E, E, jac, df, deformed != 0);
  const int nb = E / W;
#define YP(NN)                                                                   \
  parallel_blocks(nb, nthreads, [&](int b0, int b1) {                            \
    if (deformed) iprd_pyr<NN, true>(t, g, in0, in1, in2, out, b0, b1);          \
    else iprd_pyr<NN, false>(t, g, in0, in1, in2, out, b0, b1);                  \
  })
  TRI_DISPATCH(n, YP)
#undef YP
}

}  // extern "C"
