// Test driver of the Nektar++ adapter classes (ithaca-sem_gb300/adapter) built against the
// stand-in headers: it fills the stand-in expansion list, coalesced geometry and
// assembly map the way Nektar++ would, creates the operators and systems through the
// reference's factories and calls them, so that the tests can compare the adapter's
// results with the oracle. TEST INFRASTRUCTURE.
#include <Collections/Operator.h>
#include <MultiRegions/GlobalLinSys.h>

using namespace Nektar;

namespace {
std::vector<StdRegions::StdExpansionSharedPtr> Expansions(int shape, int n, int Q, int E) {
  auto e = std::make_shared<StdRegions::StdExpansion>((LibUtilities::ShapeType)shape, n, Q);
  return std::vector<StdRegions::StdExpansionSharedPtr>(E, e);
}
// per element: coefficients and quadrature points of the shape (triangles: n (n+1)/2 modes
// on Q x (Q - 1) collapsed points)
size_t ModesPerElement(int shape, int n) {
  if (shape == LibUtilities::eTriangle) return (size_t)n * (n + 1) / 2;
  if (shape == LibUtilities::eTetrahedron) return (size_t)n * (n + 1) * (n + 2) / 6;
  if (shape == LibUtilities::ePrism) return (size_t)n * n * (n + 1) / 2;
  if (shape == LibUtilities::ePyramid) return (size_t)n * (n + 1) * (2 * n + 1) / 6;
  return shape == LibUtilities::eQuadrilateral ? (size_t)n * n : (size_t)n * n * n;
}
size_t PointsPerElement(int shape, int Q) {
  if (shape == LibUtilities::eTriangle) return (size_t)Q * (Q - 1);
  if (shape == LibUtilities::eTetrahedron) return (size_t)Q * (Q - 1) * (Q - 1);
  if (shape == LibUtilities::ePrism || shape == LibUtilities::ePyramid) return (size_t)Q * Q * (Q - 1);
  return shape == LibUtilities::eQuadrilateral ? (size_t)Q * Q : (size_t)Q * Q * Q;
}
std::shared_ptr<Collections::CoalescedGeomData> Geometry(int shape, int Q, int E, const double* jac, const double* df) {
  auto g = std::make_shared<Collections::CoalescedGeomData>();
  const int dim = shape == LibUtilities::eTriangle || shape == LibUtilities::eQuadrilateral ? 2 : 3;
  const size_t npts = (size_t)E * PointsPerElement(shape, Q);
  Array<OneD, NekDouble> j(npts);
  Array<TwoD, NekDouble> d(dim * dim, npts);
  std::copy(jac, jac + npts, j.get());
  std::copy(df, df + npts * dim * dim, d.get());
  g->m_jac = j;
  g->m_df = d;
  return g;
}
}  // namespace

extern "C" {

// registered keys: Collections operators, global systems
int probe_registry(int* nops, int* nsys, int* has_gpu_full, int* has_gpu_sc) {
  *nops = (int)Collections::GetOperatorFactory().m_map.size();
  *nsys = (int)MultiRegions::GetGlobalLinSysFactory().m_map.size();
  *has_gpu_full = MultiRegions::GetGlobalLinSysFactory().ModuleExists("IterativeFullGPU");
  *has_gpu_sc = MultiRegions::GetGlobalLinSysFactory().ModuleExists("IterativeStaticCondGPU");
  return 0;
}

// Collection Helmholtz_GPU through the factory; returns 0, or 1 with the NekError message.
int probe_helmholtz(int shape, int n, int Q, int E, const double* jac, const double* df, double lambda,
                    const double* in, double* out, char* msg, int msglen) {
  try {
    auto exps = Expansions(shape, n, Q, E);
    auto op = Collections::GetOperatorFactory().CreateInstance(
        Collections::OperatorKey((LibUtilities::ShapeType)shape, Collections::eHelmholtz, Collections::eGPU, false),
        exps, Geometry(shape, Q, E, jac, df));
    const size_t nloc = (size_t)E * ModesPerElement(shape, n);
    Array<OneD, NekDouble> a(nloc), b(nloc), w;
    std::copy(in, in + nloc, a.get());
    StdRegions::ConstFactorMap f{{StdRegions::eFactorLambda, lambda}};
    (*op)(a, b, w, w, w, f);
    std::copy(b.get(), b.get() + nloc, out);
    return 0;
  } catch (const ErrorUtil::NekError& e) {
    snprintf(msg, msglen, "%s", e.what());
    return 1;
  }
}

// Collection operator plus global system `name` through the factories: GlobalLinSys::Solve
// of the element forcing `in` (Dirichlet values, if any, already in `out`), tolerance tol.
int probe_solve(const char* name, int shape, int n, int Q, int E, const double* jac, const double* df, double lambda,
                const int* l2g, const double* sign, int nglobal, int ndir, double tol, const double* in, double* out,
                char* msg, int msglen) {
  try {
    auto exps = Expansions(shape, n, Q, E);
    auto op = Collections::GetOperatorFactory().CreateInstance(
        Collections::OperatorKey((LibUtilities::ShapeType)shape, Collections::eHelmholtz, Collections::eGPU, false),
        exps, Geometry(shape, Q, E, jac, df));
    auto expList = std::make_shared<MultiRegions::ExpList>();
    expList->m_exp = exps;
    auto map = std::make_shared<MultiRegions::AssemblyMap>();
    const size_t nloc = (size_t)E * ModesPerElement(shape, n);
    Array<OneD, int> m(nloc);
    Array<OneD, NekDouble> s(nloc);
    std::copy(l2g, l2g + nloc, m.get());
    std::copy(sign, sign + nloc, s.get());
    map->m_l2g = m;
    map->m_sign = s;
    map->m_nglobal = nglobal;
    map->m_ndir = ndir;
    map->m_tol = tol;
    MultiRegions::GlobalLinSysKey key({{StdRegions::eFactorLambda, lambda}});
    auto sys = MultiRegions::GetGlobalLinSysFactory().CreateInstance(name, key, expList, map);
    Array<OneD, NekDouble> a(nloc), b(nloc);
    std::copy(in, in + nloc, a.get());
    std::copy(out, out + nloc, b.get());
    sys->Solve(a, b, map);
    std::copy(b.get(), b.get() + nloc, out);
    return 0;
  } catch (const ErrorUtil::NekError& e) {
    snprintf(msg, msglen, "%s", e.what());
    return 1;
  }
}

}  // extern "C"
