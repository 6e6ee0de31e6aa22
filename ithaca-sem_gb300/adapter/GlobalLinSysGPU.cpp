// Global linear systems "IterativeFullGPU" and "IterativeStaticCondGPU" for the
// reference's GlobalLinSysFactory (MultiRegions/GlobalLinSys.h:62-68, selected by
// GlobalSysSoln, GlobalLinSys.cpp:49-97). Their v_Solve mirror
// GlobalLinSysIterativeFull::v_Solve (GlobalLinSysIterativeFull.cpp:110-209) and
// GlobalLinSysStaticCond::v_Solve (GlobalLinSysStaticCond.cpp:104-238); the CG recurrence,
// preconditioner and (for the full system) the successive-RHS projection run in the GB300
// library. The element operator is the Collections "GPU" operator of the same expansion
// list (registered by CollectionsGPU.cpp).
#include <iostream>

#include <MultiRegions/GlobalLinSys.h>

#include "ithaca_gpu_adapter.hpp"

namespace Nektar {
namespace MultiRegions {

using GpuAdapter::Check;

static ithaca_gpu_op* GpuOperatorOf(const std::weak_ptr<ExpList>& expList) {
  auto e = expList.lock();
  auto it = GpuAdapter::OperatorRegistry().find(e ? e->GetExp(0).get() : nullptr);
  if (it == GpuAdapter::OperatorRegistry().end())
    NEKERROR(ErrorUtil::efatal, "the GPU global systems need the GPU collection operators (COLLECTIONS DEFAULT=\"GPU\")");
  return it->second;
}

class GlobalLinSysIterativeFullGPU : public GlobalLinSys {
 public:
  static std::shared_ptr<GlobalLinSys> create(const GlobalLinSysKey& key, const std::weak_ptr<ExpList>& expList,
                                              const std::shared_ptr<AssemblyMap>& map) {
    return std::shared_ptr<GlobalLinSys>(new GlobalLinSysIterativeFullGPU(key, expList, map));
  }
  static std::string className;
  ~GlobalLinSysIterativeFullGPU() override {
    if (m_cg) ithaca_gpu_cg_destroy(m_cg);
  }

 private:
  ithaca_gpu_cg* m_cg = nullptr;
  bool m_mixed = false;  // a session option such as -I GPUPrecision=mixed would set it

  GlobalLinSysIterativeFullGPU(const GlobalLinSysKey& key, const std::weak_ptr<ExpList>& expList,
                               const std::shared_ptr<AssemblyMap>& map)
      : GlobalLinSys(key, expList, map) {
    const Array<OneD, const int>& l2g = map->GetLocalToGlobalMap();
    const Array<OneD, NekDouble>& sign = map->GetLocalToGlobalSign();
    Check(ithaca_gpu_cg_create(GpuOperatorOf(expList), l2g.get(), sign.get(), map->GetNumGlobalCoeffs(),
                               map->GetNumGlobalDirBndCoeffs(), &m_cg));
    if (map->GetSuccessiveRHS() != 0)  // AssemblyMap.cpp:168-175
      Check(ithaca_gpu_cg_set_successive_rhs(m_cg, map->GetSuccessiveRHS()));
  }

  void v_Solve(const Array<OneD, const NekDouble>& in, Array<OneD, NekDouble>& out,
               const std::shared_ptr<AssemblyMap>& map, const Array<OneD, const NekDouble>&) override {
    // `in` is the element forcing minus the Dirichlet lift, as in the reference
    const int nGlobal = map->GetNumGlobalCoeffs();
    Array<OneD, NekDouble> rhs(nGlobal), x(nGlobal, 0.0);
    map->Assemble(in, rhs);
    ithaca_gpu_cg_opts o;
    ithaca_gpu_cg_default_opts(&o);
    o.tol = map->GetIterativeTolerance();   // AssemblyMap.cpp:137-147
    o.max_iter = map->GetMaxIterations();   // :160-162
    o.mode = m_mixed ? ITHACA_GPU_SOLVE_MIXED_FP32 : ITHACA_GPU_SOLVE_FP64;
    ithaca_gpu_cg_result r;
    Check(ithaca_gpu_cg_solve(m_cg, m_linSysKey.GetConstFactor(StdRegions::eFactorLambda), rhs.get(), x.get(), &o,
                              &r, 0));
    map->GlobalToLocal(x, out);
    if (m_verbose) std::cout << "CG iterations made = " << r.iterations << std::endl;
  }
  void v_SolveLinearSystem(const int, const Array<OneD, const NekDouble>&, Array<OneD, NekDouble>&,
                           const std::shared_ptr<AssemblyMap>&, const int) override {
    NEKERROR(ErrorUtil::efatal, "the GPU system solves through v_Solve");
  }
};

class GlobalLinSysIterativeStaticCondGPU : public GlobalLinSys {
 public:
  static std::shared_ptr<GlobalLinSys> create(const GlobalLinSysKey& key, const std::weak_ptr<ExpList>& expList,
                                              const std::shared_ptr<AssemblyMap>& map) {
    return std::shared_ptr<GlobalLinSys>(new GlobalLinSysIterativeStaticCondGPU(key, expList, map));
  }
  static std::string className;
  ~GlobalLinSysIterativeStaticCondGPU() override {
    if (m_sc) ithaca_gpu_sc_destroy(m_sc);
  }

 private:
  ithaca_gpu_sc* m_sc = nullptr;

  GlobalLinSysIterativeStaticCondGPU(const GlobalLinSysKey& key, const std::weak_ptr<ExpList>& expList,
                                     const std::shared_ptr<AssemblyMap>& map)
      : GlobalLinSys(key, expList, map) {
    Check(ithaca_gpu_sc_create(GpuOperatorOf(expList), map->GetLocalToGlobalMap().get(),
                               map->GetLocalToGlobalSign().get(), map->GetNumGlobalCoeffs(),
                               map->GetNumGlobalDirBndCoeffs(), &m_sc));
  }

  // `in`: the element forcing; `out`: the Dirichlet coefficients (and any initial guess)
  // already in local storage, as ContField::v_HelmSolve leaves them
  void v_Solve(const Array<OneD, const NekDouble>& in, Array<OneD, NekDouble>& out,
               const std::shared_ptr<AssemblyMap>& map, const Array<OneD, const NekDouble>&) override {
    ithaca_gpu_cg_opts o;
    ithaca_gpu_cg_default_opts(&o);
    o.tol = map->GetIterativeTolerance();
    o.max_iter = map->GetMaxIterations();
    ithaca_gpu_cg_result r;
    Check(ithaca_gpu_sc_solve(m_sc, m_linSysKey.GetConstFactor(StdRegions::eFactorLambda), in.get(), out.get(), &o,
                              &r, 0));
    if (m_verbose) std::cout << "CG iterations made = " << r.iterations << std::endl;
  }
  void v_SolveLinearSystem(const int, const Array<OneD, const NekDouble>&, Array<OneD, NekDouble>&,
                           const std::shared_ptr<AssemblyMap>&, const int) override {
    NEKERROR(ErrorUtil::efatal, "the GPU system solves through v_Solve");
  }
};

std::string GlobalLinSysIterativeFullGPU::className = GetGlobalLinSysFactory().RegisterCreatorFunction(
    "IterativeFullGPU", GlobalLinSysIterativeFullGPU::create, "GPU conjugate gradient");
std::string GlobalLinSysIterativeStaticCondGPU::className = GetGlobalLinSysFactory().RegisterCreatorFunction(
    "IterativeStaticCondGPU", GlobalLinSysIterativeStaticCondGPU::create, "GPU statically condensed conjugate gradient");

}  // namespace MultiRegions
}  // namespace Nektar
