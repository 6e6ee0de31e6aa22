// Stand-in of MultiRegions/GlobalLinSys.h:62-160 and GlobalMatrixKey.h:78: the global
// system base class with its pure virtual solves, its key's constant factors and the
// factory selected by GlobalSysSoln.
#pragma once
#include "AssemblyMap/AssemblyMap.h"

namespace Nektar {
namespace MultiRegions {
// MultiRegions/ExpList.h: GetExp(n), the n-th element expansion
class ExpList {
 public:
  const StdRegions::StdExpansionSharedPtr& GetExp(int n) const { return m_exp.at(n); }
  std::vector<StdRegions::StdExpansionSharedPtr> m_exp;
};
class GlobalLinSysKey {
 public:
  explicit GlobalLinSysKey(StdRegions::ConstFactorMap f = {}) : m_factors(f) {}
  NekDouble GetConstFactor(const StdRegions::ConstFactorType& t) const { return m_factors.at(t); }
  StdRegions::ConstFactorMap m_factors;
};

class GlobalLinSys {
 public:
  GlobalLinSys(const GlobalLinSysKey& key, const std::weak_ptr<ExpList>& expList,
               const std::shared_ptr<AssemblyMap>& locToGloMap)
      : m_linSysKey(key), m_expList(expList), m_verbose(false) {
    (void)locToGloMap;
  }
  virtual ~GlobalLinSys() = default;
  void Solve(const Array<OneD, const NekDouble>& in, Array<OneD, NekDouble>& out,
             const std::shared_ptr<AssemblyMap>& map,
             const Array<OneD, const NekDouble>& dirForcing = NullNekDouble1DArray) {
    v_Solve(in, out, map, dirForcing);
  }
 protected:
  const GlobalLinSysKey m_linSysKey;
  const std::weak_ptr<ExpList> m_expList;
  bool m_verbose;
 private:
  virtual void v_Solve(const Array<OneD, const NekDouble>& in, Array<OneD, NekDouble>& out,
                       const std::shared_ptr<AssemblyMap>& locToGloMap,
                       const Array<OneD, const NekDouble>& dirForcing = NullNekDouble1DArray) = 0;
  virtual void v_SolveLinearSystem(const int pNumRows, const Array<OneD, const NekDouble>& pInput,
                                   Array<OneD, NekDouble>& pOutput, const std::shared_ptr<AssemblyMap>& locToGloMap,
                                   const int pNumDir) = 0;
};
typedef std::shared_ptr<GlobalLinSys> GlobalLinSysSharedPtr;
typedef NekFactory<std::string, GlobalLinSys, const GlobalLinSysKey&, const std::weak_ptr<ExpList>&,
                   const std::shared_ptr<AssemblyMap>&>
    GlobalLinSysFactory;
inline GlobalLinSysFactory& GetGlobalLinSysFactory() {
  static GlobalLinSysFactory f;
  return f;
}
}  // namespace MultiRegions
}  // namespace Nektar
