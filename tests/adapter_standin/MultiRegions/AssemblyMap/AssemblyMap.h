// Stand-in of MultiRegions/AssemblyMap/AssemblyMap.h:80-308: the accessors of the
// local-to-global map that the GPU systems read, and Assemble / GlobalToLocal.
#pragma once
#include "../../nektar_standin_core.hpp"

namespace Nektar {
namespace MultiRegions {
class AssemblyMap {
 public:
  const Array<OneD, const int>& GetLocalToGlobalMap() { return m_l2g; }
  const Array<OneD, NekDouble>& GetLocalToGlobalSign() const { return m_sign; }
  int GetNumGlobalCoeffs() const { return m_nglobal; }
  int GetNumGlobalDirBndCoeffs() const { return m_ndir; }
  NekDouble GetIterativeTolerance() const { return m_tol; }
  int GetMaxIterations() const { return m_maxiter; }
  int GetSuccessiveRHS() const { return m_successive; }
  void Assemble(const Array<OneD, const NekDouble>& loc, Array<OneD, NekDouble>& global) const {
    for (size_t i = 0; i < global.size(); ++i) global[i] = 0.0;
    for (size_t l = 0; l < m_l2g.size(); ++l) global[m_l2g[l]] += m_sign[l] * loc[l];
  }
  void GlobalToLocal(const Array<OneD, const NekDouble>& global, Array<OneD, NekDouble>& loc) const {
    for (size_t l = 0; l < m_l2g.size(); ++l) loc[l] = m_sign[l] * global[m_l2g[l]];
  }
  Array<OneD, const int> m_l2g;
  Array<OneD, NekDouble> m_sign;
  int m_nglobal = 0, m_ndir = 0, m_maxiter = 5000, m_successive = 0;
  NekDouble m_tol = 1e-9;
};
typedef std::shared_ptr<AssemblyMap> AssemblyMapSharedPtr;
}  // namespace MultiRegions
}  // namespace Nektar
