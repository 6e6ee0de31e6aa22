// Stand-in of Collections/CoalescedGeomData.h:58-90 (GetJac, GetDerivFactors).
#pragma once
#include "../nektar_standin_core.hpp"

namespace Nektar {
namespace Collections {
class CoalescedGeomData {
 public:
  const Array<OneD, const NekDouble>& GetJac(std::vector<StdRegions::StdExpansionSharedPtr>&) { return m_jac; }
  const Array<TwoD, const NekDouble>& GetDerivFactors(std::vector<StdRegions::StdExpansionSharedPtr>&) { return m_df; }
  bool IsDeformed(std::vector<StdRegions::StdExpansionSharedPtr>&) { return true; }
  Array<OneD, const NekDouble> m_jac;
  Array<TwoD, const NekDouble> m_df;
};
typedef std::shared_ptr<CoalescedGeomData> CoalescedGeomDataSharedPtr;
}  // namespace Collections
}  // namespace Nektar
