// Stand-in of Collections/Operator.h:45-175: the operator base class, its key, the
// OPERATOR_CREATE macro and the factory, with "GPU" added to the implementation types as
// the adapter requires (Operator.h:84-103).
#pragma once
#include "CoalescedGeomData.h"

#define OPERATOR_CREATE(cname)                                                          \
  static OperatorKey m_type;                                                            \
  static OperatorKey m_typeArr[];                                                       \
  friend class MemoryManager<cname>;                                                    \
  static OperatorSharedPtr create(std::vector<StdRegions::StdExpansionSharedPtr> pCollExp, \
                                  std::shared_ptr<CoalescedGeomData> GeomData) {        \
    return MemoryManager<cname>::AllocateSharedPtr(pCollExp, GeomData);                 \
  }

namespace Nektar {
namespace Collections {
enum OperatorType { eBwdTrans, eIProductWRTBase, eIProductWRTDerivBase, ePhysDeriv, eHelmholtz };
enum ImplementationType { eNoImpType, eIterPerExp, eStdMat, eSumFac, eMatrixFree, eGPU, eNoCollection };
typedef bool ExpansionIsNodal;

class Operator {
 public:
  Operator(std::vector<StdRegions::StdExpansionSharedPtr> pCollExp, std::shared_ptr<CoalescedGeomData>)
      : m_isDeformed(true), m_stdExp(pCollExp.at(0)->GetStdExp()), m_numElmt((unsigned)pCollExp.size()) {}
  virtual void operator()(const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output0,
                          Array<OneD, NekDouble>& output1, Array<OneD, NekDouble>& output2,
                          Array<OneD, NekDouble>& wsp = NullNekDouble1DArray,
                          const StdRegions::ConstFactorMap& factors = StdRegions::NullConstFactorMap) = 0;
  virtual void operator()(int dir, const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output,
                          Array<OneD, NekDouble>& wsp = NullNekDouble1DArray) = 0;
  virtual ~Operator() = default;
 protected:
  bool m_isDeformed;
  StdRegions::StdExpansionSharedPtr m_stdExp;
  unsigned int m_numElmt;
  unsigned int m_wspSize = 0;
};
typedef std::shared_ptr<Operator> OperatorSharedPtr;
typedef std::tuple<LibUtilities::ShapeType, OperatorType, ImplementationType, ExpansionIsNodal> OperatorKey;
typedef NekFactory<OperatorKey, Operator, std::vector<StdRegions::StdExpansionSharedPtr>,
                   std::shared_ptr<CoalescedGeomData>>
    OperatorFactory;
inline OperatorFactory& GetOperatorFactory() {
  static OperatorFactory f;
  return f;
}
}  // namespace Collections
}  // namespace Nektar
