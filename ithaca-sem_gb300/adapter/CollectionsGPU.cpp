// Implementation type "GPU" for the Collections operators (Collections/Operator.h:113-165,
// registrations as Collections/Helmholtz.cpp:484-503): BwdTrans, IProductWRTBase,
// PhysDeriv, IProductWRTDerivBase and Helmholtz of collections of every shape
// (triangles, quadrilaterals, tetrahedra, pyramids, prisms, hexahedra) run in the GB300 library. Nektar's arrays are passed unchanged: the C ABI
// keeps the reference's element-contiguous layouts and CoalescedGeomData's geometry.
#include <Collections/Operator.h>

#include "ithaca_gpu_adapter.hpp"

namespace Nektar {
namespace Collections {

using GpuAdapter::Check;

// Common construction: one library operator per collection (FP64), from the coalesced
// geometry (CoalescedGeomData::GetJac / GetDerivFactors, CoalescedGeomData.cpp:53-313).
class GpuOperatorBase : public Operator {
 protected:
  GpuOperatorBase(std::vector<StdRegions::StdExpansionSharedPtr> pCollExp, CoalescedGeomDataSharedPtr pGeomData)
      : Operator(pCollExp, pGeomData) {
    const auto shape = pCollExp[0]->DetShapeType();
    if (shape < LibUtilities::eTriangle || shape > LibUtilities::eHexahedron)
      NEKERROR(ErrorUtil::efatal, "GPU operators are built for two- and three-dimensional elements");
    const int nm = pCollExp[0]->GetBasis(0)->GetNumModes();
    const int nq = pCollExp[0]->GetBasis(0)->GetNumPoints();
    const Array<OneD, const NekDouble>& jac = pGeomData->GetJac(pCollExp);
    const Array<TwoD, const NekDouble>& df = pGeomData->GetDerivFactors(pCollExp);
    Check(ithaca_gpu_op_create(GpuAdapter::GpuContext(), (int)shape, nm, nq, (int)m_numElmt, jac.get(), df.get(),
                               m_isDeformed ? 1 : 0, ITHACA_GPU_FP64, 0, &m_op));
    GpuAdapter::OperatorRegistry()[pCollExp[0].get()] = m_op;
    m_dim = shape == LibUtilities::eTriangle || shape == LibUtilities::eQuadrilateral ? 2 : 3;
  }
  ~GpuOperatorBase() override {
    if (m_op) ithaca_gpu_op_destroy(m_op);
  }
  void operator()(int, const Array<OneD, const NekDouble>&, Array<OneD, NekDouble>&, Array<OneD, NekDouble>&) override {
    NEKERROR(ErrorUtil::efatal, "Not valid for this operator.");
  }
  ithaca_gpu_op* m_op = nullptr;
  int m_dim = 2;
};

class BwdTrans_GPU final : public GpuOperatorBase {
 public:
  OPERATOR_CREATE(BwdTrans_GPU)
  using GpuOperatorBase::operator();
  void operator()(const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output0, Array<OneD, NekDouble>&,
                  Array<OneD, NekDouble>&, Array<OneD, NekDouble>&, const StdRegions::ConstFactorMap&) override {
    Check(ithaca_gpu_bwdtrans(m_op, input.get(), output0.get(), 0));
  }
 private:
  BwdTrans_GPU(std::vector<StdRegions::StdExpansionSharedPtr> e, CoalescedGeomDataSharedPtr g) : GpuOperatorBase(e, g) {}
};

class IProductWRTBase_GPU final : public GpuOperatorBase {
 public:
  OPERATOR_CREATE(IProductWRTBase_GPU)
  using GpuOperatorBase::operator();
  void operator()(const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output0, Array<OneD, NekDouble>&,
                  Array<OneD, NekDouble>&, Array<OneD, NekDouble>&, const StdRegions::ConstFactorMap&) override {
    Check(ithaca_gpu_iproduct(m_op, input.get(), output0.get(), 0));
  }
 private:
  IProductWRTBase_GPU(std::vector<StdRegions::StdExpansionSharedPtr> e, CoalescedGeomDataSharedPtr g)
      : GpuOperatorBase(e, g) {}
};

class PhysDeriv_GPU final : public GpuOperatorBase {
 public:
  OPERATOR_CREATE(PhysDeriv_GPU)
  using GpuOperatorBase::operator();
  void operator()(const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output0,
                  Array<OneD, NekDouble>& output1, Array<OneD, NekDouble>& output2, Array<OneD, NekDouble>&,
                  const StdRegions::ConstFactorMap&) override {
    Check(ithaca_gpu_physderiv(m_op, input.get(), output0.get(), output1.get(), m_dim == 3 ? output2.get() : nullptr,
                               0));
  }
 private:
  PhysDeriv_GPU(std::vector<StdRegions::StdExpansionSharedPtr> e, CoalescedGeomDataSharedPtr g) : GpuOperatorBase(e, g) {}
};

// entry0..2 hold the derivative components and the result goes to the entry after the
// last component (Collections/IProductWRTDerivBase.cpp:446-470)
class IProductWRTDerivBase_GPU final : public GpuOperatorBase {
 public:
  OPERATOR_CREATE(IProductWRTDerivBase_GPU)
  using GpuOperatorBase::operator();
  void operator()(const Array<OneD, const NekDouble>& entry0, Array<OneD, NekDouble>& entry1,
                  Array<OneD, NekDouble>& entry2, Array<OneD, NekDouble>& entry3, Array<OneD, NekDouble>&,
                  const StdRegions::ConstFactorMap&) override {
    NekDouble* out = m_dim == 2 ? entry2.get() : entry3.get();
    Check(ithaca_gpu_iproduct_deriv(m_op, entry0.get(), entry1.get(), m_dim == 3 ? entry2.get() : nullptr, out, 0));
  }
 private:
  IProductWRTDerivBase_GPU(std::vector<StdRegions::StdExpansionSharedPtr> e, CoalescedGeomDataSharedPtr g)
      : GpuOperatorBase(e, g) {}
};

class Helmholtz_GPU final : public GpuOperatorBase {
 public:
  OPERATOR_CREATE(Helmholtz_GPU)
  using GpuOperatorBase::operator();
  void operator()(const Array<OneD, const NekDouble>& input, Array<OneD, NekDouble>& output0, Array<OneD, NekDouble>&,
                  Array<OneD, NekDouble>&, Array<OneD, NekDouble>&, const StdRegions::ConstFactorMap& factors) override {
    const NekDouble lambda = factors.at(StdRegions::eFactorLambda);  // Collections/Helmholtz.cpp:409-414
    Check(ithaca_gpu_helmholtz(m_op, lambda, input.get(), output0.get(), 0));
  }
 private:
  Helmholtz_GPU(std::vector<StdRegions::StdExpansionSharedPtr> e, CoalescedGeomDataSharedPtr g) : GpuOperatorBase(e, g) {}
};

#define ITHACA_GPU_REGISTER(cls, op, name)                                                                      \
  OperatorKey cls::m_typeArr[] = {                                                                            \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::eTriangle, op, eGPU, false),      \
                                                   cls::create, name "_Tri"),                                  \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::eQuadrilateral, op, eGPU, false), \
                                                   cls::create, name "_Quad"),                                 \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::eTetrahedron, op, eGPU, false),   \
                                                   cls::create, name "_Tet"),                                  \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::ePyramid, op, eGPU, false),       \
                                                   cls::create, name "_Pyr"),                                  \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::ePrism, op, eGPU, false),         \
                                                   cls::create, name "_Prism"),                                \
      GetOperatorFactory().RegisterCreatorFunction(OperatorKey(LibUtilities::eHexahedron, op, eGPU, false),    \
                                                   cls::create, name "_Hex")};

ITHACA_GPU_REGISTER(BwdTrans_GPU, eBwdTrans, "BwdTrans_GPU")
ITHACA_GPU_REGISTER(IProductWRTBase_GPU, eIProductWRTBase, "IProductWRTBase_GPU")
ITHACA_GPU_REGISTER(PhysDeriv_GPU, ePhysDeriv, "PhysDeriv_GPU")
ITHACA_GPU_REGISTER(IProductWRTDerivBase_GPU, eIProductWRTDerivBase, "IProductWRTDerivBase_GPU")
ITHACA_GPU_REGISTER(Helmholtz_GPU, eHelmholtz, "Helmholtz_GPU")
#undef ITHACA_GPU_REGISTER

}  // namespace Collections
}  // namespace Nektar
