// Stand-ins for the few Nektar++ types the GPU adapter classes touch, so that
// ithaca-sem_gb300/adapter/*.cpp compile and link here without the reference's build
// (Boost, TinyXML, BLAS are absent). Each declaration follows the reference signature it
// stands in for (file:line in the comments); only what the adapters use is declared.
// TEST INFRASTRUCTURE: nothing here runs a Nektar++ computation.
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace Nektar {

typedef double NekDouble;  // LibUtilities/BasicConst/NektarUnivTypeDefs.hpp

// LibUtilities/BasicUtils/SharedArray.hpp: reference-counted host arrays; get() is the
// contiguous storage, which the C ABI reads directly.
struct OneD {};
struct TwoD {};
template <typename Dim, typename T>
class Array;
template <typename T>
class Array<OneD, T> {
 public:
  Array() = default;
  explicit Array(size_t n, T v = T()) : m_data(std::make_shared<std::vector<typename std::remove_const<T>::type>>(n, v)) {}
  template <typename U>
  Array(const Array<OneD, U>& o) : m_data(o.m_data), m_off(o.m_off) {}
  T* get() const { return m_data ? m_data->data() + m_off : nullptr; }
  size_t size() const { return m_data ? m_data->size() - m_off : 0; }
  T& operator[](size_t i) const { return get()[i]; }
  Array operator+(size_t off) const {
    Array a(*this);
    a.m_off += off;
    return a;
  }
  std::shared_ptr<std::vector<typename std::remove_const<T>::type>> m_data;
  size_t m_off = 0;
};
template <typename T>
class Array<TwoD, T> {
 public:
  Array() = default;
  Array(size_t n0, size_t n1, T v = T()) : m_data(std::make_shared<std::vector<typename std::remove_const<T>::type>>(n0 * n1, v)) {}
  template <typename U>
  Array(const Array<TwoD, U>& o) : m_data(o.m_data) {}
  T* get() const { return m_data ? m_data->data() : nullptr; }  // row-major [dir][point]
  std::shared_ptr<std::vector<typename std::remove_const<T>::type>> m_data;
};
static Array<OneD, NekDouble> NullNekDouble1DArray;

// LibUtilities/BasicUtils/ErrorUtil.hpp:59,209-240
namespace ErrorUtil {
enum ErrType { efatal, ewarning };
struct NekError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
}  // namespace ErrorUtil
#define NEKERROR(type, msg) throw ::Nektar::ErrorUtil::NekError(std::string(msg))

// LibUtilities/BasicUtils/SharedPtr.hpp / MemoryManager
template <typename T>
struct MemoryManager {
  template <typename... A>
  static std::shared_ptr<T> AllocateSharedPtr(A&&... a) {
    return std::shared_ptr<T>(new T(std::forward<A>(a)...));
  }
};

// LibUtilities/BasicUtils/NekFactory.hpp:47-60 (key -> creator, with a description)
template <typename Key, typename Base, typename... Args>
class NekFactory {
 public:
  typedef std::shared_ptr<Base> (*CreatorFunction)(Args...);
  Key RegisterCreatorFunction(const Key& k, CreatorFunction f, const std::string& desc = "") {
    m_map[k] = {f, desc};
    return k;
  }
  std::shared_ptr<Base> CreateInstance(const Key& k, Args... a) { return m_map.at(k).first(a...); }
  bool ModuleExists(const Key& k) const { return m_map.count(k) > 0; }
  std::map<Key, std::pair<CreatorFunction, std::string>> m_map;
};

namespace LibUtilities {
// LibUtilities/BasicUtils/ShapeType.hpp
enum ShapeType { eNoShapeType, ePoint, eSegment, eTriangle, eQuadrilateral, eTetrahedron, ePyramid, ePrism, eHexahedron };
// LibUtilities/Foundations/Basis.h: modes and points of a 1-D basis
class Basis {
 public:
  Basis(int nm, int nq) : m_nm(nm), m_nq(nq) {}
  int GetNumModes() const { return m_nm; }
  int GetNumPoints() const { return m_nq; }
 private:
  int m_nm, m_nq;
};
typedef std::shared_ptr<Basis> BasisSharedPtr;
}  // namespace LibUtilities

namespace StdRegions {
// StdRegions/StdRegions.hpp: constant factors of an operator
enum ConstFactorType { eFactorLambda, eFactorTau };
typedef std::map<ConstFactorType, NekDouble> ConstFactorMap;
static ConstFactorMap NullConstFactorMap;
// StdRegions/StdExpansion.h
class StdExpansion {
 public:
  StdExpansion(LibUtilities::ShapeType s, int nm, int nq) : m_shape(s), m_basis(std::make_shared<LibUtilities::Basis>(nm, nq)) {}
  LibUtilities::ShapeType DetShapeType() const { return m_shape; }
  const LibUtilities::BasisSharedPtr& GetBasis(int) const { return m_basis; }
  std::shared_ptr<StdExpansion> GetStdExp() const { return std::make_shared<StdExpansion>(*this); }
 private:
  LibUtilities::ShapeType m_shape;
  LibUtilities::BasisSharedPtr m_basis;
};
typedef std::shared_ptr<StdExpansion> StdExpansionSharedPtr;
}  // namespace StdRegions

}  // namespace Nektar
