// Stand-in for boost::alignment::aligned_allocator<T, Align>, used by the reference
// tinysimd allocator; a minimal C++17 allocator written for the oracle build only.
#ifndef ORACLE_SHIM_BOOST_ALIGNED_ALLOCATOR_HPP
#define ORACLE_SHIM_BOOST_ALIGNED_ALLOCATOR_HPP
#include <cstddef>
#include <new>
namespace boost {
namespace alignment {
template <class T, std::size_t Align = alignof(T)>
struct aligned_allocator {
  using value_type = T;
  static constexpr std::size_t kAlign = Align < alignof(T) ? alignof(T) : Align;
  template <class U>
  struct rebind { using other = aligned_allocator<U, Align>; };
  aligned_allocator() noexcept = default;
  template <class U>
  aligned_allocator(const aligned_allocator<U, Align>&) noexcept {}
  T* allocate(std::size_t n) {
    return static_cast<T*>(::operator new(n * sizeof(T), std::align_val_t(kAlign)));
  }
  void deallocate(T* p, std::size_t) noexcept { ::operator delete(p, std::align_val_t(kAlign)); }
  template <class U>
  bool operator==(const aligned_allocator<U, Align>&) const noexcept { return true; }
  template <class U>
  bool operator!=(const aligned_allocator<U, Align>&) const noexcept { return false; }
};
}  // namespace alignment
}  // namespace boost
#endif
