// Stand-in for the one Boost utility the reference Polylib / MatrixFreeOps
// kernels use (boost::ignore_unused); written for the oracle build only.
#ifndef ORACLE_SHIM_BOOST_IGNORE_UNUSED_HPP
#define ORACLE_SHIM_BOOST_IGNORE_UNUSED_HPP
namespace boost {
template <typename... Ts>
inline void ignore_unused(Ts const&...) {}
}  // namespace boost
#endif
