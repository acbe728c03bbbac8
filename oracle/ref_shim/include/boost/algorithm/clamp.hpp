// Minimal stand-in for boost/algorithm/clamp.hpp (only clamp(v, lo, hi) is used,
// color_generator.cpp:59-61).
#ifndef PARS_SHIM_BOOST_ALGORITHM_CLAMP_HPP
#define PARS_SHIM_BOOST_ALGORITHM_CLAMP_HPP
namespace boost { namespace algorithm {
template <typename T>
const T& clamp(const T& value, const T& lo, const T& hi)
{
  return value < lo ? lo : (hi < value ? hi : value);
}
}}
#endif
