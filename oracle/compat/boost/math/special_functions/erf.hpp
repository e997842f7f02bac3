#pragma once
#include <cmath>
#include <stdexcept>
// erf/erfc map to the C library; the inverse functions have no stand-in (they are not used
// by any workload this oracle checks) and throw if reached.
namespace boost { namespace math {
inline double erf(double x) { return std::erf(x); }
inline double erfc(double x) { return std::erfc(x); }
inline double erf_inv(double) { throw std::runtime_error("erf_inv has no std stand-in"); }
inline double erfc_inv(double) { throw std::runtime_error("erfc_inv has no std stand-in"); }
} }
