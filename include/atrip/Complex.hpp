// atrip_gb300 drop-in: atrip's complex field type (src/atrip/Complex.hpp of
// the reference).  std::complex<double> is stored as (re, im), the layout
// the C ABI takes for ATRIP_FIELD_COMPLEX.
#ifndef ATRIP_GB300_COMPLEX_HPP_
#define ATRIP_GB300_COMPLEX_HPP_

#include <complex>

namespace atrip {
using Complex = std::complex<double>;
}  // namespace atrip

#endif
