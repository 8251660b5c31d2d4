// atrip_gb300 drop-in: the scalar conjugation helper of atrip's operations
// header (src/atrip/Operations.hpp:28-52 of the reference), host side only:
// identity for real fields, complex conjugate for atrip::Complex.  Drivers
// use it in CTF transforms when they prepare the (cT) intermediates.
#ifndef ATRIP_GB300_OPERATIONS_HPP_
#define ATRIP_GB300_OPERATIONS_HPP_

#include <complex>

#include <atrip/Complex.hpp>

namespace atrip {
namespace acc {

template <typename F>
inline F maybe_conjugate_scalar(const F &a) {
  return a;
}
template <>
inline Complex maybe_conjugate_scalar<Complex>(const Complex &a) {
  return std::conj(a);
}

}  // namespace acc
}  // namespace atrip

#endif
