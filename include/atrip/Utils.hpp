// atrip_gb300 drop-in: atrip's printf-style string helper
// (_FORMAT(fmt, ...) -> std::string, src/atrip/Utils.hpp of the reference),
// defined only where the caller has not defined it already.
#ifndef ATRIP_GB300_UTILS_HPP_
#define ATRIP_GB300_UTILS_HPP_

#include <cstdarg>
#include <cstdio>
#include <string>

namespace atrip {
namespace detail {
inline std::string format(const char *fmt, ...) {
  va_list ap, ap2;
  va_start(ap, fmt);
  va_copy(ap2, ap);
  const int n = std::vsnprintf(nullptr, 0, fmt, ap);
  va_end(ap);
  std::string s(n > 0 ? (size_t)n : 0, '\0');
  if (n > 0) std::vsnprintf(&s[0], (size_t)n + 1, fmt, ap2);
  va_end(ap2);
  return s;
}
}  // namespace detail
}  // namespace atrip

#ifndef _FORMAT
#define _FORMAT(_fmt, ...) ::atrip::detail::format(_fmt, __VA_ARGS__)
#endif

#endif
