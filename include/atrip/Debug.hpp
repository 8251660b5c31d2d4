// atrip_gb300 drop-in: the iteration-progress hook of atrip
// (src/atrip/Debug.hpp:96-109 of the reference).  A caller registers one
// callback; Atrip::run calls it as the tuple list advances (between the
// device queue's chunks) with the position, the list length and the
// seconds since the call began.
#ifndef ATRIP_GB300_DEBUG_HPP_
#define ATRIP_GB300_DEBUG_HPP_

#include <cstddef>
#include <functional>

namespace atrip {

struct IterationDescription;
using IterationDescriptor = std::function<void(IterationDescription const &)>;
struct IterationDescription {
  static IterationDescriptor &descriptor() {
    static IterationDescriptor d;
    return d;
  }
  size_t current_iteration;
  size_t total_iterations;
  double current_elapsed_time;
};
inline void register_iteration_descriptor(IterationDescriptor d) {
  IterationDescription::descriptor() = d;
}

}  // namespace atrip

#endif
