// atrip_gb300 drop-in: atrip's timing types (src/atrip/Chrono.hpp:30-40 of
// the reference), so that callers reading Atrip::chrono["..."].count()
// compile unchanged.  Atrip::run fills "iterations" (device time of the
// triples loop) and "run" (wall time of the whole call).
#ifndef ATRIP_GB300_CHRONO_HPP_
#define ATRIP_GB300_CHRONO_HPP_

#include <chrono>
#include <map>
#include <string>

namespace atrip {

// Accumulating stopwatch: start()/stop() pairs add up; count() in seconds.
struct Timer {
  using Clock = std::chrono::steady_clock;
  std::chrono::duration<double> duration{0.0};
  Clock::time_point t0{};
  void start() noexcept { t0 = Clock::now(); }
  void stop() noexcept { duration += Clock::now() - t0; }
  void clear() noexcept { duration = std::chrono::duration<double>(0.0); }
  double count() const noexcept { return duration.count(); }
  // add a span measured elsewhere (e.g. CUDA-event device time)
  void add(double seconds) noexcept { duration += std::chrono::duration<double>(seconds); }
};
using Timings = std::map<std::string, Timer>;

}  // namespace atrip

#endif
