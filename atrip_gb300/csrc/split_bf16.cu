// Split-precision form (BF16 slices, tcgen05) -- entry points.
#include "split.cuh"

namespace atrip_gb300 {

void split_invalidate(SplitState &s) { s.valid = false; }
void split_free(SplitState &s) { s.valid = false; s.impl = nullptr; }

int split_run(SplitState &, const DeviceTensors &, int, int, int, const uint32_t *,
              const uint32_t *, int, int64_t, int64_t, double, bool, int, unsigned long long *,
              double *, double *, cudaStream_t, int64_t *) {
  set_error("split-BF16 form not built yet");
  return ATRIP_ERR_UNSUPPORTED;
}

}  // namespace atrip_gb300
