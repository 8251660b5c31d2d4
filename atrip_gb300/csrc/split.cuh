// Split-precision (BF16 slices on tcgen05 tensor cores) form of the triples
// kernel: state kept per context and the entry point used by atrip_gpu_run.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "engine.cuh"

namespace atrip_gb300 {

struct SplitState {
  bool valid = false;  // pre-split operands match the uploaded tensors
  int slices = 0;
  void *impl = nullptr;
  uint64_t generation = 0;  // bumped whenever device buffers are (re)allocated
  int stage_cap = 0;        // operand ring depth limit (0 = as many as fit)
  bool w_global = false;    // energy warps read W from L2 even when it fits in smem
  int variant = 0;          // 2: transposed kernel (stacked slices as M) where eligible
  bool prefetch = false;    // L2 prefetch of the next part's slab tiles
  bool f16 = false;         // FP16 digit slices (radix 2^11) instead of BF16 (2^8)
  long long wait_cycles = 0;  // bounded-wait limit in SM cycles (0 = built-in ~2 s)
  bool unpublished = false;   // test: the producer publishes no tuple
};

void split_invalidate(SplitState &s);
void split_free(SplitState &s);

// Cut the digit slices and build the tensor maps (host work, allocations).
int split_prepare(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
                  bool use_j, int slices, const uint32_t *triples, int n_triples,
                  cudaStream_t st, int64_t *launches);
// Queue one launch over tuples [t_begin, t_end) on st (no host sync; may be
// captured into a CUDA graph).  The caller zeroes *queue first.
int split_enqueue(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
                  const uint32_t *tuples, const uint32_t *triples, int n_triples, int64_t t_begin,
                  int64_t t_end, const uint32_t *order, double tai_sign, bool use_j,
                  unsigned long long *queue, double *e, double *ect, cudaStream_t st,
                  int64_t *launches);
// Device status word of the last launch (0 = fine) and its host check.
const int *split_status_ptr(const SplitState &s);
int split_status_check(int status);

// Runs tuples [t_begin, t_end) in the split form, writing e[t], ect[t].
int split_run(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
              const uint32_t *tuples, const uint32_t *triples, int n_triples, int64_t t_begin,
              int64_t t_end, const uint32_t *order, double tai_sign, bool use_j, int slices,
              unsigned long long *queue, double *e, double *ect, cudaStream_t st,
              int64_t *launches);

}  // namespace atrip_gb300
