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
  bool profile = false;       // launch the kernel built with role counters
};

void split_invalidate(SplitState &s);
// Role profile of the last profiled launch: the counters listed at
// atrip_gpu_split_profile (include/atrip_gb300.h), n of them.
int split_profile_read(const SplitState &s, unsigned long long *out, int n);
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

// Several systems (contexts) in ONE persistent launch of the transposed
// split kernel: a work queue over the concatenation of their tuple ranges,
// per-system tensor maps and arguments in a device table.  Each system's
// SplitState must be prepared (split_prepare) with the same slice format.
struct SplitMultiSystem {
  SplitState *state;
  const DeviceTensors *dt;
  int No, Nv;
  const uint32_t *tuples, *triples;
  int n_triples;
  int64_t t_begin, t_end;
  bool use_j;
  double *e, *ect;
};
struct SplitMultiBuffers {  // owned by the caller; freed by split_multi_free
  void *h_desc = nullptr, *d_desc = nullptr;  // descriptor table (pinned host, device)
  int64_t *h_prefix = nullptr, *d_prefix = nullptr;
  float *wglobal = nullptr;
  size_t wglobal_floats = 0;
  int *d_status = nullptr;
  unsigned long long *d_queue = nullptr;
  int cap = 0;  // systems the tables hold
  // launch layout of the last prepare
  int n = 0, slices = 0, f16 = 0, no_lay = 0, npass_lay = 1, nstages = 0, wsmem = 0, vsm = 0;
  size_t stage_bytes = 0, smem = 0;
};
// Checks the systems fit one launch (the transposed kernel for each, one
// shared-memory layout), sizes the buffers and fills the host tables.
// ATRIP_ERR_UNSUPPORTED (no error state kept) when they do not.
int split_multi_prepare(const SplitMultiSystem *sys, int n, int slices, bool f16, int sm_count,
                        SplitMultiBuffers &b);
// Table copies, queue and status reset and the launch, on st (capturable).
int split_multi_enqueue(const SplitMultiBuffers &b, double tai_sign, int sm_count,
                        cudaStream_t st, int64_t *launches);
void split_multi_free(SplitMultiBuffers &b);

// Runs tuples [t_begin, t_end) in the split form, writing e[t], ect[t].
int split_run(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
              const uint32_t *tuples, const uint32_t *triples, int n_triples, int64_t t_begin,
              int64_t t_end, const uint32_t *order, double tai_sign, bool use_j, int slices,
              unsigned long long *queue, double *e, double *ect, cudaStream_t st,
              int64_t *launches);

}  // namespace atrip_gb300
