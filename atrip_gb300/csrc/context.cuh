// Internal definition of the opaque atrip_gpu_context (shared by the
// single-system and batch entry points).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "atrip_gb300.h"
#include "engine.cuh"
#include "split.cuh"

struct atrip_gpu_context {
  int No = 0, Nv = 0, device = 0, sm_count = 0;
  int field = ATRIP_FIELD_REAL;  // enum atrip_field: doubles per element = 1 + field
  int64_t n_tuples = 0;
  int n_triples = 0;
  bool have[ATRIP_N_TENSORS] = {};
  atrip_gb300::DeviceTensors dt;
  uint32_t *d_tuples = nullptr;
  uint32_t *d_triples = nullptr;
  double *d_e = nullptr, *d_ect = nullptr;
  int64_t e_lo = 0, e_hi = 0;  // tuple range holding energies of the last run
  double last_sums[4] = {};    // (sum, compensation) of e and ect over that range
  double *d_workspace = nullptr;
  size_t workspace_doubles = 0;
  unsigned long long *d_queue = nullptr;
  double *d_partials = nullptr, *d_sum = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  atrip_gb300::SplitState split;
  atrip_tuning tune = {};
  // processing order of the last range (tuple_block > 1), see build_order
  std::vector<uint32_t> h_tuples;  // packed list, host copy
  uint32_t *d_order = nullptr;
  int64_t order_cap = 0, order_lo = -1, order_hi = -1;
  int order_block = 0;
};
