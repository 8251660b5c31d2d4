// Batching form: many independent systems (contexts) in one run.
//
// FP64: one persistent launch of the batch kernel over the concatenated
// tuple lists of all systems (a single device work-queue cursor; the table of
// per-system descriptors is ordered by per-tuple cost, largest first, so the
// queue drains the expensive tuples before the cheap ones), then one kernel
// that reduces every system's energies.  Split form: one persistent launch
// per system (each has its own pre-split operands and tensor maps) and the
// same reduction.  Either sequence is captured once into a CUDA graph and
// replayed; the descriptor table is a graph node that copies from pinned host
// memory, so re-uploaded tensors need no re-capture in the FP64 form.
//
// The reference has no multi-system driver: each Atrip::run
// (src/atrip/Atrip.cxx:78-1111) handles one system.  A batch replaces a loop
// of Atrip::run calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "atrip_gb300.h"
#include "context.cuh"
#include "engine.cuh"
#include "split.cuh"

using namespace atrip_gb300;

struct atrip_gpu_batch {
  std::vector<atrip_gpu_context *> sys;  // in the caller's order
  std::vector<int32_t> order;            // table slot -> caller index
  int device = 0, sm_count = 0, max_no = 0;
  TriplesArgs *h_table = nullptr;  // pinned, one descriptor per table slot
  TriplesArgs *d_table = nullptr;
  int64_t *h_prefix = nullptr;  // pinned, n + 1 entries
  int64_t *d_prefix = nullptr;
  unsigned long long *d_queue = nullptr;  // 8 counters per system (own cache line)
  double *d_workspace = nullptr;
  int64_t ws_stride = 0;
  int grid = 0;
  double *d_sums = nullptr, *h_sums = nullptr;  // 2 per table slot
  int *h_status = nullptr;                      // split: one per system
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // captured graph and what it was captured for
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> key;
  int64_t graph_launches = 0;
  atrip_tuning tune = {};  // FP64 batch-kernel launch parameters
  int max_per_sm = 1;      // CTAs per SM the workspace is sized for
  SplitMultiBuffers multi;  // split form: every system in one launch
  bool multi_used = false;  // the captured graph holds that one launch
};

namespace {

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

// Relative per-tuple cost of the FP64 kernel for (No, Nv): row tiles of 64
// (p,q) pairs x column groups of 8 x (Nv + No) K steps.
double tuple_cost(int no, int nv) {
  const double tiles = (double)((no * no + 63) / 64);
  const double cols = (double)((no + 7) / 8);
  return tiles * cols * (double)(nv + no);
}

int split_ctas(const atrip_gpu_context *c) {
  return c->tune.split_ctas > 0 ? std::min(c->sm_count, (int)c->tune.split_ctas) : c->sm_count;
}

void destroy_graph(atrip_gpu_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->key.clear();
}

// Fill the pinned descriptor table from the contexts' current device state.
void fill_table(atrip_gpu_batch *b, int64_t first, int64_t max_it, double tai_sign, bool use_j,
                std::vector<int64_t> &prefix) {
  const int n = (int)b->sys.size();
  prefix.assign(n + 1, 0);
  for (int k = 0; k < n; ++k) {
    atrip_gpu_context *c = b->sys[b->order[k]];
    int64_t t_end = c->n_tuples;
    if (max_it != 0) t_end = std::min<int64_t>(t_end, max_it + 1);
    const int64_t t_begin = std::min<int64_t>(first, t_end);
    TriplesArgs &a = b->h_table[k];
    a.No = c->No;
    a.Nv = c->Nv;
    a.epsi = c->dt.epsi;
    a.epsa = c->dt.epsa;
    a.tai = c->dt.tai;
    a.Ta = c->dt.Ta;
    a.Tp = c->dt.Tp;
    a.Vhh = c->dt.Vhh;
    a.Vht = c->dt.Vht;
    a.Vpt = c->dt.Vpt;
    a.Jht = c->dt.Jht;
    a.Jpt = c->dt.Jpt;
    a.tuples = c->d_tuples;
    a.triples = c->d_triples;
    a.n_triples = c->n_triples;
    a.t_begin = t_begin;
    a.t_end = t_end;
    a.order = nullptr;
    a.queue = b->d_queue + 8 * k;
    a.tai_sign = tai_sign;
    a.use_j = (use_j && c->have[ATRIP_JIJKA] && c->have[ATRIP_JABCI]) ? 1 : 0;
    a.e = c->d_e;
    a.ect = c->d_ect;
    a.workspace = nullptr;
    a.rows_tile = c->tune.fp64_tile_rows == 32 ? 32 : 64;
    a.claim = 1;
    a.min_blocks = 0;
    prefix[k + 1] = prefix[k] + (t_end - t_begin);
  }
}

}  // namespace

extern "C" {

int atrip_gpu_batch_plan(const int32_t *no, const int32_t *nv, int32_t n, int32_t *order) {
  clear_error();
  if (n < 0 || (n > 0 && (!no || !nv || !order))) return fail(ATRIP_ERR_ARGUMENT, "bad arguments");
  std::vector<int32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) {
    return tuple_cost(no[x], nv[x]) > tuple_cost(no[y], nv[y]);
  });
  std::copy(idx.begin(), idx.end(), order);
  return ATRIP_OK;
}

int atrip_gpu_batch_create(atrip_gpu_context *const *systems, int32_t n, atrip_gpu_batch **out) {
  clear_error();
  if (!systems || !out || n <= 0) return fail(ATRIP_ERR_ARGUMENT, "need n >= 1 systems");
  *out = nullptr;
  for (int s = 0; s < n; ++s) {
    if (!systems[s]) return fail(ATRIP_ERR_ARGUMENT, "null system " + std::to_string(s));
    if (systems[s]->device != systems[0]->device)
      return fail(ATRIP_ERR_ARGUMENT, "systems live on different devices");
    if (systems[s]->field != ATRIP_FIELD_REAL)
      return fail(ATRIP_ERR_UNSUPPORTED, "batches hold real-field systems only");
    if (systems[s]->No > kBatchMaxNo)
      return fail(ATRIP_ERR_UNSUPPORTED, "batch systems need No <= " + std::to_string(kBatchMaxNo));
    for (int t = 0; t < s; ++t)
      if (systems[t] == systems[s])
        return fail(ATRIP_ERR_ARGUMENT, "system " + std::to_string(s) + " listed twice");
  }
  auto *b = new atrip_gpu_batch();
  b->sys.assign(systems, systems + n);
  b->device = systems[0]->device;
  b->sm_count = systems[0]->sm_count;
  std::vector<int32_t> no(n), nv(n);
  for (int s = 0; s < n; ++s) {
    no[s] = systems[s]->No;
    nv[s] = systems[s]->Nv;
    b->max_no = std::max(b->max_no, no[s]);
  }
  b->order.resize(n);
  atrip_gpu_batch_plan(no.data(), nv.data(), n, b->order.data());
#define BATCH_TRY(call)                    \
  do {                                     \
    int _rc = [&]() -> int {               \
      ATRIP_CUDA_TRY(call);                \
      return ATRIP_OK;                     \
    }();                                   \
    if (_rc != ATRIP_OK) {                 \
      atrip_gpu_batch_destroy(b);          \
      return _rc;                          \
    }                                      \
  } while (0)
  BATCH_TRY(cudaSetDevice(b->device));
  BATCH_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BATCH_TRY(cudaEventCreate(&b->ev0));
  BATCH_TRY(cudaEventCreate(&b->ev1));
  BATCH_TRY(cudaMallocHost(&b->h_table, sizeof(TriplesArgs) * n));
  BATCH_TRY(cudaMalloc(&b->d_table, sizeof(TriplesArgs) * n));
  BATCH_TRY(cudaMallocHost(&b->h_prefix, sizeof(int64_t) * (n + 1)));
  BATCH_TRY(cudaMalloc(&b->d_prefix, sizeof(int64_t) * (n + 1)));
  BATCH_TRY(cudaMalloc(&b->d_queue, sizeof(unsigned long long) * 8 * (n + 1)));
  BATCH_TRY(cudaMalloc(&b->d_sums, sizeof(double) * 2 * n));
  BATCH_TRY(cudaMallocHost(&b->h_sums, sizeof(double) * 2 * n));
  BATCH_TRY(cudaMallocHost(&b->h_status, sizeof(int) * n));
  b->max_per_sm = std::max({1, triples_fp64_batch_max_blocks_per_sm(b->max_no, 0),
                            triples_fp64_batch_max_blocks_per_sm(b->max_no, 2)});
  b->grid = b->sm_count * std::max(1, triples_fp64_batch_max_blocks_per_sm(b->max_no, 0));
  const int64_t No = b->max_no;
  b->ws_stride = 2 * No * No * No;
  BATCH_TRY(cudaMalloc(&b->d_workspace,
                       sizeof(double) * b->ws_stride * b->sm_count * b->max_per_sm));
#undef BATCH_TRY
  *out = b;
  return ATRIP_OK;
}

int atrip_gpu_batch_run(atrip_gpu_batch *b, const atrip_run_options *opts,
                        atrip_result *results) {
  clear_error();
  if (!b || !opts || !results) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  if (opts->form != ATRIP_FORM_FP64 && opts->form != ATRIP_FORM_SPLIT_BF16 &&
      opts->form != ATRIP_FORM_AUTO && opts->form != ATRIP_FORM_SPLIT_F16)
    return fail(ATRIP_ERR_ARGUMENT, "unknown form " + std::to_string(opts->form));
  if (opts->first_iteration < 0 || opts->max_iterations < 0)
    return fail(ATRIP_ERR_ARGUMENT, "negative iteration bound");
  if (opts->start_energy != 0.0)
    return fail(ATRIP_ERR_ARGUMENT, "start_energy is per system: resume systems one by one");
  const int n = (int)b->sys.size();
  const int needed[] = {ATRIP_EPSI, ATRIP_EPSA, ATRIP_TAI, ATRIP_TABIJ,
                        ATRIP_VABIJ, ATRIP_VIJKA, ATRIP_VABCI};
  for (int s = 0; s < n; ++s)
    for (int t : needed)
      if (!b->sys[s]->have[t])
        return fail(ATRIP_ERR_STATE, "system " + std::to_string(s) + ": input tensor " +
                                         std::to_string(t) + " not uploaded");
  ATRIP_CUDA_TRY(cudaSetDevice(b->device));
  cudaStream_t st = opts->stream ? (cudaStream_t)opts->stream : b->stream;
  const int form = opts->form == ATRIP_FORM_AUTO ? ATRIP_FORM_SPLIT_BF16 : opts->form;
  const int slices = opts->slices > 0 ? opts->slices : form == ATRIP_FORM_SPLIT_F16 ? 2 : 3;
  const double tai_sign = opts->ijkabc ? -1.0 : 1.0;
  std::vector<int64_t> prefix;
  fill_table(b, opts->first_iteration, opts->max_iterations, tai_sign, opts->use_j != 0, prefix);
  std::copy(prefix.begin(), prefix.end(), b->h_prefix);
  int64_t prep_launches = 0;

  // What the captured graph depends on besides the table (copied at replay).
  std::vector<uintptr_t> key = {(uintptr_t)form, (uintptr_t)(form == ATRIP_FORM_FP64 ? 0 : slices),
                                (uintptr_t)prefix[n], (uintptr_t)b->grid,
                                (uintptr_t)b->tune.fp64_min_blocks,
                                (uintptr_t)b->tune.tuples_per_claim};
  if (form != ATRIP_FORM_FP64) {
    // cut every system's operand slices; with one launch for all systems
    // (the default where one shared-memory layout serves them all) the W
    // buffers are the batch's own, so the contexts keep minimal ones
    auto prepare_all = [&](bool one_launch) -> int {
      for (int k = 0; k < n; ++k) {
        atrip_gpu_context *c = b->sys[b->order[k]];
        const TriplesArgs &a = b->h_table[k];
        c->split.stage_cap = c->tune.split_stages;
        c->split.w_global = c->tune.split_w_global != 0;
        c->split.variant = c->tune.split_variant;
        c->split.prefetch = c->tune.split_prefetch != 0;
        c->split.f16 = form == ATRIP_FORM_SPLIT_F16;
        int rc = split_prepare(c->split, c->dt, c->No, c->Nv, one_launch ? 1 : split_ctas(c),
                               a.use_j != 0, slices, a.triples, a.n_triples, st, &prep_launches);
        if (rc != ATRIP_OK) return rc;
      }
      return ATRIP_OK;
    };
    b->multi_used = false;
    if (b->tune.split_variant != 1) {
      int rc = prepare_all(true);
      if (rc != ATRIP_OK) return rc;
      std::vector<SplitMultiSystem> ms(n);
      for (int k = 0; k < n; ++k) {
        atrip_gpu_context *c = b->sys[b->order[k]];
        const TriplesArgs &a = b->h_table[k];
        ms[k] = {&c->split, &c->dt, c->No, c->Nv, a.tuples, a.triples, a.n_triples,
                 a.t_begin, a.t_end, a.use_j != 0, a.e, a.ect};
      }
      rc = split_multi_prepare(ms.data(), n, slices, form == ATRIP_FORM_SPLIT_F16, b->sm_count,
                               b->multi);
      if (rc == ATRIP_OK) b->multi_used = true;
      else if (rc != ATRIP_ERR_UNSUPPORTED) return rc;
      clear_error();
    }
    if (!b->multi_used) {
      const int rc = prepare_all(false);  // one launch per system (batch split_variant 1)
      if (rc != ATRIP_OK) return rc;
    }
    for (int k = 0; k < n; ++k) {
      atrip_gpu_context *c = b->sys[b->order[k]];
      const TriplesArgs &a = b->h_table[k];
      const uintptr_t more[] = {(uintptr_t)c->split.generation, (uintptr_t)c->split.impl,
                                (uintptr_t)a.epsi, (uintptr_t)a.epsa, (uintptr_t)a.tai,
                                (uintptr_t)a.Vhh, (uintptr_t)a.tuples, (uintptr_t)a.triples,
                                (uintptr_t)a.e, (uintptr_t)a.ect, (uintptr_t)a.use_j,
                                (uintptr_t)a.t_begin, (uintptr_t)a.t_end,
                                (uintptr_t)opts->ijkabc, (uintptr_t)c->split.stage_cap,
                                (uintptr_t)c->split.w_global, (uintptr_t)c->split.variant,
                                (uintptr_t)c->split.prefetch,
                                (uintptr_t)split_ctas(c)};
      key.insert(key.end(), std::begin(more), std::end(more));
    }
    const uintptr_t more[] = {(uintptr_t)b->multi_used, (uintptr_t)b->multi.smem,
                              (uintptr_t)b->multi.nstages, (uintptr_t)b->multi.no_lay,
                              (uintptr_t)b->multi.npass_lay, (uintptr_t)b->multi.wglobal,
                              (uintptr_t)b->multi.stage_bytes, (uintptr_t)b->multi.wsmem,
                              (uintptr_t)b->multi.d_desc, (uintptr_t)b->multi.n};
    key.insert(key.end(), std::begin(more), std::end(more));
    // the split operands were cut on st; the capture stream must see them
    ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (!b->exec || key != b->key) {
    destroy_graph(b);
    BatchArgs ba;
    ba.systems = b->d_table;
    ba.prefix = b->d_prefix;
    ba.n = n;
    ba.queue = b->d_queue + 8 * n;
    ba.workspace = b->d_workspace;
    ba.ws_stride = b->ws_stride;
    ba.claim = std::max(1, (int)b->tune.tuples_per_claim);
    int64_t launches = 0;
    cudaGraph_t graph = nullptr;
    ATRIP_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    int rc = [&]() -> int {
      ATRIP_CUDA_TRY(cudaMemcpyAsync(b->d_table, b->h_table, sizeof(TriplesArgs) * n,
                                     cudaMemcpyHostToDevice, b->stream));
      ATRIP_CUDA_TRY(cudaMemcpyAsync(b->d_prefix, b->h_prefix, sizeof(int64_t) * (n + 1),
                                     cudaMemcpyHostToDevice, b->stream));
      ATRIP_CUDA_TRY(
          cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned long long) * 8 * (n + 1), b->stream));
      if (form == ATRIP_FORM_FP64) {
        if (prefix[n] > 0) {
          const int grid = (int)std::min<int64_t>(b->grid, prefix[n]);
          ATRIP_CUDA_TRY(launch_triples_fp64_batch(ba, b->max_no, b->tune.fp64_min_blocks, grid,
                                                   b->stream));
          launches += 1;
        }
      } else if (b->multi_used) {
        ATRIP_CUDA_TRY(cudaMemsetAsync(b->multi.d_status, 0, sizeof(int), b->stream));
        int rc2 = split_multi_enqueue(b->multi, tai_sign, b->sm_count, b->stream, &launches);
        if (rc2 != ATRIP_OK) return rc2;
        ATRIP_CUDA_TRY(cudaMemcpyAsync(b->h_status, b->multi.d_status, sizeof(int),
                                       cudaMemcpyDeviceToHost, b->stream));
      } else {
        for (int k = 0; k < n; ++k) {
          atrip_gpu_context *c = b->sys[b->order[k]];
          const TriplesArgs &a = b->h_table[k];
          if (a.t_end == a.t_begin) continue;
          int rc2 = split_enqueue(c->split, c->dt, c->No, c->Nv, split_ctas(c), a.tuples,
                                  a.triples, a.n_triples, a.t_begin, a.t_end, nullptr, tai_sign,
                                  a.use_j != 0, b->d_queue + 8 * k, a.e, a.ect, b->stream,
                                  &launches);
          if (rc2 != ATRIP_OK) return rc2;
          ATRIP_CUDA_TRY(cudaMemcpyAsync(b->h_status + b->order[k], split_status_ptr(c->split),
                                         sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        }
      }
      ATRIP_CUDA_TRY(launch_batch_energy_sum(ba, b->d_sums, b->stream));
      launches += 1;
      ATRIP_CUDA_TRY(cudaMemcpyAsync(b->h_sums, b->d_sums, sizeof(double) * 2 * n,
                                     cudaMemcpyDeviceToHost, b->stream));
      return ATRIP_OK;
    }();
    cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
    if (rc != ATRIP_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    ATRIP_CUDA_TRY(ce);
    cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    ATRIP_CUDA_TRY(ie);
    b->key = key;
    b->graph_launches = launches;
  }
  std::fill(b->h_status, b->h_status + n, 0);
  ATRIP_CUDA_TRY(cudaEventRecord(b->ev0, st));
  ATRIP_CUDA_TRY(cudaGraphLaunch(b->exec, st));
  ATRIP_CUDA_TRY(cudaEventRecord(b->ev1, st));
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  ATRIP_CUDA_TRY(cudaGetLastError());
  float ms = 0.f;
  ATRIP_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  for (int s = 0; s < n; ++s) {
    const int rc = split_status_check(b->h_status[s]);
    if (rc != ATRIP_OK)
      return fail(rc, "system " + std::to_string(s) + ": " + atrip_gpu_last_error());
  }
  const double sign = opts->ijkabc ? 1.0 : -1.0;  // src/atrip/Atrip.cxx:1108-1111
  for (int k = 0; k < n; ++k) {
    const int s = b->order[k];
    atrip_gpu_context *c = b->sys[s];
    const TriplesArgs &a = b->h_table[k];
    c->e_lo = a.t_begin;
    c->e_hi = a.t_end;
    atrip_result &r = results[s];
    r.energy = sign * b->h_sums[2 * k];
    r.ct_energy = sign * b->h_sums[2 * k + 1];
    r.tuples_done = a.t_end - a.t_begin;
    r.next_iteration = a.t_end;
    r.device_ms = ms;
    r.form_used = form;
    r.slices_used = form == ATRIP_FORM_FP64 ? 0 : slices;
    r.kernel_launches = b->graph_launches + prep_launches;
  }
  return ATRIP_OK;
}

int atrip_gpu_batch_set_tuning(atrip_gpu_batch *b, const atrip_tuning *t) {
  clear_error();
  if (!b || !t) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  if (t->fp64_ctas_per_sm < 0 || t->tuples_per_claim < 0 || t->tuples_per_claim > 64)
    return fail(ATRIP_ERR_ARGUMENT, "tuning value out of range");
  if (t->fp64_min_blocks != 0 && t->fp64_min_blocks != 2)
    return fail(ATRIP_ERR_ARGUMENT, "fp64_min_blocks must be 0 or 2");
  ATRIP_CUDA_TRY(cudaSetDevice(b->device));
  int per_sm = std::max(1, triples_fp64_batch_max_blocks_per_sm(b->max_no, t->fp64_min_blocks));
  if (t->fp64_ctas_per_sm > 0) per_sm = std::min(per_sm, (int)t->fp64_ctas_per_sm);
  per_sm = std::min(per_sm, b->max_per_sm);
  b->tune = *t;
  b->grid = b->sm_count * per_sm;
  return ATRIP_OK;
}

int atrip_gpu_batch_destroy(atrip_gpu_batch *b) {
  if (!b) return ATRIP_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  destroy_graph(b);
  split_multi_free(b->multi);
  cudaFreeHost(b->h_table);
  cudaFreeHost(b->h_prefix);
  cudaFreeHost(b->h_sums);
  cudaFreeHost(b->h_status);
  cudaFree(b->d_table);
  cudaFree(b->d_prefix);
  cudaFree(b->d_queue);
  cudaFree(b->d_sums);
  cudaFree(b->d_workspace);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return ATRIP_OK;
}

}  // extern "C"
