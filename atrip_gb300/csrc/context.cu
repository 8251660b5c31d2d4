// C-ABI entry points: context life cycle, uploads, runs, results.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "atrip_gb300.h"
#include "engine.cuh"
#include "split.cuh"
#include "context.cuh"

namespace atrip_gb300 {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

}  // namespace atrip_gb300

using namespace atrip_gb300;

namespace {

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

// Processing order of tuples [t_begin, t_end) for block side L >= 2: a
// stable counting sort of the list positions by the block triple
// (a/L, b/L, c/L), so that the tuples the persistent CTAs hold at any
// moment read the slabs of few a, b, c values and find them in L2 (in list
// order ~150 tuples in flight touch ~150 different c slabs).  Within a block
// triple the list order is kept.  Writes order[q] = position - t_begin.
int build_order(atrip_gpu_context *c, int64_t t_begin, int64_t t_end, int L, cudaStream_t st) {
  if (c->order_lo == t_begin && c->order_hi == t_end && c->order_block == L && c->d_order)
    return ATRIP_OK;
  const int64_t n = t_end - t_begin;
  while (((int64_t)c->Nv + L - 1) / L > 400) ++L;  // at most 400^3 block triples
  const int64_t nb = (c->Nv + L - 1) / L;
  std::vector<uint32_t> count((size_t)(nb * nb * nb) + 1, 0), out((size_t)n);
  auto key = [&](uint32_t pk) {
    const int64_t a = pk & 0x3ff, b = (pk >> 10) & 0x3ff, cc = (pk >> 20) & 0x3ff;
    return (size_t)(((a / L) * nb + b / L) * nb + cc / L);
  };
  for (int64_t t = t_begin; t < t_end; ++t) count[key(c->h_tuples[(size_t)t]) + 1]++;
  for (size_t k = 1; k < count.size(); ++k) count[k] += count[k - 1];
  for (int64_t t = t_begin; t < t_end; ++t)
    out[count[key(c->h_tuples[(size_t)t])]++] = (uint32_t)(t - t_begin);
  if (n > c->order_cap) {
    cudaFree(c->d_order);
    c->d_order = nullptr;
    c->order_cap = 0;
    ATRIP_CUDA_TRY(cudaMalloc(&c->d_order, sizeof(uint32_t) * (size_t)n));
    c->order_cap = n;
  }
  ATRIP_CUDA_TRY(cudaMemcpyAsync(c->d_order, out.data(), sizeof(uint32_t) * (size_t)n,
                                 cudaMemcpyHostToDevice, st));
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));  // out is released on return
  c->order_lo = t_begin;
  c->order_hi = t_end;
  c->order_block = L;
  return ATRIP_OK;
}

int64_t expected_elements(const atrip_gpu_context *c, int t) {
  const int64_t No = c->No, Nv = c->Nv;
  switch (t) {
    case ATRIP_EPSI: return No;
    case ATRIP_EPSA: return Nv;
    case ATRIP_TAI: return Nv * No;
    case ATRIP_TABIJ:
    case ATRIP_VABIJ: return Nv * Nv * No * No;
    case ATRIP_VIJKA:
    case ATRIP_JIJKA: return No * No * No * Nv;
    case ATRIP_VABCI:
    case ATRIP_JABCI: return Nv * Nv * Nv * No;
    default: return -1;
  }
}

// Shape and source strides of the permutation that takes tensor t from its
// column-major input to its engine layout (see engine.cuh); returns the
// destination buffer(s) through out pointers.
struct PermutePlan {
  double **dst[2] = {nullptr, nullptr};
  int64_t n[2][4];
  int64_t s[2][4];
  int count = 0;
};

PermutePlan plan_for(atrip_gpu_context *c, int t) {
  const int64_t No = c->No, Nv = c->Nv;
  PermutePlan p;
  auto add = [&](double **d, int64_t n0, int64_t n1, int64_t n2, int64_t n3, int64_t s0,
                 int64_t s1, int64_t s2, int64_t s3) {
    p.dst[p.count] = d;
    p.n[p.count][0] = n0; p.n[p.count][1] = n1; p.n[p.count][2] = n2; p.n[p.count][3] = n3;
    p.s[p.count][0] = s0; p.s[p.count][1] = s1; p.s[p.count][2] = s2; p.s[p.count][3] = s3;
    p.count++;
  };
  switch (t) {
    case ATRIP_TABIJ:
      // Ta[x][q][p][E] = T[x,E,p,q]
      add(&c->dt.Ta, Nv, No, No, Nv, Nv, Nv * Nv, Nv * Nv * No, 1);
      // Tp[x][y][n][m] = T[x,y,m,n]
      add(&c->dt.Tp, No, No, Nv, Nv, Nv * Nv, Nv * Nv * No, Nv, 1);
      break;
    case ATRIP_VABIJ: add(&c->dt.Vhh, No, No, Nv, Nv, Nv * Nv, Nv * Nv * No, Nv, 1); break;
    case ATRIP_VIJKA:  // Vht[w][q][p][L] = Vh[p,q,L,w]
      add(&c->dt.Vht, No, No, No, Nv, No * No, 1, No, No * No * No);
      break;
    case ATRIP_JIJKA: add(&c->dt.Jht, No, No, No, Nv, No * No, 1, No, No * No * No); break;
    case ATRIP_VABCI:  // Vpt[y][z][r][E] = Vp[y,z,E,r]
      add(&c->dt.Vpt, Nv, No, Nv, Nv, Nv * Nv, Nv * Nv * Nv, Nv, 1);
      break;
    case ATRIP_JABCI: add(&c->dt.Jpt, Nv, No, Nv, Nv, Nv * Nv, Nv * Nv * Nv, Nv, 1); break;
    default: break;
  }
  return p;
}

double **direct_slot(atrip_gpu_context *c, int t) {
  switch (t) {
    case ATRIP_EPSI: return &c->dt.epsi;
    case ATRIP_EPSA: return &c->dt.epsa;
    case ATRIP_TAI: return &c->dt.tai;
    default: return nullptr;
  }
}

void free_tensor(atrip_gpu_context *c, int t) {
  if (double **d = direct_slot(c, t)) {
    cudaFree(*d);
    *d = nullptr;
  } else {
    PermutePlan p = plan_for(c, t);
    for (int i = 0; i < p.count; ++i) {
      cudaFree(*p.dst[i]);
      *p.dst[i] = nullptr;
    }
  }
  c->have[t] = false;
  split_invalidate(c->split);
}

// Host uploads above this many elements are staged in chunks (default 2^28
// elements, 2 GiB of FP64; ATRIP_GB300_STAGING_ELEMS overrides it).
int64_t staging_elems() {
  static const int64_t v = [] {
    const char *e = std::getenv("ATRIP_GB300_STAGING_ELEMS");
    const long long x = e ? std::atoll(e) : 0;
    return x > 0 ? (int64_t)x : (int64_t(1) << 28);
  }();
  return v;
}

int upload_impl(atrip_gpu_context *c, int32_t tensor, const double *src, int64_t n,
                bool src_on_device) {
  clear_error();
  if (!c) return fail(ATRIP_ERR_ARGUMENT, "null context");
  if (tensor < 0 || tensor >= ATRIP_N_TENSORS)
    return fail(ATRIP_ERR_ARGUMENT, "unknown tensor id " + std::to_string(tensor));
  const int64_t want = expected_elements(c, tensor);
  if (n != want)
    return fail(ATRIP_ERR_ARGUMENT, "tensor " + std::to_string(tensor) + ": got " +
                                        std::to_string(n) + " elements, expected " +
                                        std::to_string(want));
  if (!src && n > 0) return fail(ATRIP_ERR_ARGUMENT, "null source pointer");
  ATRIP_CUDA_TRY(cudaSetDevice(c->device));
  if (c->have[tensor]) free_tensor(c, tensor);
  const cudaMemcpyKind kind = src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const bool cplx = c->field == ATRIP_FIELD_COMPLEX;
  const size_t elem = sizeof(double) * (cplx ? 2 : 1);
  if (double **d = direct_slot(c, tensor)) {
    ATRIP_CUDA_TRY(cudaMalloc(d, elem * std::max<int64_t>(n, 1)));
    ATRIP_CUDA_TRY(cudaMemcpyAsync(*d, src, elem * n, kind, c->stream));
  } else if (!src_on_device && n > staging_elems()) {
    // Large host tensor: stream it through a bounded staging buffer, a run
    // of values of the source's slowest index at a time, so the upload
    // needs the destination layouts plus at most kStagingElems elements.
    PermutePlan p = plan_for(c, tensor);
    const double *hsrc = src;
    for (int i = 0; i < p.count; ++i)
      ATRIP_CUDA_TRY(cudaMalloc(p.dst[i], elem * std::max<int64_t>(n, 1)));
    int dslow[2];
    int64_t m = 0, S = 0;
    for (int i = 0; i < p.count; ++i) {
      int d = 0;
      for (int k = 1; k < 4; ++k)
        if (p.s[i][k] > p.s[i][d]) d = k;
      dslow[i] = d;
      m = p.n[i][d];
      S = p.s[i][d];  // every plan of one tensor has the same source
    }
    const int64_t cv = std::max<int64_t>(1, staging_elems() / S);
    double *staging = nullptr;
    ATRIP_CUDA_TRY(cudaMalloc(&staging, elem * std::min<int64_t>(n, cv * S)));
    int rc = ATRIP_OK;
    for (int64_t v0 = 0; v0 < m && rc == ATRIP_OK; v0 += cv) {
      const int64_t nv = std::min<int64_t>(cv, m - v0);
      // the previous chunk's permutes must be done before the buffer is reused
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(staging, hsrc + (size_t)(v0 * S) * (cplx ? 2 : 1), elem * nv * S,
                            kind, c->stream);
      for (int i = 0; i < p.count && e == cudaSuccess; ++i) {
        int64_t nb[4], t[4];
        for (int k = 0; k < 4; ++k) nb[k] = p.n[i][k];
        t[0] = 1;
        for (int k = 1; k < 4; ++k) t[k] = t[k - 1] * p.n[i][k - 1];
        nb[dslow[i]] = nv;
        double *dst = *p.dst[i] + (size_t)(v0 * t[dslow[i]]) * (cplx ? 2 : 1);
        e = launch_permute4_box(dst, staging, nb, p.s[i], t, c->stream, cplx);
      }
      if (e != cudaSuccess) {
        set_error(std::string("chunked upload: ") + cudaGetErrorString(e));
        rc = e == cudaErrorMemoryAllocation ? ATRIP_ERR_OUT_OF_MEMORY : ATRIP_ERR_CUDA;
      }
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(staging);
    if (rc != ATRIP_OK) return rc;
  } else {
    PermutePlan p = plan_for(c, tensor);
    const double *colmajor = src;
    double *staging = nullptr;
    if (!src_on_device) {
      ATRIP_CUDA_TRY(cudaMalloc(&staging, elem * std::max<int64_t>(n, 1)));
      cudaError_t e = cudaMemcpyAsync(staging, src, elem * n, kind, c->stream);
      if (e != cudaSuccess) {
        cudaFree(staging);
        ATRIP_CUDA_TRY(e);
      }
      colmajor = staging;
    }
    for (int i = 0; i < p.count; ++i) {
      cudaError_t e = cudaMalloc(p.dst[i], elem * std::max<int64_t>(n, 1));
      if (e == cudaSuccess)
        e = launch_permute4(*p.dst[i], colmajor, p.n[i], p.s[i], c->stream, cplx);
      if (e != cudaSuccess) {
        if (staging) {
          cudaStreamSynchronize(c->stream);
          cudaFree(staging);
        }
        ATRIP_CUDA_TRY(e);
      }
    }
    if (staging) {
      ATRIP_CUDA_TRY(cudaStreamSynchronize(c->stream));
      ATRIP_CUDA_TRY(cudaFree(staging));
    }
  }
  ATRIP_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->have[tensor] = true;
  split_invalidate(c->split);
  return ATRIP_OK;
}

}  // namespace

extern "C" {

const char *atrip_gpu_last_error(void) { return g_last_error.c_str(); }

const char *atrip_gpu_version(void) { return "atrip_gb300 0.1 (sm_103a)"; }

int64_t atrip_gpu_n_tuples(int32_t nv) {
  const int64_t n = nv;
  return n < 1 ? 0 : n * (n + 1) * (n + 2) / 6 - n;
}

int atrip_gpu_tuple_at(int32_t nv, int64_t t, int32_t *a, int32_t *b, int32_t *c) {
  clear_error();
  if (!a || !b || !c || t < 0 || t >= atrip_gpu_n_tuples(nv))
    return fail(ATRIP_ERR_ARGUMENT, "tuple index out of range");
  // Walk the lexicographic a <= b <= c list (src/atrip/Tuples.cxx:122-134)
  // block by block: tuples with first index x number (Nv-x)(Nv-x+1)/2 - 1.
  int64_t r = t;
  for (int32_t x = 0; x < nv; ++x) {
    const int64_t m = nv - x, nx = m * (m + 1) / 2 - 1;
    if (r >= nx) {
      r -= nx;
      continue;
    }
    for (int32_t y = x; y < nv; ++y) {
      const int64_t ny = (nv - y) - (y == x ? 1 : 0);  // c in [y, nv), minus a==b==c
      if (r >= ny) {
        r -= ny;
        continue;
      }
      *a = x;
      *b = y;
      *c = (int32_t)(y + r + (y == x ? 1 : 0));
      return ATRIP_OK;
    }
  }
  return fail(ATRIP_ERR_ARGUMENT, "tuple index out of range");
}

int atrip_gpu_create(const atrip_dims *dims, atrip_gpu_context **out) {
  clear_error();
  if (!dims || !out) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  if (dims->no < 1 || dims->no > 64)
    return fail(ATRIP_ERR_UNSUPPORTED, "No must be in [1, 64], got " + std::to_string(dims->no));
  if (dims->nv < 1 || dims->nv > 1023)
    return fail(ATRIP_ERR_UNSUPPORTED, "Nv must be in [1, 1023], got " + std::to_string(dims->nv));
  if (dims->field != ATRIP_FIELD_REAL && dims->field != ATRIP_FIELD_COMPLEX)
    return fail(ATRIP_ERR_ARGUMENT, "unknown field " + std::to_string(dims->field));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(ATRIP_ERR_NO_DEVICE, "no CUDA device visible");
  if (dims->device < 0 || dims->device >= ndev)
    return fail(ATRIP_ERR_ARGUMENT, "device ordinal out of range");
  cudaDeviceProp prop;
  ATRIP_CUDA_TRY(cudaGetDeviceProperties(&prop, dims->device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(ATRIP_ERR_NO_DEVICE, std::string("this build targets sm_103a; device is ") +
                                         prop.name + " sm_" + std::to_string(prop.major) +
                                         std::to_string(prop.minor));
  ATRIP_CUDA_TRY(cudaSetDevice(dims->device));
  auto *c = new atrip_gpu_context();
  c->No = dims->no;
  c->Nv = dims->nv;
  c->device = dims->device;
  c->field = dims->field;
  c->sm_count = prop.multiProcessorCount;
  c->n_tuples = atrip_gpu_n_tuples(c->Nv);
  auto bail = [&](int code) {
    atrip_gpu_destroy(c);
    return code;
  };
#define CREATE_TRY(call)                                                                  \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      set_error(std::string(#call) + ": " + cudaGetErrorString(_e));                      \
      return bail(_e == cudaErrorMemoryAllocation ? ATRIP_ERR_OUT_OF_MEMORY : ATRIP_ERR_CUDA); \
    }                                                                                     \
  } while (0)
  CREATE_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CREATE_TRY(cudaEventCreate(&c->ev0));
  CREATE_TRY(cudaEventCreate(&c->ev1));
  // tuple list, packed a | b << 10 | c << 20 (src/atrip/Tuples.cxx:122-134)
  {
    std::vector<uint32_t> h;
    h.reserve((size_t)c->n_tuples);
    for (uint32_t a = 0; a < (uint32_t)c->Nv; ++a)
      for (uint32_t b = a; b < (uint32_t)c->Nv; ++b)
        for (uint32_t cc = b; cc < (uint32_t)c->Nv; ++cc)
          if (!(a == b && b == cc)) h.push_back(a | (b << 10) | (cc << 20));
    CREATE_TRY(cudaMalloc(&c->d_tuples, sizeof(uint32_t) * std::max<size_t>(h.size(), 1)));
    CREATE_TRY(cudaMemcpy(c->d_tuples, h.data(), sizeof(uint32_t) * h.size(),
                          cudaMemcpyHostToDevice));
    c->h_tuples.swap(h);
  }
  // (i >= j >= k) triples in the loop order of src/atrip/Equations.cxx:111-124
  {
    std::vector<uint32_t> h;
    for (uint32_t k = 0; k < (uint32_t)c->No; ++k)
      for (uint32_t j = k; j < (uint32_t)c->No; ++j)
        for (uint32_t i = j; i < (uint32_t)c->No; ++i) h.push_back(i | (j << 8) | (k << 16));
    c->n_triples = (int)h.size();
    CREATE_TRY(cudaMalloc(&c->d_triples, sizeof(uint32_t) * h.size()));
    CREATE_TRY(cudaMemcpy(c->d_triples, h.data(), sizeof(uint32_t) * h.size(),
                          cudaMemcpyHostToDevice));
  }
  CREATE_TRY(cudaMalloc(&c->d_e, sizeof(double) * std::max<int64_t>(c->n_tuples, 1)));
  CREATE_TRY(cudaMalloc(&c->d_ect, sizeof(double) * std::max<int64_t>(c->n_tuples, 1)));
  CREATE_TRY(cudaMalloc(&c->d_queue, sizeof(unsigned long long) * 4));
  CREATE_TRY(cudaMalloc(&c->d_partials, sizeof(double) * 4 * kSumBlocks));
  CREATE_TRY(cudaMalloc(&c->d_sum, sizeof(double) * 8));
#undef CREATE_TRY
  *out = c;
  return ATRIP_OK;
}

int atrip_gpu_upload(atrip_gpu_context *ctx, int32_t tensor, const double *host, int64_t n) {
  return upload_impl(ctx, tensor, host, n, false);
}

int atrip_gpu_upload_device(atrip_gpu_context *ctx, int32_t tensor, const double *dev, int64_t n) {
  return upload_impl(ctx, tensor, dev, n, true);
}

int atrip_gpu_release(atrip_gpu_context *ctx, int32_t tensor) {
  clear_error();
  if (!ctx) return fail(ATRIP_ERR_ARGUMENT, "null context");
  if (tensor < 0 || tensor >= ATRIP_N_TENSORS) return fail(ATRIP_ERR_ARGUMENT, "unknown tensor id");
  ATRIP_CUDA_TRY(cudaSetDevice(ctx->device));
  if (ctx->have[tensor]) free_tensor(ctx, tensor);
  return ATRIP_OK;
}

int atrip_gpu_run(atrip_gpu_context *c, const atrip_run_options *opts, atrip_result *out) {
  clear_error();
  if (!c || !opts || !out) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  const int needed[] = {ATRIP_EPSI, ATRIP_EPSA, ATRIP_TAI, ATRIP_TABIJ,
                        ATRIP_VABIJ, ATRIP_VIJKA, ATRIP_VABCI};
  for (int t : needed)
    if (!c->have[t])
      return fail(ATRIP_ERR_STATE, "input tensor " + std::to_string(t) + " not uploaded");
  if (opts->form != ATRIP_FORM_FP64 && opts->form != ATRIP_FORM_SPLIT_BF16 &&
      opts->form != ATRIP_FORM_AUTO && opts->form != ATRIP_FORM_SPLIT_F16)
    return fail(ATRIP_ERR_ARGUMENT, "unknown form " + std::to_string(opts->form));
  if (opts->first_iteration < 0 || opts->max_iterations < 0)
    return fail(ATRIP_ERR_ARGUMENT, "negative iteration bound");
  ATRIP_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t st = opts->stream ? (cudaStream_t)opts->stream : c->stream;
  const bool use_j = opts->use_j && c->have[ATRIP_JIJKA] && c->have[ATRIP_JABCI];
  // tuple range: first_iteration .. max_iterations inclusive
  // (src/atrip/Atrip.cxx:686-688, 1052-1056)
  int64_t t_end = c->n_tuples;
  if (opts->max_iterations != 0) t_end = std::min<int64_t>(t_end, opts->max_iterations + 1);
  const int64_t t_begin = std::min<int64_t>(opts->first_iteration, t_end);
  const int64_t n = t_end - t_begin;
  const bool cplx = c->field == ATRIP_FIELD_COMPLEX;
  int form = opts->form == ATRIP_FORM_AUTO ? (cplx ? ATRIP_FORM_FP64 : ATRIP_FORM_SPLIT_BF16)
                                           : opts->form;
  if (cplx && form != ATRIP_FORM_FP64)
    return fail(ATRIP_ERR_UNSUPPORTED, "complex field: only the FP64 form is built");
  const int slices = opts->slices > 0 ? opts->slices : form == ATRIP_FORM_SPLIT_F16 ? 2 : 3;
  int64_t launches = 0;
  const uint32_t *order = nullptr;
  if (n > 0 && c->tune.tuple_block > 1) {
    const int rc = build_order(c, t_begin, t_end, c->tune.tuple_block, st);
    if (rc != ATRIP_OK) return rc;
    order = c->d_order;
  }
  ATRIP_CUDA_TRY(cudaEventRecord(c->ev0, st));
  if (n > 0) {
    ATRIP_CUDA_TRY(cudaMemsetAsync(c->d_queue, 0, sizeof(unsigned long long) * 4, st));
    if (form == ATRIP_FORM_FP64) {
      const int rows_tile = c->tune.fp64_tile_rows == 32 ? 32 : 64;
      const int min_blocks = c->tune.fp64_min_blocks == 2 ? 2 : 0;
      int per_sm = std::max(1, cplx ? triples_z_max_blocks_per_sm(c->No)
                                    : triples_fp64_max_blocks_per_sm(c->No, rows_tile, min_blocks));
      if (c->tune.fp64_ctas_per_sm > 0) per_sm = std::min(per_sm, (int)c->tune.fp64_ctas_per_sm);
      const int64_t grid = std::min<int64_t>((int64_t)c->sm_count * per_sm, n);
      const size_t ws = (size_t)grid * 2 * (cplx ? 2 : 1) * (size_t)c->No * c->No * c->No;
      if (ws > c->workspace_doubles) {
        cudaFree(c->d_workspace);
        c->d_workspace = nullptr;
        c->workspace_doubles = 0;
        ATRIP_CUDA_TRY(cudaMalloc(&c->d_workspace, sizeof(double) * ws));
        c->workspace_doubles = ws;
      }
      TriplesArgs a;
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
      a.order = order;
      a.queue = c->d_queue;
      a.tai_sign = opts->ijkabc ? -1.0 : 1.0;
      a.use_j = use_j ? 1 : 0;
      a.e = c->d_e;
      a.ect = c->d_ect;
      a.workspace = c->d_workspace;
      a.rows_tile = rows_tile;
      a.claim = std::max(1, (int)c->tune.tuples_per_claim);
      a.min_blocks = min_blocks;
      if (cplx)
        ATRIP_CUDA_TRY(launch_triples_z(a, (int)grid, st));
      else
        ATRIP_CUDA_TRY(launch_triples_fp64(a, (int)grid, st));
      launches += 1;
    } else {
      c->split.stage_cap = c->tune.split_stages;
      c->split.w_global = c->tune.split_w_global != 0;
      c->split.variant = c->tune.split_variant;
      c->split.prefetch = c->tune.split_prefetch != 0;
      c->split.wait_cycles = (long long)c->tune.split_wait_kcycles * 1000;
      c->split.unpublished = c->tune.split_test_unpublished != 0;
      c->split.profile = c->tune.split_profile != 0;
      c->split.f16 = form == ATRIP_FORM_SPLIT_F16;
      const int ctas = c->tune.split_ctas > 0 ? std::min(c->sm_count, (int)c->tune.split_ctas)
                                              : c->sm_count;
      int rc = split_run(c->split, c->dt, c->No, c->Nv, ctas, c->d_tuples, c->d_triples,
                         c->n_triples, t_begin, t_end, order, opts->ijkabc ? -1.0 : 1.0, use_j,
                         slices,
                         c->d_queue, c->d_e, c->d_ect, st, &launches);
      if (rc != ATRIP_OK) return rc;
    }
    ATRIP_CUDA_TRY(launch_energy_sum(c->d_e + t_begin, c->d_ect + t_begin, n, c->d_partials,
                                     c->d_sum, st));
    launches += 2;
  }
  ATRIP_CUDA_TRY(cudaEventRecord(c->ev1, st));
  double sums[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (n > 0)
    ATRIP_CUDA_TRY(cudaMemcpyAsync(sums, c->d_sum, sizeof(double) * 6, cudaMemcpyDeviceToHost, st));
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  ATRIP_CUDA_TRY(cudaGetLastError());
  float ms = 0.f;
  ATRIP_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->e_lo = t_begin;
  c->e_hi = t_end;
  for (int k = 0; k < 4; ++k) c->last_sums[k] = sums[2 + k];
  // local energy starts at -checkpoint energy (src/atrip/Atrip.cxx:612-616);
  // final sign flip unless ijkabc (src/atrip/Atrip.cxx:1108-1111)
  const double sign = opts->ijkabc ? 1.0 : -1.0;
  out->energy = sign * (-opts->start_energy + sums[0]);
  out->ct_energy = sign * sums[1];
  out->tuples_done = n;
  out->next_iteration = t_end;
  out->device_ms = ms;
  out->form_used = form;
  out->slices_used = form == ATRIP_FORM_FP64 ? 0 : slices;
  out->kernel_launches = launches;
  return ATRIP_OK;
}

int atrip_gpu_set_tuning(atrip_gpu_context *c, const atrip_tuning *t) {
  clear_error();
  if (!c || !t) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  if (t->fp64_ctas_per_sm < 0 || t->tuples_per_claim < 0 || t->split_ctas < 0)
    return fail(ATRIP_ERR_ARGUMENT, "negative tuning value");
  if (t->fp64_tile_rows != 0 && t->fp64_tile_rows != 32 && t->fp64_tile_rows != 64)
    return fail(ATRIP_ERR_ARGUMENT, "fp64_tile_rows must be 32 or 64");
  if (t->split_variant < 0 || t->split_variant > 3)
    return fail(ATRIP_ERR_ARGUMENT, "split_variant must be 0..3");
  if (t->tuple_block < 0 || t->tuple_block > 1023)
    return fail(ATRIP_ERR_ARGUMENT, "tuple_block must be in [0, 1023]");
  if (t->split_stages != 0 && (t->split_stages < 2 || t->split_stages > 6))
    return fail(ATRIP_ERR_ARGUMENT, "split_stages must be 2..6");
  if (t->tuples_per_claim > 64) return fail(ATRIP_ERR_ARGUMENT, "tuples_per_claim must be <= 64");
  if (t->fp64_min_blocks != 0 && t->fp64_min_blocks != 2)
    return fail(ATRIP_ERR_ARGUMENT, "fp64_min_blocks must be 0 or 2");
  if (t->split_wait_kcycles < 0) return fail(ATRIP_ERR_ARGUMENT, "negative wait limit");
  if (t->split_test_unpublished != 0 && t->split_test_unpublished != 1)
    return fail(ATRIP_ERR_ARGUMENT, "split_test_unpublished must be 0 or 1");
  if (t->split_profile != 0 && t->split_profile != 1)
    return fail(ATRIP_ERR_ARGUMENT, "split_profile must be 0 or 1");
  c->tune = *t;
  return ATRIP_OK;
}

int atrip_gpu_get_tuning(const atrip_gpu_context *c, atrip_tuning *t) {
  clear_error();
  if (!c || !t) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  *t = c->tune;
  return ATRIP_OK;
}

int atrip_gpu_tuple_energies(atrip_gpu_context *c, int64_t t0, int64_t n, double *e, double *ect) {
  clear_error();
  if (!c || (!e && !ect)) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  if (n < 0 || t0 < c->e_lo || t0 + n > c->e_hi)
    return fail(ATRIP_ERR_ARGUMENT, "range outside the last run's tuples");
  ATRIP_CUDA_TRY(cudaSetDevice(c->device));
  if (e) ATRIP_CUDA_TRY(cudaMemcpy(e, c->d_e + t0, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (ect)
    ATRIP_CUDA_TRY(cudaMemcpy(ect, c->d_ect + t0, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return ATRIP_OK;
}

int atrip_gpu_device_count(int32_t *count) {
  clear_error();
  if (!count) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return ATRIP_OK;
}

int atrip_gpu_split_profile(const atrip_gpu_context *c, uint64_t *counters, int32_t n) {
  clear_error();
  if (!c || !counters || n < ATRIP_SPLIT_PROFILE_COUNTERS)
    return fail(ATRIP_ERR_ARGUMENT, "need a buffer of ATRIP_SPLIT_PROFILE_COUNTERS counters");
  cudaSetDevice(c->device);
  static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "counter width");
  return split_profile_read(c->split, reinterpret_cast<unsigned long long *>(counters), n);
}

int atrip_gpu_last_sums(const atrip_gpu_context *c, double *sums) {
  clear_error();
  if (!c || !sums) return fail(ATRIP_ERR_ARGUMENT, "null argument");
  for (int k = 0; k < 4; ++k) sums[k] = c->last_sums[k];
  return ATRIP_OK;
}

int atrip_gpu_destroy(atrip_gpu_context *c) {
  if (!c) return ATRIP_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int t = 0; t < ATRIP_N_TENSORS; ++t)
    if (c->have[t]) free_tensor(c, t);
  split_free(c->split);
  cudaFree(c->d_tuples);
  cudaFree(c->d_triples);
  cudaFree(c->d_e);
  cudaFree(c->d_ect);
  cudaFree(c->d_workspace);
  cudaFree(c->d_queue);
  cudaFree(c->d_partials);
  cudaFree(c->d_sum);
  cudaFree(c->d_order);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return ATRIP_OK;
}

}  // extern "C"
