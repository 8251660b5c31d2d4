// Plain-FP64 form, many systems per launch (the batching form's kernel and
// its per-system energy reduction; per-tuple work in fp64_tuple.cuh).
#include "fp64_tuple.cuh"

namespace atrip_gb300 {
namespace {

// process_tuple<nc, RU> for the system's own column count nc <= NC and row
// tile, so a small system in a mixed batch does not pay for the largest
// system's tile width.
template <int NC>
__device__ void process_tuple_nc(int nc, const TriplesArgs &g, Smem &sm, SinglesCtx &s,
                                 double *Wv, double *Wj, int64_t t) {
  if constexpr (NC > 1) {
    if (nc < NC) {
      process_tuple_nc<NC - 1>(nc, g, sm, s, Wv, Wj, t);
      return;
    }
  }
  if (g.rows_tile == 32)
    process_tuple<NC, 1>(g, sm, s, Wv, Wj, t);
  else
    process_tuple<NC, 2>(g, sm, s, Wv, Wj, t);
}

// Many systems in one persistent launch: a single work-queue cursor runs over
// the concatenated tuple ranges of all systems (prefix[s] .. prefix[s+1]);
// each tuple is processed with its system's descriptor.  MINB as in the
// single-system kernel.
template <int NC, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) triples_fp64_batch_kernel(BatchArgs bt) {
  __shared__ Smem sm;
  __shared__ SinglesCtx s;
  __shared__ TriplesArgs sg;
  __shared__ long long base;
  double *Wv = bt.workspace + (int64_t)blockIdx.x * bt.ws_stride;
  double *Wj = Wv + bt.ws_stride / 2;
  const int64_t total = bt.prefix[bt.n];
  const int claim = bt.claim > 0 ? bt.claim : 1;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long q = atomicAdd(bt.queue, (unsigned long long)claim);
      base = q < (unsigned long long)total ? (long long)q : -1;
    }
    __syncthreads();
    const long long q0 = base;
    if (q0 < 0) break;
    const int64_t last = q0 + claim < total ? q0 + claim : total;
    for (int64_t q = q0; q < last; ++q) {
      if (threadIdx.x == 0) {
        int lo = 0, hi = bt.n;  // prefix[lo] <= q < prefix[hi]
        while (hi - lo > 1) {
          const int mid = (lo + hi) / 2;
          if (q >= bt.prefix[mid]) lo = mid; else hi = mid;
        }
        sm.tuple_slot = q - bt.prefix[lo];
        sg = bt.systems[lo];
      }
      __syncthreads();
      process_tuple_nc<NC>((sg.No + 7) / 8, sg, sm, s, Wv, Wj, sg.t_begin + sm.tuple_slot);
    }
  }
}

// Per-system compensated sums of e and ect (block s reduces system s, in a
// fixed order): sums[2 s], sums[2 s + 1].
__global__ void batch_energy_sum(BatchArgs bt, double *sums) {
  __shared__ double sh[4][kThreads];
  const TriplesArgs &g = bt.systems[blockIdx.x];
  const int64_t n = g.t_end - g.t_begin;
  double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
  auto neu = [](double &sv, double &cv, double x) {
    const double t = sv + x;
    if (fabs(sv) >= fabs(x)) cv += (sv - t) + x; else cv += (x - t) + sv;
    sv = t;
  };
  for (int64_t t = threadIdx.x; t < n; t += kThreads) {
    neu(s0, c0, g.e[g.t_begin + t]);
    neu(s1, c1, g.ect[g.t_begin + t]);
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = c0;
  sh[2][threadIdx.x] = s1;
  sh[3][threadIdx.x] = c1;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0, b0 = 0, a1 = 0, b1 = 0;
    for (int i = 0; i < kThreads; ++i) {
      neu(a0, b0, sh[0][i]);
      b0 += sh[1][i];
      neu(a1, b1, sh[2][i]);
      b1 += sh[3][i];
    }
    sums[2 * blockIdx.x] = a0 + b0;
    sums[2 * blockIdx.x + 1] = a1 + b1;
  }
}

template <int NC>
cudaError_t launch_batch_nc(const BatchArgs &b, int min_blocks, int grid, cudaStream_t st) {
  if (min_blocks == 2)
    triples_fp64_batch_kernel<NC, 2><<<grid, kThreads, 0, st>>>(b);
  else
    triples_fp64_batch_kernel<NC, 0><<<grid, kThreads, 0, st>>>(b);
  return cudaGetLastError();
}

template <int NC>
int batch_blocks_nc(int min_blocks) {
  int n = 0;
  const cudaError_t e =
      min_blocks == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            &n, triples_fp64_batch_kernel<NC, 2>, kThreads, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            &n, triples_fp64_batch_kernel<NC, 0>, kThreads, 0);
  return e == cudaSuccess ? n : 0;
}

}  // namespace

cudaError_t launch_triples_fp64_batch(const BatchArgs &b, int max_no, int min_blocks, int grid,
                                      cudaStream_t s) {
  switch ((max_no + 7) / 8) {
    case 1: return launch_batch_nc<1>(b, min_blocks, grid, s);
    case 2: return launch_batch_nc<2>(b, min_blocks, grid, s);
    case 3: return launch_batch_nc<3>(b, min_blocks, grid, s);
    case 4: return launch_batch_nc<4>(b, min_blocks, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_batch_energy_sum(const BatchArgs &b, double *sums, cudaStream_t s) {
  batch_energy_sum<<<b.n, kThreads, 0, s>>>(b, sums);
  return cudaGetLastError();
}

int triples_fp64_batch_max_blocks_per_sm(int max_no, int min_blocks) {
  switch ((max_no + 7) / 8) {
    case 1: return batch_blocks_nc<1>(min_blocks);
    case 2: return batch_blocks_nc<2>(min_blocks);
    case 3: return batch_blocks_nc<3>(min_blocks);
    case 4: return batch_blocks_nc<4>(min_blocks);
    default: return 0;
  }
}

}  // namespace atrip_gb300
