// Plain-FP64 form, one system per launch: the persistent kernel over one
// context's tuple range (per-tuple work in fp64_tuple.cuh).
#include "fp64_tuple.cuh"

namespace atrip_gb300 {
namespace {

// A CTA claims g.claim consecutive tuples per queue access.  MINB = 0 leaves
// the register budget to the compiler; MINB = 2 caps it at 128 registers
// (two resident CTAs per SM, no spills).
template <int NC, int RU, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) triples_fp64_kernel(TriplesArgs g) {
  __shared__ Smem sm;
  __shared__ SinglesCtx s;
  const int64_t No3 = (int64_t)g.No * g.No * g.No;
  double *Wv = g.workspace + (int64_t)blockIdx.x * 2 * No3;
  double *Wj = Wv + No3;
  const int64_t n = g.t_end - g.t_begin;
  const int claim = g.claim > 0 ? g.claim : 1;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long q = atomicAdd(g.queue, (unsigned long long)claim);
      sm.tuple_slot = (q < (unsigned long long)n) ? (long long)q : -1;
    }
    __syncthreads();
    const long long slot = sm.tuple_slot;
    __syncthreads();
    if (slot < 0) break;
    const int64_t last = slot + claim < n ? slot + claim : n;
    for (int64_t u = slot; u < last; ++u)
      process_tuple<NC, RU>(g, sm, s, Wv, Wj, g.t_begin + (g.order ? (int64_t)g.order[u] : u));
  }
}

template <int NC, int RU, int MINB>
cudaError_t launch_v(const TriplesArgs &a, int grid, cudaStream_t s) {
  triples_fp64_kernel<NC, RU, MINB><<<grid, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

template <int NC>
cudaError_t launch_nc(const TriplesArgs &a, int grid, cudaStream_t s) {
  if (a.rows_tile == 32) return launch_v<NC, 1, 0>(a, grid, s);
  if (a.min_blocks == 2) return launch_v<NC, 2, 2>(a, grid, s);
  return launch_v<NC, 2, 0>(a, grid, s);
}

template <int NC>
int blocks_nc(int rows_tile, int min_blocks) {
  int n = 0;
  cudaError_t e;
  if (rows_tile == 32)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_fp64_kernel<NC, 1, 0>,
                                                      kThreads, 0);
  else if (min_blocks == 2)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_fp64_kernel<NC, 2, 2>,
                                                      kThreads, 0);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_fp64_kernel<NC, 2, 0>,
                                                      kThreads, 0);
  return e == cudaSuccess ? n : 0;
}

}  // namespace

cudaError_t launch_triples_fp64(const TriplesArgs &a, int grid, cudaStream_t s) {
  switch ((a.No + 7) / 8) {
    case 1: return launch_nc<1>(a, grid, s);
    case 2: return launch_nc<2>(a, grid, s);
    case 3: return launch_nc<3>(a, grid, s);
    case 4: return launch_nc<4>(a, grid, s);
    case 5: return launch_nc<5>(a, grid, s);
    case 6: return launch_nc<6>(a, grid, s);
    case 7: return launch_nc<7>(a, grid, s);
    case 8: return launch_nc<8>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

int triples_fp64_max_blocks_per_sm(int No, int rows_tile, int min_blocks) {
  switch ((No + 7) / 8) {
    case 1: return blocks_nc<1>(rows_tile, min_blocks);
    case 2: return blocks_nc<2>(rows_tile, min_blocks);
    case 3: return blocks_nc<3>(rows_tile, min_blocks);
    case 4: return blocks_nc<4>(rows_tile, min_blocks);
    case 5: return blocks_nc<5>(rows_tile, min_blocks);
    case 6: return blocks_nc<6>(rows_tile, min_blocks);
    case 7: return blocks_nc<7>(rows_tile, min_blocks);
    case 8: return blocks_nc<8>(rows_tile, min_blocks);
    default: return 0;
  }
}

}  // namespace atrip_gb300
