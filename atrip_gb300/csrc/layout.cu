// Layout transforms applied once at upload time, and the compensated energy
// reduction.
//
// atrip cuts its inputs into slices at start-up (SliceUnion::init ->
// slice_into_buffer, src/atrip/SliceUnion.cxx:305-332,
// src/atrip/Unions.hpp:77-278) and ships them between ranks per tuple.  Here
// every input is re-laid out once in HBM so that every contraction operand
// (a row of T_x, a column of V_yz, ...) is a contiguous run, and is then read
// in place for every tuple.
#include "engine.cuh"

namespace atrip_gb300 {
namespace {

// 4-D permutation as a gather: coalesced stores, strided loads.  Runs once
// per uploaded tensor.
// Box n0 x n1 x n2 x n3: dst[i . t] = src[i . s] (strides in elements).
// With t the packed strides of the box the stores are coalesced.
struct Box4 {
  int64_t n[4], s[4], t[4];
};

template <typename T>
__global__ void permute4_kernel(T *__restrict__ dst, const T *__restrict__ src, Box4 b) {
  const int64_t total = b.n[0] * b.n[1] * b.n[2] * b.n[3];
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = idx;
    const int64_t i0 = r % b.n[0];
    r /= b.n[0];
    const int64_t i1 = r % b.n[1];
    r /= b.n[1];
    const int64_t i2 = r % b.n[2];
    const int64_t i3 = r / b.n[2];
    dst[i0 * b.t[0] + i1 * b.t[1] + i2 * b.t[2] + i3 * b.t[3]] =
        src[i0 * b.s[0] + i1 * b.s[1] + i2 * b.s[2] + i3 * b.s[3]];
  }
}

// Neumaier accumulation of (s, c) += x.
__device__ __forceinline__ void neumaier(double &s, double &c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x))
    c += (s - t) + x;
  else
    c += (x - t) + s;
  s = t;
}

constexpr int kSumThreads = 256;

// Deterministic compensated sum: block b reduces the contiguous chunk b of
// x and y; partials[4 b .. 4 b + 3] = (sx, cx, sy, cy).
__global__ void energy_sum_stage1(const double *__restrict__ x, const double *__restrict__ y,
                                  int64_t n, double *__restrict__ partials) {
  __shared__ double sh[4][kSumThreads];
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double sx = 0, cx = 0, sy = 0, cy = 0;
  for (int64_t t = lo + threadIdx.x; t < hi; t += kSumThreads) {
    neumaier(sx, cx, x[t]);
    neumaier(sy, cy, y[t]);
  }
  sh[0][threadIdx.x] = sx;
  sh[1][threadIdx.x] = cx;
  sh[2][threadIdx.x] = sy;
  sh[3][threadIdx.x] = cy;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
    for (int i = 0; i < kSumThreads; ++i) {
      neumaier(s0, c0, sh[0][i]);
      c0 += sh[1][i];
      neumaier(s1, c1, sh[2][i]);
      c1 += sh[3][i];
    }
    partials[4 * blockIdx.x + 0] = s0;
    partials[4 * blockIdx.x + 1] = c0;
    partials[4 * blockIdx.x + 2] = s1;
    partials[4 * blockIdx.x + 3] = c1;
  }
}

__global__ void energy_sum_stage2(const double *__restrict__ partials, int nb,
                                  double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
    for (int b = 0; b < nb; ++b) {
      neumaier(s0, c0, partials[4 * b + 0]);
      c0 += partials[4 * b + 1];
      neumaier(s1, c1, partials[4 * b + 2]);
      c1 += partials[4 * b + 3];
    }
    out[0] = s0 + c0;
    out[1] = s1 + c1;
    // the compensated pairs themselves, for exact merging across processes
    out[2] = s0;
    out[3] = c0;
    out[4] = s1;
    out[5] = c1;
  }
}

}  // namespace

cudaError_t launch_permute4_box(double *dst, const double *src, const int64_t n[4],
                                const int64_t s[4], const int64_t t[4], cudaStream_t st,
                                bool complex_elems) {
  Box4 b;
  for (int d = 0; d < 4; ++d) {
    b.n[d] = n[d];
    b.s[d] = s[d];
    b.t[d] = t[d];
  }
  const int64_t total = n[0] * n[1] * n[2] * n[3];
  if (total == 0) return cudaSuccess;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  if (complex_elems)
    permute4_kernel<double2><<<(int)blocks, 256, 0, st>>>(
        reinterpret_cast<double2 *>(dst), reinterpret_cast<const double2 *>(src), b);
  else
    permute4_kernel<double><<<(int)blocks, 256, 0, st>>>(dst, src, b);
  return cudaGetLastError();
}

cudaError_t launch_permute4(double *dst, const double *src, const int64_t n[4], const int64_t s[4],
                            cudaStream_t st, bool complex_elems) {
  const int64_t t[4] = {1, n[0], n[0] * n[1], n[0] * n[1] * n[2]};
  return launch_permute4_box(dst, src, n, s, t, st, complex_elems);
}

cudaError_t launch_energy_sum(const double *x, const double *y, int64_t n, double *partials,
                              double *out, cudaStream_t st) {
  energy_sum_stage1<<<kSumBlocks, kSumThreads, 0, st>>>(x, y, n, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  energy_sum_stage2<<<1, 32, 0, st>>>(partials, kSumBlocks, out);
  return cudaGetLastError();
}

}  // namespace atrip_gb300
