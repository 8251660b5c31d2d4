// FP64 triples loop for callers that must not allocate device memory.
//
// Who needs this: hosts whose device memory is owned by someone else -- a
// quantum-chemistry code that reserves all of HBM for its own pool allocator
// at start-up, a framework that forbids cudaMalloc/cudaFree on its worker
// threads because they synchronise the whole device, or a library running
// inside such a host.  They already hold the inputs and the outputs in their
// own buffers; atrip_gpu_run_fp64_noalloc only needs those pointers.
//
// The scratch this kernel needs (the work-queue cursor, the per-CTA W
// buffers and the partial sums of the energy reduction) lives in one
// file-scope __device__ array of fixed size, kNoallocScratchBytes.  Every
// GPU that loads this library reserves that array until the process exits.
// Calls share it: the cursor is cleared by each call, and two calls whose
// kernels overlap on the GPU (different streams, or different host threads)
// race on it -- serialise them.
//
// Operands are read straight from the caller's column-major FP64 tensors
// (the layout CTF's read_all returns), so there is no upload, no re-layout
// and no tuple table: tuples are decoded from their list position and the
// (i >= j >= k) triples are enumerated in the energy loop.  The arithmetic
// is the same as the FP64 form of atrip_gpu_run (six fused particle+hole
// contractions written into W at their index permutations, Z = W + singles,
// the get_energy_{distinct,same} terms of src/atrip/Equations.cxx:101-238).
#include <cuda_runtime.h>

#include <string>

#include "atrip_gb300.h"
#include "engine.cuh"

namespace atrip_gb300 {
namespace noalloc {

constexpr size_t kScratchBytes = size_t(32) << 20;  // kNoallocScratchBytes, 32 MiB
constexpr size_t kHeaderBytes = 256;                // cursor + status
constexpr int kPartialBlocks = 128;                 // energy reduction partials
constexpr size_t kPartialBytes = sizeof(double) * 4 * kPartialBlocks;
constexpr size_t kWorkspaceOffset = kHeaderBytes + kPartialBytes;
constexpr int kThreads = 256;
constexpr int kMT = 64;
constexpr int kKC = 32;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct Args {
  int No, Nv;
  const double *epsi, *epsa, *tai, *T, *Vpp, *Vh, *Vp, *Jh, *Jp;
  int64_t t_begin, t_end;
  double tai_sign;
  int use_j;
  int ijkabc;
  double *e, *ect, *energies;
  unsigned char *scratch;  // device address of g_scratch
};

// (a,b,c) of list position t: walk the lexicographic a <= b <= c list
// (src/atrip/Tuples.cxx:122-134) block by block.
__device__ void decode_tuple(int64_t t, int Nv, int &a, int &b, int &c) {
  int64_t r = t;
  for (int x = 0; x < Nv; ++x) {
    const int64_t m = Nv - x, nx = m * (m + 1) / 2 - 1;
    if (r >= nx) { r -= nx; continue; }
    for (int y = x; y < Nv; ++y) {
      const int64_t ny = (Nv - y) - (y == x ? 1 : 0);
      if (r >= ny) { r -= ny; continue; }
      a = x;
      b = y;
      c = (int)(y + r + (y == x ? 1 : 0));
      return;
    }
  }
  a = b = c = 0;
}

struct Smem {
  double As[kKC][kMT + 1];
  double Bs[kKC][64 + 1];
  double red[kThreads / 32][2];
  long long slot;
  double ta[64], tb[64], tc[64];
};

// W = sum of the six fused terms, operands read in column-major order.
template <int NC>
__device__ void build_w(const Args &g, Smem &sm, double *W, const double *Vh, const double *Vp,
                        int a, int b, int c) {
  const int64_t No = g.No, Nv = g.Nv, No2 = No * No, NvNv = Nv * Nv;
  const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
  for (int t = 0; t < 6; ++t) {
    int x, w, y, z, u, v, holeT, sp, sq, sr;
    switch (t) {
      case 0: x = a; w = b; y = b; z = c; u = a; v = c; holeT = 0; sp = 1; sq = No; sr = No2; break;
      case 1: x = a; w = c; y = c; z = b; u = a; v = b; holeT = 0; sp = 1; sq = No2; sr = No; break;
      case 2: x = c; w = a; y = a; z = b; u = b; v = c; holeT = 1; sp = No2; sq = 1; sr = No; break;
      case 3: x = c; w = b; y = b; z = a; u = a; v = c; holeT = 1; sp = No2; sq = No; sr = 1; break;
      case 4: x = b; w = a; y = a; z = c; u = b; v = c; holeT = 0; sp = No; sq = 1; sr = No2; break;
      default: x = b; w = c; y = c; z = a; u = a; v = b; holeT = 1; sp = No; sq = No2; sr = 1; break;
    }
    for (int m0 = 0; m0 < No2; m0 += kMT) {
      double acc[2][NC];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < NC; ++j) acc[i][j] = 0.0;
      for (int seg = 0; seg < 2; ++seg) {
        const int K = seg == 0 ? (int)Nv : (int)No;
        for (int k0 = 0; k0 < K; k0 += kKC) {
          // particle rows T[x,E,p,q] are read with consecutive threads on
          // E (stride Nv), hole rows Vh[p,q,L,w] on p (contiguous): the
          // nearest addresses this column-major layout offers
          for (int idx = tid; idx < kMT * kKC; idx += kThreads) {
            const int row = seg == 0 ? idx / kKC : idx % kMT;
            const int kk = seg == 0 ? idx % kKC : idx / kMT;
            const int64_t m = m0 + row, k = k0 + kk;
            double val = 0.0;
            if (m < No2 && k < K) {
              const int64_t p = m % No, q = m / No;
              val = seg == 0 ? g.T[x + k * Nv + p * NvNv + q * NvNv * No]   // T[x,E,p,q]
                             : Vh[p + q * No + k * No2 + (int64_t)w * No2 * No];  // Vh[p,q,L,w]
            }
            sm.As[kk][row] = val;
          }
          for (int idx = tid; idx < NC * 8 * kKC; idx += kThreads) {
            // V_pphp columns Vp[y,z,E,r]: consecutive threads on E (stride Nv^2)
            const int col = seg == 0 ? idx / kKC : idx % (NC * 8);
            const int kk = seg == 0 ? idx % kKC : idx / (NC * 8);
            const int64_t k = k0 + kk;
            double val = 0.0;
            if (col < No && k < K) {
              if (seg == 0)
                val = Vp[y + z * Nv + k * NvNv + (int64_t)col * NvNv * Nv];  // Vp[y,z,E,r]
              else
                val = -(holeT ? g.T[u + v * Nv + col * NvNv + k * NvNv * No]     // T[u,v,r,L]
                              : g.T[u + v * Nv + k * NvNv + col * NvNv * No]);   // T[u,v,L,r]
            }
            sm.Bs[kk][col] = val;
          }
          __syncthreads();
#pragma unroll 8
          for (int kk = 0; kk < kKC; ++kk) {
            const double a0 = sm.As[kk][ty], a1 = sm.As[kk][ty + 32];
#pragma unroll
            for (int j = 0; j < NC; ++j) {
              const double bv = sm.Bs[kk][tx + 8 * j];
              acc[0][j] = fma(a0, bv, acc[0][j]);
              acc[1][j] = fma(a1, bv, acc[1][j]);
            }
          }
          __syncthreads();
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int m = m0 + ty + 32 * i;
        if (m < No2) {
          const int p = m % No, q = m / No;
#pragma unroll
          for (int j = 0; j < NC; ++j) {
            const int r = tx + 8 * j;
            if (r < No) {
              const int idx = p * sp + q * sq + r * sr;
              W[idx] = (t == 0 ? 0.0 : W[idx]) + acc[i][j];
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

// Z at (i,j,k): W + t1 (x) Vpphh (src/atrip/Equations.cxx:420-422).
__device__ __forceinline__ double zval(const Args &g, const Smem &sm, const double *W, int a, int b,
                                       int c, int i, int j, int k) {
  const int64_t No = g.No, Nv = g.Nv, NvNv = Nv * Nv;
  double z = W[i + No * j + No * No * k];
  z += sm.ta[i] * g.Vpp[b + c * Nv + j * NvNv + k * NvNv * No];
  z += sm.tb[j] * g.Vpp[a + c * Nv + i * NvNv + k * NvNv * No];
  z += sm.tc[k] * g.Vpp[a + b * Nv + i * NvNv + j * NvNv * No];
  return z;
}

__device__ double energy_partial(const Args &g, const Smem &sm, const double *Tb, const double *Wz,
                                 int a, int b, int c, bool distinct, double epsabc) {
  const int No = g.No;
  double sum = 0.0;
  for (int n = threadIdx.x; n < No * No * No; n += kThreads) {
    const int i = n % No, j = (n / No) % No, k = n / (No * No);
    if (i < j || j < k) continue;
    const double facjk = j == k ? 0.5 : 1.0, facij = i == j ? 0.5 : 1.0;
    const double denominator = epsabc - ((g.epsi[i] + g.epsi[j]) + g.epsi[k]);
    double value;
    if (distinct) {
      const double U = zval(g, sm, Wz, a, b, c, i, j, k), V = zval(g, sm, Wz, a, b, c, i, k, j),
                   W = zval(g, sm, Wz, a, b, c, j, i, k), X = zval(g, sm, Wz, a, b, c, j, k, i),
                   Y = zval(g, sm, Wz, a, b, c, k, i, j), Z = zval(g, sm, Wz, a, b, c, k, j, i);
      const double A = Tb[i + No * j + No * No * k], B = Tb[i + No * k + No * No * j],
                   C = Tb[j + No * i + No * No * k], D = Tb[j + No * k + No * No * i],
                   E = Tb[k + No * i + No * No * j], F = Tb[k + No * j + No * No * i];
      const double UXY = U + (X + Y), VWZ = V + (W + Z), ADE = A + (D + E), BCF = B + (C + F);
      const double first = A * U + (B * V + (C * W + (D * X + (E * Y + F * Z))));
      value = 3.0 * first + ((UXY - 2.0 * VWZ) * ADE + (VWZ - 2.0 * UXY) * BCF);
    } else {
      const double U = zval(g, sm, Wz, a, b, c, i, j, k), V = zval(g, sm, Wz, a, b, c, j, k, i),
                   W = zval(g, sm, Wz, a, b, c, k, i, j);
      const double A = Tb[i + No * j + No * No * k], B = Tb[j + No * k + No * No * i],
                   C = Tb[k + No * i + No * No * j];
      value = 3.0 * ((A * U + B * V) + C * W) - (A + (B + C)) * (U + (V + W));
    }
    sum += (2.0 * value / denominator) * (facjk * facij);
  }
  return sum;
}

__device__ double block_sum(double v, Smem &sm, int slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5][slot] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) r += sm.red[w][slot];
  return r;
}

template <int NC>
__global__ void __launch_bounds__(kThreads) triples_noalloc_kernel(Args g) {
  __shared__ Smem sm;
  unsigned long long *cursor = reinterpret_cast<unsigned long long *>(g.scratch);
  const int64_t No3 = (int64_t)g.No * g.No * g.No;
  double *Wv = reinterpret_cast<double *>(g.scratch + kWorkspaceOffset) + blockIdx.x * 2 * No3;
  double *Wj = Wv + No3;
  const int64_t n = g.t_end - g.t_begin;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long q = atomicAdd(cursor, 1ull);
      sm.slot = q < (unsigned long long)n ? (long long)q : -1;
    }
    __syncthreads();
    const long long slot = sm.slot;
    __syncthreads();
    if (slot < 0) break;
    const int64_t t = g.t_begin + slot;
    int a, b, c;
    decode_tuple(t, g.Nv, a, b, c);
    if (threadIdx.x < g.No) {
      const int i = threadIdx.x;
      sm.ta[i] = g.tai_sign * g.tai[a + (int64_t)i * g.Nv];
      sm.tb[i] = g.tai_sign * g.tai[b + (int64_t)i * g.Nv];
      sm.tc[i] = g.tai_sign * g.tai[c + (int64_t)i * g.Nv];
    }
    build_w<NC>(g, sm, Wv, g.Vh, g.Vp, a, b, c);
    int cls = 0;  // src/atrip/Atrip.cxx:640-642
    if (a == b) cls++;
    if (b == c) cls--;
    const double epsabc = g.epsa[a] + g.epsa[b] + g.epsa[c];
    const double e = block_sum(energy_partial(g, sm, Wv, Wv, a, b, c, cls == 0, epsabc), sm, 0);
    double ect = e;
    if (g.use_j) {
      build_w<NC>(g, sm, Wj, g.Jh, g.Jp, a, b, c);
      ect = block_sum(energy_partial(g, sm, Wj, Wv, a, b, c, cls == 0, epsabc), sm, 1);
    }
    if (threadIdx.x == 0) {
      g.e[slot] = e;
      g.ect[slot] = ect;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void neumaier(double &s, double &c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x))
    c += (s - t) + x;
  else
    c += (x - t) + s;
  s = t;
}

// Compensated sum of e[0..n), ect[0..n) into the caller's energies[0..1],
// with the sign of src/atrip/Atrip.cxx:1108-1111.
__global__ void noalloc_sum_stage1(Args g, int64_t n) {
  __shared__ double sh[4][kThreads];
  double *partials = reinterpret_cast<double *>(g.scratch + kHeaderBytes);
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
  for (int64_t t = lo + threadIdx.x; t < hi; t += kThreads) {
    neumaier(s0, c0, g.e[t]);
    neumaier(s1, c1, g.ect[t]);
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = c0;
  sh[2][threadIdx.x] = s1;
  sh[3][threadIdx.x] = c1;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0, b0 = 0, a1 = 0, b1 = 0;
    for (int i = 0; i < kThreads; ++i) {
      neumaier(a0, b0, sh[0][i]);
      b0 += sh[1][i];
      neumaier(a1, b1, sh[2][i]);
      b1 += sh[3][i];
    }
    partials[4 * blockIdx.x + 0] = a0;
    partials[4 * blockIdx.x + 1] = b0;
    partials[4 * blockIdx.x + 2] = a1;
    partials[4 * blockIdx.x + 3] = b1;
  }
}

__global__ void noalloc_sum_stage2(Args g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double *partials = reinterpret_cast<const double *>(g.scratch + kHeaderBytes);
  double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
  for (int b = 0; b < kPartialBlocks; ++b) {
    neumaier(s0, c0, partials[4 * b + 0]);
    c0 += partials[4 * b + 1];
    neumaier(s1, c1, partials[4 * b + 2]);
    c1 += partials[4 * b + 3];
  }
  const double sign = g.ijkabc ? 1.0 : -1.0;
  g.energies[0] = sign * (s0 + c0);
  g.energies[1] = sign * (s1 + c1);
}

template <int NC>
int launch(const Args &a, int device, cudaStream_t st) {
  int per_sm = 0, sms = 0;
  ATRIP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, triples_noalloc_kernel<NC>,
                                                               kThreads, 0));
  ATRIP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const size_t per_cta = sizeof(double) * 2 * (size_t)a.No * a.No * a.No;
  const int64_t fit = (int64_t)((kScratchBytes - kWorkspaceOffset) / per_cta);
  int64_t grid = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
  if (grid > fit) grid = fit;
  const int64_t n = a.t_end - a.t_begin;
  if (grid > n) grid = n;
  if (grid < 1) grid = 1;
  triples_noalloc_kernel<NC><<<(int)grid, kThreads, 0, st>>>(a);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}

// Device address of g_scratch on the current device.  Looked up on every
// call (cudaGetSymbolAddress is a cheap table lookup once the module is
// loaded): an address cached across calls would go stale after a
// cudaDeviceReset or a re-created primary context, which loads the module
// again elsewhere.
unsigned char *scratch_address(int *status) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetSymbolAddress(g_scratch): ") + cudaGetErrorString(e));
    *status = ATRIP_ERR_CUDA;
    return nullptr;
  }
  *status = ATRIP_OK;
  return static_cast<unsigned char *>(p);
}

}  // namespace noalloc
}  // namespace atrip_gb300

using namespace atrip_gb300;

extern "C" int atrip_gpu_run_fp64_noalloc(int32_t no, int32_t nv, const atrip_device_inputs *in,
                                          int64_t first_iteration, int64_t max_iterations,
                                          int32_t ijkabc, int32_t use_j, double *tuple_e,
                                          double *tuple_ect, double *energies, void *stream) {
  clear_error();
  if (!in || !tuple_e || !tuple_ect || !energies) {
    set_error("null argument");
    return ATRIP_ERR_ARGUMENT;
  }
  if (no < 1 || no > 64 || nv < 1 || nv > 1023) {
    set_error("No must be in [1, 64] and Nv in [1, 1023]");
    return ATRIP_ERR_UNSUPPORTED;
  }
  if (!in->epsi || !in->epsa || !in->tai || !in->tabij || !in->vabij || !in->vijka || !in->vabci) {
    set_error("a required input pointer is null");
    return ATRIP_ERR_ARGUMENT;
  }
  if (first_iteration < 0 || max_iterations < 0) {
    set_error("negative iteration bound");
    return ATRIP_ERR_ARGUMENT;
  }
  const size_t per_cta = sizeof(double) * 2 * (size_t)no * no * no;
  if (per_cta > noalloc::kScratchBytes - noalloc::kWorkspaceOffset) {
    set_error("No=" + std::to_string(no) + " needs " + std::to_string(per_cta) +
              " bytes of scratch per CTA; the no-allocation entry point has " +
              std::to_string(noalloc::kScratchBytes - noalloc::kWorkspaceOffset));
    return ATRIP_ERR_UNSUPPORTED;
  }
  int device = 0;
  ATRIP_CUDA_TRY(cudaGetDevice(&device));
  int status = ATRIP_OK;
  unsigned char *scratch = noalloc::scratch_address(&status);
  if (!scratch) return status;
  const int64_t n_all = atrip_gpu_n_tuples(nv);
  int64_t t_end = n_all;
  if (max_iterations != 0 && max_iterations + 1 < t_end) t_end = max_iterations + 1;
  const int64_t t_begin = first_iteration < t_end ? first_iteration : t_end;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  noalloc::Args a;
  a.No = no;
  a.Nv = nv;
  a.epsi = in->epsi;
  a.epsa = in->epsa;
  a.tai = in->tai;
  a.T = in->tabij;
  a.Vpp = in->vabij;
  a.Vh = in->vijka;
  a.Vp = in->vabci;
  a.Jh = in->jijka;
  a.Jp = in->jabci;
  a.t_begin = t_begin;
  a.t_end = t_end;
  a.tai_sign = ijkabc ? -1.0 : 1.0;
  a.use_j = (use_j && in->jijka && in->jabci) ? 1 : 0;
  a.ijkabc = ijkabc ? 1 : 0;
  a.e = tuple_e;
  a.ect = tuple_ect;
  a.energies = energies;
  a.scratch = scratch;
  // the cursor must start at zero; the partials are overwritten by every call
  ATRIP_CUDA_TRY(cudaMemsetAsync(scratch, 0, noalloc::kHeaderBytes, st));
  const int64_t n = t_end - t_begin;
  if (n > 0) {
    int rc = ATRIP_OK;
    switch ((no + 7) / 8) {
      case 1: rc = noalloc::launch<1>(a, device, st); break;
      case 2: rc = noalloc::launch<2>(a, device, st); break;
      case 3: rc = noalloc::launch<3>(a, device, st); break;
      case 4: rc = noalloc::launch<4>(a, device, st); break;
      case 5: rc = noalloc::launch<5>(a, device, st); break;
      case 6: rc = noalloc::launch<6>(a, device, st); break;
      case 7: rc = noalloc::launch<7>(a, device, st); break;
      default: rc = noalloc::launch<8>(a, device, st); break;
    }
    if (rc != ATRIP_OK) return rc;
  }
  ATRIP_CUDA_TRY(cudaMemsetAsync(scratch + noalloc::kHeaderBytes, 0, noalloc::kPartialBytes, st));
  noalloc::noalloc_sum_stage1<<<n > 0 ? noalloc::kPartialBlocks : 1, noalloc::kThreads, 0, st>>>(a, n);
  ATRIP_CUDA_TRY(cudaGetLastError());
  noalloc::noalloc_sum_stage2<<<1, 32, 0, st>>>(a);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}
