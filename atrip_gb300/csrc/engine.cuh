// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "atrip_gb300.h"

namespace atrip_gb300 {

// Thread-local last-error text behind atrip_gpu_last_error().
void set_error(const std::string &msg);
void clear_error();

#define ATRIP_CUDA_TRY(call)                                                      \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      ::atrip_gb300::set_error(std::string(#call) + ": " + cudaGetErrorString(_e) + \
                               " (" + __FILE__ + ":" + std::to_string(__LINE__) + ")"); \
      return _e == cudaErrorMemoryAllocation ? ATRIP_ERR_OUT_OF_MEMORY : ATRIP_ERR_CUDA; \
    }                                                                             \
  } while (0)

// Kernel-friendly HBM layouts of the inputs (element counts in comments).
//   Ta [x][q][p][E]  = Tabij[x,E,p,q]   rows (p,q) of T_x, E contiguous  Nv*No*No*Nv
//   Tp [x][y][n][m]  = Tabij[x,y,m,n]   No x No pair blocks              Nv*Nv*No*No
//   Vhh[x][y][n][m]  = Vabij[x,y,m,n]   pair blocks for the singles      Nv*Nv*No*No
//   Vht[w][q][p][L]  = Vijka[p,q,L,w]   rows (p,q) of Vh_w, L contiguous Nv*No*No*No
//   Vpt[y][z][r][E]  = Vabci[y,z,E,r]   columns r of V_yz, E contiguous  Nv*Nv*No*Nv
//   Jht, Jpt         same as Vht, Vpt for the (cT) intermediates
struct DeviceTensors {
  double *epsi = nullptr, *epsa = nullptr, *tai = nullptr;
  double *Ta = nullptr, *Tp = nullptr, *Vhh = nullptr;
  double *Vht = nullptr, *Vpt = nullptr, *Jht = nullptr, *Jpt = nullptr;
};

// Arguments of one FP64 triples launch.
struct TriplesArgs {
  int No, Nv;
  const double *epsi, *epsa, *tai;
  const double *Ta, *Tp, *Vhh, *Vht, *Vpt, *Jht, *Jpt;
  const uint32_t *tuples;   // packed a | b << 10 | c << 20, list order
  const uint32_t *triples;  // packed i | j << 8 | k << 16 with i >= j >= k
  int n_triples;
  int64_t t_begin, t_end;   // tuple-list range of this launch
  const uint32_t *order;    // processing order: queue slot q runs list position
                            // t_begin + order[q] (nullptr: t_begin + q)
  unsigned long long *queue;// work-queue cursor (zeroed before launch)
  double tai_sign;          // -1 for ijkabc (src/atrip/Atrip.cxx:183-187)
  int use_j;
  double *e, *ect;          // per-tuple energies, indexed by list position
  double *workspace;        // per-CTA scratch, 2 * No^3 doubles each
  int rows_tile;            // (p,q) rows per register tile: 32 or 64
  int claim;                // tuples a CTA takes from the queue at once (>= 1)
  int min_blocks;           // 2: kernel variant capped at 128 registers, else 0
};

cudaError_t launch_triples_fp64(const TriplesArgs &a, int grid, cudaStream_t s);

// Several systems in one persistent launch (systems[] and prefix[] in device
// memory; prefix[n] = total tuples; workspace ws_stride doubles per CTA).
struct BatchArgs {
  const TriplesArgs *systems;
  const int64_t *prefix;
  int n;
  unsigned long long *queue;
  double *workspace;
  int64_t ws_stride;
  int claim;  // tuples a CTA takes from the queue at once (>= 1)
};
// Batch systems have No <= kBatchMaxNo.
constexpr int kBatchMaxNo = 32;
cudaError_t launch_triples_fp64_batch(const BatchArgs &b, int max_no, int min_blocks, int grid,
                                      cudaStream_t s);
cudaError_t launch_batch_energy_sum(const BatchArgs &b, double *sums, cudaStream_t s);
int triples_fp64_max_blocks_per_sm(int No, int rows_tile, int min_blocks);
int triples_fp64_batch_max_blocks_per_sm(int max_no, int min_blocks);

// dst[i0 + n0 (i1 + n1 (i2 + n2 i3))] = src[i0 s0 + i1 s1 + i2 s2 + i3 s3],
// elements of one double, or of two (re, im) when complex_elems
cudaError_t launch_permute4(double *dst, const double *src, const int64_t n[4],
                            const int64_t s[4], cudaStream_t st, bool complex_elems);
// General box: dst[i . t] = src[i . s] over the n0 x n1 x n2 x n3 box.
cudaError_t launch_permute4_box(double *dst, const double *src, const int64_t n[4],
                                const int64_t s[4], const int64_t t[4], cudaStream_t st,
                                bool complex_elems);

// Complex field: the same launch arguments, every tensor pointer holding
// interleaved (re, im) pairs, workspace 4 No^3 doubles per CTA.
cudaError_t launch_triples_z(const TriplesArgs &a, int grid, cudaStream_t s);
int triples_z_max_blocks_per_sm(int No);

// Compensated two-stage sum of x[0..n) and y[0..n) into out[0], out[1].
cudaError_t launch_energy_sum(const double *x, const double *y, int64_t n, double *partials,
                              double *out, cudaStream_t st);
constexpr int kSumBlocks = 256;

}  // namespace atrip_gb300
