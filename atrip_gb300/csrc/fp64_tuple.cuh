// Plain-FP64 form of the per-(a,b,c) triples kernel: the per-tuple device
// code shared by the single-system and the batch kernels.
//
// One persistent CTA per slot pulls tuples from a device work queue (an
// atomic cursor over the lexicographic tuple list, src/atrip/Tuples.cxx:
// 122-134) and, per tuple:
//   1. builds W = Tijk from six fused contractions.  Each pairs one particle
//      term of src/atrip/Equations.cxx:709-725 with the hole term that has
//      the same output layout (:692-708), so one tile loop runs K = Nv + No:
//        R[(p,q), r] = sum_E A_x[(p,q),E] V_yz[E,r] - sum_L Vh_w[(p,q),L] T_uv[L,r]
//      and R is added into W at the index permutation of that term (the
//      reorder<> kernels of src/atrip/Equations.cxx:27-83, fused);
//   2. forms Zijk = W + singles on the fly (src/atrip/Equations.cxx:387-426);
//   3. reduces get_energy_{distinct,same} (src/atrip/Equations.cxx:101-238)
//      over i >= j >= k with a block reduction;
//   4. for (cT) builds W from the J intermediates and reduces again with the
//      same Z (src/atrip/Atrip.cxx:928-963).
// FP64 throughput on this part is ~1 TFLOP/s for DFMA and DMMA alike, so the
// contraction is a register-tiled DFMA GEMM; the tiles are staged through
// shared memory with coalesced loads.
#pragma once

#include "engine.cuh"

namespace atrip_gb300 {
namespace {

constexpr int kThreads = 256;
constexpr int kMT = 64;  // largest row tile: 32 row groups x RU rows, RU <= 2
constexpr int kKC = 32;  // K elements per shared-memory stage

struct Term {
  const double *Apart;  // Ta_x   rows m, K = Nv
  const double *Ahole;  // Vht_w  rows m, K = No
  const double *Bpart;  // Vpt_yz cols r, K = Nv
  const double *Bhole;  // Tp_uv  No x No block
  int holeT;            // 0: B[L][r] = T[u,v,L,r]; 1: B[L][r] = T[u,v,r,L]
  int sp, sq, sr;       // W index = p sp + q sq + r sr
};

// The six fused terms of tuple (a,b,c); index roles a<->i, b<->j, c<->k.
__device__ __forceinline__ Term make_term(int t, const TriplesArgs &g, const double *Vht,
                                          const double *Vpt, int a, int b, int c) {
  const int64_t No = g.No, Nv = g.Nv, No2 = No * No, No3 = No2 * No;
  int x, w, y, z, u, v, holeT, sp, sq, sr;
  switch (t) {
    case 0: x = a; w = b; y = b; z = c; u = a; v = c; holeT = 0; sp = 1; sq = No; sr = No2; break;
    case 1: x = a; w = c; y = c; z = b; u = a; v = b; holeT = 0; sp = 1; sq = No2; sr = No; break;
    case 2: x = c; w = a; y = a; z = b; u = b; v = c; holeT = 1; sp = No2; sq = 1; sr = No; break;
    case 3: x = c; w = b; y = b; z = a; u = a; v = c; holeT = 1; sp = No2; sq = No; sr = 1; break;
    case 4: x = b; w = a; y = a; z = c; u = b; v = c; holeT = 0; sp = No; sq = 1; sr = No2; break;
    default: x = b; w = c; y = c; z = a; u = a; v = b; holeT = 1; sp = No; sq = No2; sr = 1; break;
  }
  Term r;
  r.Apart = g.Ta + (int64_t)x * No2 * Nv;
  r.Ahole = Vht + (int64_t)w * No3;
  r.Bpart = Vpt + ((int64_t)y * Nv + z) * No * Nv;
  r.Bhole = g.Tp + ((int64_t)u * Nv + v) * No2;
  r.holeT = holeT;
  r.sp = sp;
  r.sq = sq;
  r.sr = sr;
  return r;
}

struct Smem {
  double As[kKC][kMT + 1];
  double Bs[kKC][64 + 1];
  double red[kThreads / 32][2];
  long long tuple_slot;
};

// W (No^3, in the per-CTA workspace) = sum of the six fused terms.  Tile:
// 32 RU rows (p,q) x 8 NC columns r; thread (ty, tx) owns rows ty + 32 u
// (u < RU) and columns tx + 8 v.
template <int NC, int RU>
__device__ void build_w(const TriplesArgs &g, Smem &sm, double *W, const double *Vht,
                        const double *Vpt, int a, int b, int c) {
  constexpr int MT = 32 * RU;
  const int No = g.No, Nv = g.Nv, No2 = No * No;
  const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
  for (int t = 0; t < 6; ++t) {
    const Term tm = make_term(t, g, Vht, Vpt, a, b, c);
    for (int m0 = 0; m0 < No2; m0 += MT) {
      double acc[RU][NC];
#pragma unroll
      for (int u = 0; u < RU; ++u)
#pragma unroll
        for (int v = 0; v < NC; ++v) acc[u][v] = 0.0;
      for (int seg = 0; seg < 2; ++seg) {
        const int K = seg == 0 ? Nv : No;
        const double *A = seg == 0 ? tm.Apart : tm.Ahole;
        for (int k0 = 0; k0 < K; k0 += kKC) {
          for (int idx = tid; idx < MT * kKC; idx += kThreads) {
            const int row = idx / kKC, kk = idx % kKC, m = m0 + row, k = k0 + kk;
            sm.As[kk][row] = (m < No2 && k < K) ? A[(int64_t)m * K + k] : 0.0;
          }
          for (int idx = tid; idx < NC * 8 * kKC; idx += kThreads) {
            const int col = idx / kKC, kk = idx % kKC, k = k0 + kk;
            double val = 0.0;
            if (col < No && k < K) {
              if (seg == 0)
                val = tm.Bpart[(int64_t)col * Nv + k];
              else
                val = -(tm.holeT ? tm.Bhole[k * No + col] : tm.Bhole[col * No + k]);
            }
            sm.Bs[kk][col] = val;
          }
          __syncthreads();
#pragma unroll 8
          for (int kk = 0; kk < kKC; ++kk) {
            double av[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u) av[u] = sm.As[kk][ty + 32 * u];
#pragma unroll
            for (int v = 0; v < NC; ++v) {
              const double bv = sm.Bs[kk][tx + 8 * v];
#pragma unroll
              for (int u = 0; u < RU; ++u) acc[u][v] = fma(av[u], bv, acc[u][v]);
            }
          }
          __syncthreads();
        }
      }
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const int m = m0 + ty + 32 * u;
        if (m < No2) {
          const int p = m % No, q = m / No;
#pragma unroll
          for (int v = 0; v < NC; ++v) {
            const int r = tx + 8 * v;
            if (r < No) {
              const int idx = p * tm.sp + q * tm.sq + r * tm.sr;
              W[idx] = (t == 0 ? 0.0 : W[idx]) + acc[u][v];
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

struct SinglesCtx {
  const double *Vbc, *Vac, *Vab;  // No x No blocks V[x,y,m,n] at [n*No + m]
  double ta[64], tb[64], tc[64];  // signed t1[a,.], t1[b,.], t1[c,.]
};

// Zijk at (i,j,k) = W + t1 (x) V, in the order of src/atrip/Equations.cxx:420-422.
__device__ __forceinline__ double zval(const double *W, const SinglesCtx &s, int No, int i, int j,
                                       int k) {
  double z = W[i + No * j + No * No * k];
  z += s.ta[i] * s.Vbc[j + k * No];
  z += s.tb[j] * s.Vac[i + k * No];
  z += s.tc[k] * s.Vab[i + j * No];
  return z;
}

// One tuple's energy over i >= j >= k (src/atrip/Equations.cxx:101-238):
// T from Tb, Z from Wz + singles.  Returns this thread's partial sum.
__device__ double energy_partial(const TriplesArgs &g, const double *Tb, const double *Wz,
                                 const SinglesCtx &s, bool distinct, double epsabc) {
  const int No = g.No;
  double sum = 0.0;
  for (int n = threadIdx.x; n < g.n_triples; n += kThreads) {
    const uint32_t pk = g.triples[n];
    const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff;
    const double facjk = j == k ? 0.5 : 1.0, facij = i == j ? 0.5 : 1.0;
    const double denominator = epsabc - ((g.epsi[i] + g.epsi[j]) + g.epsi[k]);
    double value;
    if (distinct) {
      const double U = zval(Wz, s, No, i, j, k), V = zval(Wz, s, No, i, k, j),
                   W = zval(Wz, s, No, j, i, k), X = zval(Wz, s, No, j, k, i),
                   Y = zval(Wz, s, No, k, i, j), Z = zval(Wz, s, No, k, j, i);
      const double A = Tb[i + No * j + No * No * k], B = Tb[i + No * k + No * No * j],
                   C = Tb[j + No * i + No * No * k], D = Tb[j + No * k + No * No * i],
                   E = Tb[k + No * i + No * No * j], F = Tb[k + No * j + No * No * i];
      const double UXY = U + (X + Y), VWZ = V + (W + Z), ADE = A + (D + E), BCF = B + (C + F);
      const double first = A * U + (B * V + (C * W + (D * X + (E * Y + F * Z))));
      value = 3.0 * first + ((UXY - 2.0 * VWZ) * ADE + (VWZ - 2.0 * UXY) * BCF);
    } else {
      const double U = zval(Wz, s, No, i, j, k), V = zval(Wz, s, No, j, k, i),
                   W = zval(Wz, s, No, k, i, j);
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
  return r;  // valid in thread 0
}

// One tuple t of the system described by g: W (and W_J), energies e[t],
// ect[t].  All threads of the block take part.
template <int NC, int RU>
__device__ void process_tuple(const TriplesArgs &g, Smem &sm, SinglesCtx &s, double *Wv,
                              double *Wj, int64_t t) {
  const uint32_t pk = g.tuples[t];
  const int a = pk & 0x3ff, b = (pk >> 10) & 0x3ff, c = (pk >> 20) & 0x3ff;
  const int No = g.No, Nv = g.Nv, No2 = No * No;
  if (threadIdx.x < No) {
    const int i = threadIdx.x;
    s.ta[i] = g.tai_sign * g.tai[a + i * Nv];
    s.tb[i] = g.tai_sign * g.tai[b + i * Nv];
    s.tc[i] = g.tai_sign * g.tai[c + i * Nv];
  }
  if (threadIdx.x == 0) {
    s.Vbc = g.Vhh + ((int64_t)b * Nv + c) * No2;
    s.Vac = g.Vhh + ((int64_t)a * Nv + c) * No2;
    s.Vab = g.Vhh + ((int64_t)a * Nv + b) * No2;
  }
  build_w<NC, RU>(g, sm, Wv, g.Vht, g.Vpt, a, b, c);
  // classification of src/atrip/Atrip.cxx:640-642
  int cls = 0;
  if (a == b) cls++;
  if (b == c) cls--;
  const bool distinct = cls == 0;
  const double epsabc = g.epsa[a] + g.epsa[b] + g.epsa[c];
  const double e = block_sum(energy_partial(g, Wv, Wv, s, distinct, epsabc), sm, 0);
  double ect = e;
  if (g.use_j) {
    build_w<NC, RU>(g, sm, Wj, g.Jht, g.Jpt, a, b, c);
    ect = block_sum(energy_partial(g, Wj, Wv, s, distinct, epsabc), sm, 1);
  }
  if (threadIdx.x == 0) {
    g.e[t] = e;
    g.ect[t] = ect;
  }
  __syncthreads();
}

}  // namespace
}  // namespace atrip_gb300
