// Complex field (atrip's run<Complex>, src/atrip/Atrip.cxx:1136): the
// plain-FP64 triples kernel on interleaved (re, im) operands.
//
// Same persistent work-queue structure and fused terms as the real kernel
// (fp64_tuple.cuh), with the Complex semantics of the reference's default
// (DGEMM) route:
//   * hole terms use conj(V_hhhp) (MAYBE_CONJ before the hole GEMMs,
//     src/atrip/Equations.cxx:599-632, Operations.hpp:28-44); particle terms
//     and the singles use the operands as they are;
//   * the energy pairs conj(Tijk) with Zijk (get_energy_{distinct,same},
//     src/atrip/Equations.cxx:101-238), divides by the complex denominator
//     epsabc - (eps_i + eps_j + eps_k) with epsabc the real part of the
//     eps_a sum (src/atrip/Atrip.cxx:643-646), and keeps the real part of the
//     tuple's sum, i.e. the sum of the terms' real parts.
// Complex quotients use Smith's algorithm (R. L. Smith, CACM 5(8), 1962).
#include "engine.cuh"

namespace atrip_gb300 {
namespace {

constexpr int kThreads = 256;
constexpr int kMT = 64;  // rows (p,q) per tile: 32 row groups x 2
constexpr int kKC = 16;  // complex K elements per shared-memory stage

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 cscale(double s, double2 a) {
  return make_double2(s * a.x, s * a.y);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// Real part of a / d (Smith's algorithm).
__device__ __forceinline__ double cdiv_re(double2 a, double2 d) {
  if (fabs(d.y) <= fabs(d.x)) {
    const double r = d.y / d.x, den = d.x + d.y * r;
    return (a.x + a.y * r) / den;
  }
  const double r = d.x / d.y, den = d.x * r + d.y;
  return (a.x * r + a.y) / den;
}

struct ZArgs {
  int No, Nv;
  const double2 *epsi, *epsa, *tai;
  const double2 *Ta, *Tp, *Vhh, *Vht, *Vpt, *Jht, *Jpt;
  const uint32_t *tuples, *triples;
  int n_triples;
  int64_t t_begin, t_end;
  const uint32_t *order;
  unsigned long long *queue;
  double tai_sign;
  int use_j;
  double *e, *ect;
  double2 *workspace;  // 2 No^3 per CTA
};

struct ZTerm {
  const double2 *Apart, *Ahole, *Bpart, *Bhole;
  int holeT, sp, sq, sr;
};

// The six fused terms (same table as the real kernel).
__device__ __forceinline__ ZTerm make_zterm(int t, const ZArgs &g, const double2 *Vht,
                                            const double2 *Vpt, int a, int b, int c) {
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
  ZTerm r;
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

struct ZSmem {
  double2 As[kKC][kMT + 1];
  double2 Bs[kKC][64 + 1];
  double red[kThreads / 32];
  long long tuple_slot;
};

struct ZSingles {
  const double2 *Vbc, *Vac, *Vab;
  double2 ta[64], tb[64], tc[64];
};

template <int NC>
__device__ void build_w_z(const ZArgs &g, ZSmem &sm, double2 *W, const double2 *Vht,
                          const double2 *Vpt, int a, int b, int c) {
  const int No = g.No, Nv = g.Nv, No2 = No * No;
  const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
  for (int t = 0; t < 6; ++t) {
    const ZTerm tm = make_zterm(t, g, Vht, Vpt, a, b, c);
    for (int m0 = 0; m0 < No2; m0 += kMT) {
      double2 acc[2][NC];
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < NC; ++v) acc[u][v] = make_double2(0.0, 0.0);
      for (int seg = 0; seg < 2; ++seg) {
        const int K = seg == 0 ? Nv : No;
        const double2 *A = seg == 0 ? tm.Apart : tm.Ahole;
        for (int k0 = 0; k0 < K; k0 += kKC) {
          for (int idx = tid; idx < kMT * kKC; idx += kThreads) {
            const int row = idx / kKC, kk = idx % kKC, m = m0 + row, k = k0 + kk;
            double2 val = make_double2(0.0, 0.0);
            if (m < No2 && k < K) {
              val = A[(int64_t)m * K + k];
              if (seg == 1) val = cconj(val);  // conj(V_hhhp) in the hole terms
            }
            sm.As[kk][row] = val;
          }
          for (int idx = tid; idx < NC * 8 * kKC; idx += kThreads) {
            const int col = idx / kKC, kk = idx % kKC, k = k0 + kk;
            double2 val = make_double2(0.0, 0.0);
            if (col < No && k < K) {
              if (seg == 0) {
                val = tm.Bpart[(int64_t)col * Nv + k];
              } else {
                const double2 h = tm.holeT ? tm.Bhole[k * No + col] : tm.Bhole[col * No + k];
                val = make_double2(-h.x, -h.y);
              }
            }
            sm.Bs[kk][col] = val;
          }
          __syncthreads();
#pragma unroll 4
          for (int kk = 0; kk < kKC; ++kk) {
            const double2 a0 = sm.As[kk][ty], a1 = sm.As[kk][ty + 32];
#pragma unroll
            for (int v = 0; v < NC; ++v) {
              const double2 bv = sm.Bs[kk][tx + 8 * v];
              acc[0][v] = cfma(a0, bv, acc[0][v]);
              acc[1][v] = cfma(a1, bv, acc[1][v]);
            }
          }
          __syncthreads();
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int m = m0 + ty + 32 * u;
        if (m < No2) {
          const int p = m % No, q = m / No;
#pragma unroll
          for (int v = 0; v < NC; ++v) {
            const int r = tx + 8 * v;
            if (r < No) {
              const int idx = p * tm.sp + q * tm.sq + r * tm.sr;
              W[idx] = t == 0 ? acc[u][v] : cadd(W[idx], acc[u][v]);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

// Zijk = W + t1 (x) V (src/atrip/Equations.cxx:420-422).
__device__ __forceinline__ double2 zval_z(const double2 *W, const ZSingles &s, int No, int i,
                                          int j, int k) {
  double2 z = W[i + No * j + No * No * k];
  z = cadd(z, cmul(s.ta[i], s.Vbc[j + k * No]));
  z = cadd(z, cmul(s.tb[j], s.Vac[i + k * No]));
  z = cadd(z, cmul(s.tc[k], s.Vab[i + j * No]));
  return z;
}

__device__ double energy_partial_z(const ZArgs &g, const double2 *Tb, const double2 *Wz,
                                   const ZSingles &s, bool distinct, double epsabc) {
  const int No = g.No;
  double sum = 0.0;
  for (int n = threadIdx.x; n < g.n_triples; n += kThreads) {
    const uint32_t pk = g.triples[n];
    const int i = pk & 0xff, j = (pk >> 8) & 0xff, k = (pk >> 16) & 0xff;
    const double fac = (j == k ? 0.5 : 1.0) * (i == j ? 0.5 : 1.0);
    const double2 eijk = cadd(cadd(g.epsi[i], g.epsi[j]), g.epsi[k]);
    const double2 den = make_double2(epsabc - eijk.x, -eijk.y);
#define TB(p, q, r) cconj(Tb[(p) + No * (q) + No * No * (r)])
    double2 value;
    if (distinct) {
      const double2 U = zval_z(Wz, s, No, i, j, k), V = zval_z(Wz, s, No, i, k, j),
                    W = zval_z(Wz, s, No, j, i, k), X = zval_z(Wz, s, No, j, k, i),
                    Y = zval_z(Wz, s, No, k, i, j), Z = zval_z(Wz, s, No, k, j, i);
      const double2 A = TB(i, j, k), B = TB(i, k, j), C = TB(j, i, k), D = TB(j, k, i),
                    E = TB(k, i, j), F = TB(k, j, i);
      const double2 UXY = cadd(U, cadd(X, Y)), VWZ = cadd(V, cadd(W, Z)),
                    ADE = cadd(A, cadd(D, E)), BCF = cadd(B, cadd(C, F));
      const double2 first =
          cadd(cmul(A, U),
               cadd(cmul(B, V), cadd(cmul(C, W), cadd(cmul(D, X), cadd(cmul(E, Y), cmul(F, Z))))));
      const double2 second = cmul(csub(UXY, cscale(2.0, VWZ)), ADE);
      const double2 third = cmul(csub(VWZ, cscale(2.0, UXY)), BCF);
      value = cadd(cscale(3.0, first), cadd(second, third));
    } else {
      const double2 U = zval_z(Wz, s, No, i, j, k), V = zval_z(Wz, s, No, j, k, i),
                    W = zval_z(Wz, s, No, k, i, j);
      const double2 A = TB(i, j, k), B = TB(j, k, i), C = TB(k, i, j);
      value = csub(cscale(3.0, cadd(cadd(cmul(A, U), cmul(B, V)), cmul(C, W))),
                   cmul(cadd(A, cadd(B, C)), cadd(U, cadd(V, W))));
    }
#undef TB
    sum += cdiv_re(cscale(2.0, value), den) * fac;
  }
  return sum;
}

__device__ double block_sum_z(double v, ZSmem &sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) r += sm.red[w];
  __syncthreads();
  return r;  // valid in thread 0
}

template <int NC>
__global__ void __launch_bounds__(kThreads) triples_z_kernel(ZArgs g) {
  __shared__ ZSmem sm;
  __shared__ ZSingles s;
  const int No = g.No, Nv = g.Nv, No2 = No * No;
  const int64_t No3 = (int64_t)No2 * No;
  double2 *Wv = g.workspace + (int64_t)blockIdx.x * 2 * No3;
  double2 *Wj = Wv + No3;
  const int64_t n = g.t_end - g.t_begin;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long q = atomicAdd(g.queue, 1ull);
      sm.tuple_slot = (q < (unsigned long long)n) ? (long long)q : -1;
    }
    __syncthreads();
    const long long slot = sm.tuple_slot;
    __syncthreads();
    if (slot < 0) break;
    const int64_t t = g.t_begin + (g.order ? (int64_t)g.order[slot] : (int64_t)slot);
    const uint32_t pk = g.tuples[t];
    const int a = pk & 0x3ff, b = (pk >> 10) & 0x3ff, c = (pk >> 20) & 0x3ff;
    if (threadIdx.x < No) {
      const int i = threadIdx.x;
      s.ta[i] = cscale(g.tai_sign, g.tai[a + i * Nv]);
      s.tb[i] = cscale(g.tai_sign, g.tai[b + i * Nv]);
      s.tc[i] = cscale(g.tai_sign, g.tai[c + i * Nv]);
    }
    if (threadIdx.x == 0) {
      s.Vbc = g.Vhh + ((int64_t)b * Nv + c) * No2;
      s.Vac = g.Vhh + ((int64_t)a * Nv + c) * No2;
      s.Vab = g.Vhh + ((int64_t)a * Nv + b) * No2;
    }
    build_w_z<NC>(g, sm, Wv, g.Vht, g.Vpt, a, b, c);
    int cls = 0;  // src/atrip/Atrip.cxx:640-642
    if (a == b) cls++;
    if (b == c) cls--;
    const double epsabc = g.epsa[a].x + g.epsa[b].x + g.epsa[c].x;
    const double e = block_sum_z(energy_partial_z(g, Wv, Wv, s, cls == 0, epsabc), sm);
    double ect = e;
    if (g.use_j) {
      build_w_z<NC>(g, sm, Wj, g.Jht, g.Jpt, a, b, c);
      ect = block_sum_z(energy_partial_z(g, Wj, Wv, s, cls == 0, epsabc), sm);
    }
    if (threadIdx.x == 0) {
      g.e[t] = e;
      g.ect[t] = ect;
    }
    __syncthreads();
  }
}

template <int NC>
cudaError_t launch_z_nc(const ZArgs &a, int grid, cudaStream_t s) {
  triples_z_kernel<NC><<<grid, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_triples_z(const TriplesArgs &ta, int grid, cudaStream_t s) {
  ZArgs a;
  a.No = ta.No;
  a.Nv = ta.Nv;
  a.epsi = reinterpret_cast<const double2 *>(ta.epsi);
  a.epsa = reinterpret_cast<const double2 *>(ta.epsa);
  a.tai = reinterpret_cast<const double2 *>(ta.tai);
  a.Ta = reinterpret_cast<const double2 *>(ta.Ta);
  a.Tp = reinterpret_cast<const double2 *>(ta.Tp);
  a.Vhh = reinterpret_cast<const double2 *>(ta.Vhh);
  a.Vht = reinterpret_cast<const double2 *>(ta.Vht);
  a.Vpt = reinterpret_cast<const double2 *>(ta.Vpt);
  a.Jht = reinterpret_cast<const double2 *>(ta.Jht);
  a.Jpt = reinterpret_cast<const double2 *>(ta.Jpt);
  a.tuples = ta.tuples;
  a.triples = ta.triples;
  a.n_triples = ta.n_triples;
  a.t_begin = ta.t_begin;
  a.t_end = ta.t_end;
  a.order = ta.order;
  a.queue = ta.queue;
  a.tai_sign = ta.tai_sign;
  a.use_j = ta.use_j;
  a.e = ta.e;
  a.ect = ta.ect;
  a.workspace = reinterpret_cast<double2 *>(ta.workspace);
  switch ((a.No + 7) / 8) {
    case 1: return launch_z_nc<1>(a, grid, s);
    case 2: return launch_z_nc<2>(a, grid, s);
    case 3: return launch_z_nc<3>(a, grid, s);
    case 4: return launch_z_nc<4>(a, grid, s);
    case 5: return launch_z_nc<5>(a, grid, s);
    case 6: return launch_z_nc<6>(a, grid, s);
    case 7: return launch_z_nc<7>(a, grid, s);
    case 8: return launch_z_nc<8>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

int triples_z_max_blocks_per_sm(int No) {
  int n = 0;
  cudaError_t e = cudaErrorInvalidValue;
  switch ((No + 7) / 8) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<1>, kThreads, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<2>, kThreads, 0); break;
    case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<3>, kThreads, 0); break;
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<4>, kThreads, 0); break;
    case 5: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<5>, kThreads, 0); break;
    case 6: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<6>, kThreads, 0); break;
    case 7: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<7>, kThreads, 0); break;
    case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, triples_z_kernel<8>, kThreads, 0); break;
    default: break;
  }
  return e == cudaSuccess ? n : 0;
}

}  // namespace atrip_gb300
