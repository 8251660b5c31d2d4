// Split-precision form of the triples kernel: FP64 operands cut into BF16
// "digit" slices, contractions on the tcgen05 tensor cores with FP32
// accumulation in TMEM, exact integer / FP64 recombination.
//
// Splitting (done once per upload, in FP64).  With one power-of-two scale per
// tensor (2^eT for T, 2^eV shared by V_pphp and V_hhhp so that particle and
// hole products land on the same grid), an element x is written as
//     x = 2^(e-7) * sum_p q_p 2^(-8p),   q_p integer, |q_p| <= 128,
// q_p = rint of the running remainder.  Each q_p is exact in BF16, every
// product q_p q'_q is an integer below 2^14, and a dot product of up to 1024
// such terms is an integer below 2^24, hence exact in the FP32 accumulator.
// Products are grouped by level L = p + q (pairs with L < S are kept; S =
// slices); level 0 is exact, levels >= 1 carry a 2^-8L smaller weight.
//
// Contraction structure.  The six fused particle+hole terms of the FP64
// form (src/atrip/Equations.cxx:455-728) pair up by output column index:
// term t and its partner share the column index and run over the same pair
// of row indices in opposite order.  Loading the partner's A rows from a
// transposed copy makes both land in the same TMEM rows, so each pair is one
// K-concatenated GEMM (K = 2 (Nv + No)) into one accumulator:
//   G0  rows (i,j), column k:  T_a/Vh_b (natural)  + T_b/Vh_a (transposed)
//   G1  rows (i,k), column j:  T_a/Vh_c            + T_c/Vh_a
//   G2  rows (j,k), column i:  T_b/Vh_c            + T_c/Vh_b
// and W[i,j,k] = G0 + G1 + G2, accumulated per element as an exact int32
// (level 0) plus an FP32 remainder (levels >= 1) in shared memory.  The
// energy loop converts W = unit * (int + rem) to FP64 and evaluates Zijk and
// get_energy_{distinct,same} (src/atrip/Equations.cxx:101-238, 387-426) in
// FP64.
//
// Kernel roles (512 threads, one persistent CTA per SM):
//   warp 0          TMA producer: owns the tuple queue, loads the operand
//                   tiles of every unit into the shared-memory ring
//   warp 1          TMEM owner and single-thread tcgen05.mma issuer
//   warps 4..7      epilogue: tcgen05.ld of the accumulators, level
//                   recombination, stores of the group's W cells
//   warps 2, 3, 8..15  energy: W in FP64, Zijk, get_energy_{distinct,same}
//                   and the block reduction, one tuple behind the MMAs
// Smem ring of operand stages (full/empty mbarriers), two TMEM accumulator
// buffers (full/empty mbarriers), a 4-slot tuple hand-off ring and two W
// buffer sets; every wait is bounded (sm100.cuh).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstring>
#include <string>
#include <type_traits>

#include "engine.cuh"
#include "sm100.cuh"
#include "split.cuh"

namespace atrip_gb300 {
namespace {

using namespace sm100;

constexpr int kThreads = 512;
constexpr int kMaxStages = 6;
constexpr int kSmemLimit = 232448;  // opt-in dynamic shared memory per block
constexpr int kTailBytes = 384 + 3 * 64 * 8 + 16 * 8 + 64 * 8;  // + W copy, staging
constexpr int kKChunk = 64;              // BF16 elements per 128-byte row
constexpr int kATileBytes = 128 * 128;   // 128 rows x 128 B
constexpr int kHoleK = 64;               // hole K (L) padded to one chunk

enum : int {
  kErrTimeoutFull = 1,
  kErrTimeoutEmpty = 2,
  kErrTimeoutAccFull = 3,
  kErrTimeoutAccEmpty = 4
};

struct SplitMaps {
  CUtensorMap TaN, TaT, VhN, VhT, Vp, TpN, TpT;
  CUtensorMap JhN, JhT, Jp;  // (cT) intermediates in place of V_hhhp, V_pphp
  // transposed variant: boxes of jt2 (p,q) row groups for the N side, all S
  // slices stacked for the M side
  CUtensorMap TaN2, TaT2, VhN2, VhT2, Vp2, TpN2, TpT2, JhN2, JhT2, Jp2;
  // ... and the r-column operand with 2S-1 slices, one load per K chunk
  // shared by the S slice units (MSHARE)
  CUtensorMap Vp3, TpN3, TpT3, Jp3;
};

struct SysDesc;

struct SplitArgs {
  int No, Nv, jt, ntiles, kch;  // j per M-tile, M-tiles per group, K chunks of Nv
  int jt2, ntiles2, nmma;       // transposed variant: q per N-tile, N-tiles, MMA N
  int prefetch;                 // 1: L2 prefetch of the next part's (p,q)-row tiles
  int unpublished;              // test: the producer publishes no tuple (waits run out)
  long long wait_cycles;        // limit of every bounded wait, SM cycles
  // several systems in one launch: per-system descriptors, prefix sums of
  // their tuple counts (the work queue runs over the concatenation)
  const SysDesc *sys;
  const int64_t *prefix;
  int nsys;
  int no_lay, npass_lay;  // shared memory / W buffer layout: the largest system
  int mslot_bytes;              // MSHARE: bytes of one shared M-tile slot
  int nstages;                 // operand ring depth
  int stage_bytes;             // bytes of one ring stage
  int b_off;                   // offset of the N-side tile within a stage
  const double *epsi, *epsa, *tai, *Vhh;
  const uint32_t *tuples, *triples;
  const double2 *tri_ef;  // per (i,j,k) triple: (e_i + e_j) + e_k, 2 fac_jk fac_ij
  int n_triples;
  int64_t t_begin, t_end;
  const uint32_t *order;  // queue slot q runs list position t_begin + order[q]
  unsigned long long *queue;
  double tai_sign, unit, unit_j;
  int use_j;  // second pass with the J intermediates ((cT) energy)
  double *e, *ect;
  int *status;
  float *wglobal;  // two W buffers per CTA (one 8-byte cell per element)
  unsigned long long *prof;  // role profile counters (profiled launches only)
  int vsm;  // 1: the singles' V_hhpp blocks are copied to shared memory per tuple
};

// ------------------------------------------------------------------ prep

__global__ void absmax_kernel(const double *__restrict__ x, int64_t n,
                              unsigned long long *__restrict__ out) {
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(x[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Per (i,j,k) triple of the energy loop, independent of the tuple: the
// occupied-orbital part of the denominator, summed as the loop summed it,
// and the weight 2 fac_jk fac_ij of src/atrip/Equations.cxx:101-238 (both
// factors 1/2 on equal indices; a power of two, so applying it to the
// reciprocal instead of the quotient is exact).
__global__ void triple_table_kernel(const uint32_t *__restrict__ triples, int n,
                                    const double *__restrict__ epsi, double2 *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t tp = triples[t];
    const int i = tp & 0xff, j = (tp >> 8) & 0xff, k = (tp >> 16) & 0xff;
    const double fac = (j == k ? 0.5 : 1.0) * (i == j ? 0.5 : 1.0);
    out[t] = make_double2((epsi[i] + epsi[j]) + epsi[k], 2.0 * fac);
  }
}

__device__ __noinline__ double recip_div(double d) { return 1.0 / d; }

// Exact conversions to FP64 done with integer instructions.  The energy
// warps are bound by this GPU's narrow FP64 pipe; integer operations run
// beside it.
// |n| < 2^51: 1.5 2^52 + n has ulp 1, so its bit pattern is that of
// 1.5 2^52 plus n in the low mantissa bits; subtracting 1.5 2^52 is exact.
__device__ __forceinline__ double i64_to_f64_exact(long long n) {
  return __longlong_as_double(0x4338000000000000ll + n) - 6755399441055744.0;
}
// Normal FP32 values: same sign and mantissa, exponent rebiased (127 ->
// 1023); zero, subnormal, infinity and NaN take the conversion instruction.
__device__ __forceinline__ double f32_to_f64_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) |
                                  ((unsigned long long)(e + 896u) << 52) |
                                  ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// 1/d for the energy denominators: d truncated to FP32 (integer
// operations), its FP32 reciprocal (rounded to nearest), widened exactly,
// refined by one Newton-Raphson step x1 = x0 + x0 (1 - d x0) in FP64.
// With |x0 d - 1| <= ~1.5 2^-23 the relative error of x1 is about its
// square (< 2^-44) plus one rounding; outside the FP32 exponent range it
// falls back to the division (out of line: the orbital-energy gaps never
// get there).
__device__ __forceinline__ double recip_nr(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;
  if (e < -125 || e > 126) return recip_div(d);
  const uint32_t fb = ((uint32_t)(b >> 32) & 0x80000000u) | ((uint32_t)(e + 127) << 23) |
                      ((uint32_t)(b >> 29) & 0x7fffffu);
  const double x0 = f32_to_f64_exact(__frcp_rn(__uint_as_float(fb)));
  const double err = fma(-d, x0, 1.0);
  return fma(x0, err, x0);
}

// dst[s][R][k] (pitch Kp) = sign * digit_s(src(R, k) * scale) for k < K,
// 0 for K <= k < Kp.  Row R = (o * n1 + r1) * n2 + r2.  Digits of radix
// 2^bits, |q| <= 2^(bits-1): BF16 values for bits = 8, FP16 for bits = 11
// (integers up to 2^8 and 2^11 are exact in them).
struct SliceJob {
  const double *src;
  __nv_bfloat16 *dst;
  int64_t nrows, n1, n2, so, s1, s2, sk;
  int K, Kp, S, bits;
  double scale, sign;
};

__global__ void slice_kernel(SliceJob j) {
  const int64_t total = j.nrows * j.Kp;
  const int64_t plane = total;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t R = idx / j.Kp;
    const int k = (int)(idx - R * j.Kp);
    double y = 0.0;
    if (k < j.K) {
      const int64_t r2 = R % j.n2, t = R / j.n2, r1 = t % j.n1, o = t / j.n1;
      y = j.src[o * j.so + r1 * j.s1 + r2 * j.s2 + k * j.sk] * j.scale;
    }
    const double radix = j.bits == 11 ? 2048.0 : 256.0;
    for (int s = 0; s < j.S; ++s) {
      const double q = rint(y);
      if (j.bits == 11)
        reinterpret_cast<__half *>(j.dst)[s * plane + idx] = __double2half(j.sign * q);
      else
        j.dst[s * plane + idx] = __double2bfloat16(j.sign * q);
      y = (y - q) * radix;
    }
  }
}

// --------------------------------------------------------------- kernel

__device__ __forceinline__ void named_bar_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// Barrier over n threads that also ANDs a predicate across them.
__device__ __forceinline__ bool named_bar_and(int id, int n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

struct Part {
  const CUtensorMap *amap, *bmap, *bmap3;
  int ax, bz, by;  // A: tensor index (x or w); B: (z, y) or (v, u)
  bool particle;
};

// Operand sources of group g, part pt (0 nat particle, 1 nat hole,
// 2 transposed particle, 3 transposed hole) for tuple (a,b,c).
__device__ __forceinline__ Part part_of(const SplitMaps &m, int g, int pt, int a, int b, int c,
                                        int pass, bool tv) {
  // per group: natural (x, w, (y,z), hole (u,v), holeT), transposed likewise
  int x, w, y, z, u, v, holeT;
  const bool tr = pt >= 2;
  if (g == 0) {
    if (!tr) { x = a; w = b; y = b; z = c; u = a; v = c; holeT = 0; }
    else     { x = b; w = a; y = a; z = c; u = b; v = c; holeT = 0; }
  } else if (g == 1) {
    if (!tr) { x = a; w = c; y = c; z = b; u = a; v = b; holeT = 0; }
    else     { x = c; w = a; y = a; z = b; u = b; v = c; holeT = 1; }
  } else {
    if (!tr) { x = b; w = c; y = c; z = a; u = a; v = b; holeT = 1; }
    else     { x = c; w = b; y = b; z = a; u = a; v = c; holeT = 1; }
  }
  Part p;
  p.particle = (pt & 1) == 0;
  // amap: the (p,q)-row operand (T_x or V_hhhp[w] slab), bmap: the r-column
  // operand (V_yz or T_uv); tv selects the maps of the transposed variant
  if (p.particle) {
    p.amap = tv ? (tr ? &m.TaT2 : &m.TaN2) : (tr ? &m.TaT : &m.TaN);
    p.ax = x;
    p.bmap = tv ? (pass ? &m.Jp2 : &m.Vp2) : (pass ? &m.Jp : &m.Vp);
    p.bmap3 = pass ? &m.Jp3 : &m.Vp3;
    p.bz = z;
    p.by = y;
  } else {
    p.amap = tv ? (pass ? (tr ? &m.JhT2 : &m.JhN2) : (tr ? &m.VhT2 : &m.VhN2))
                : (pass ? (tr ? &m.JhT : &m.JhN) : (tr ? &m.VhT : &m.VhN));
    p.ax = w;
    p.bmap = tv ? (holeT ? &m.TpT2 : &m.TpN2) : (holeT ? &m.TpT : &m.TpN);
    p.bmap3 = holeT ? &m.TpT3 : &m.TpN3;
    p.bz = v;
    p.by = u;
  }
  return p;
}

template <int S, int NP, bool SPLIT0>
struct KernelShape {
  static constexpr int kNacc = S + (SPLIT0 ? 1 : 0);
  static constexpr int kBufCols = kNacc * NP;
  static constexpr int kNbuf = (2 * kBufCols <= 512) ? 2 : 1;
  static constexpr int kCols = kNbuf * kBufCols;
  static constexpr int kAllocCols = kCols <= 32 ? 32 : kCols <= 64 ? 64 : kCols <= 128 ? 128
                                    : kCols <= 256 ? 256 : 512;
  static constexpr int kBTile = NP * 128;
  static constexpr int kStageBytes = kATileBytes + S * kBTile;
};

// Transposed variant: M = 128 rows holding the S slices of the r-column
// operand stacked (row s No + r), N = nmma <= 256 columns of (p,q) pairs,
// one 128 x 256 FP32 accumulator per item, double-buffered (all 512 TMEM
// columns).  The ring stages are sized at launch (t_stage).
template <int S, bool MSHARE = false>
struct KernelShapeT {
  static constexpr int kBufCols = 256;
  static constexpr int kNbuf = 2;
  static constexpr int kAllocCols = 512;
};
constexpr int kMSlots = 2;
constexpr int kStageCols = 64;   // epilogue staging: 128 rows x 64 FP32 columns,
constexpr int kStagePitch = 65;  // padded against bank conflicts

// Tuple hand-off ring: the producer owns the work queue and publishes each
// tuple to the MMA issuer, the epilogue warps and the energy warps.
constexpr int kTupleSlots = 4;
constexpr int kEnergyWarps = 10;  // warps 2, 3 and 8 .. 15
constexpr int kEnergyThreads = kEnergyWarps * 32;

struct TupleSlot {
  int64_t t;  // list position, -1 = no more work
  int a, b, c;
  int s;      // system (multi-system launches), else 0
};

// One system of a multi-system launch: its tensor maps (global memory) and
// the arguments that differ between systems.
struct SysDesc {
  SplitMaps maps;
  const double *epsa, *tai, *Vhh;
  const uint32_t *tuples, *triples;
  const double2 *tri_ef;
  double *e, *ect;
  double unit, unit_j;
  int64_t t_begin;  // list position of the system's first queued tuple
  int No, Nv, jt2, ntiles2, nmma, kch, b_off, n_triples, use_j;
};

// The per-system values of the tuple a role works on: the launch's own
// arguments, or the tuple's system descriptor.
struct SysRef {
  const SplitMaps *maps;
  const double *epsa, *tai, *Vhh;
  const uint32_t *tuples, *triples;
  int64_t t_begin;
  const double2 *tri_ef;
  double *e, *ect;
  double unit, unit_j;
  int No, Nv, jt, ntiles, kch, nmma, b_off, n_triples, use_j;
};

template <bool MULTI, bool TV>
__device__ __forceinline__ SysRef sys_ref(const SplitArgs &g, const SplitMaps &maps, int s) {
  SysRef r;
  if constexpr (MULTI) {
    const SysDesc &d = g.sys[s];
    r.maps = &d.maps;
    r.epsa = d.epsa;
    r.tai = d.tai;
    r.Vhh = d.Vhh;
    r.tuples = d.tuples;
    r.t_begin = d.t_begin;
    r.triples = d.triples;
    r.tri_ef = d.tri_ef;
    r.e = d.e;
    r.ect = d.ect;
    r.unit = d.unit;
    r.unit_j = d.unit_j;
    r.No = d.No;
    r.Nv = d.Nv;
    r.jt = d.jt2;
    r.ntiles = d.ntiles2;
    r.kch = d.kch;
    r.nmma = d.nmma;
    r.b_off = d.b_off;
    r.n_triples = d.n_triples;
    r.use_j = d.use_j;
  } else {
    r.maps = &maps;
    r.epsa = g.epsa;
    r.tai = g.tai;
    r.Vhh = g.Vhh;
    r.tuples = g.tuples;
    r.t_begin = g.t_begin;
    r.triples = g.triples;
    r.tri_ef = g.tri_ef;
    r.e = g.e;
    r.ect = g.ect;
    r.unit = g.unit;
    r.unit_j = g.unit_j;
    r.No = g.No;
    r.Nv = g.Nv;
    r.jt = TV ? g.jt2 : g.jt;
    r.ntiles = TV ? g.ntiles2 : g.ntiles;
    r.kch = g.kch;
    r.nmma = g.nmma;
    r.b_off = g.b_off;
    r.n_triples = g.n_triples;
    r.use_j = g.use_j;
  }
  return r;
}

// Make a tensor map written to global memory before the launch visible to
// the bulk-copy engine (multi-system launches keep their maps there).
__device__ __forceinline__ void tensormap_acquire(const void *map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                   reinterpret_cast<uint64_t>(map))
               : "memory");
}

// Role profile of a launch (kernel instantiations with PROF only): SM cycles
// each role spends in total and in each of its waits, summed over the CTAs.
enum ProfSlot {
  kProfProdTotal, kProfProdEmpty, kProfProdTupleEmpty,
  kProfMmaTotal, kProfMmaTupleFull, kProfMmaAccEmpty, kProfMmaFull,
  kProfEpiTotal, kProfEpiTupleFull, kProfEpiWFree, kProfEpiAccFull,
  kProfEnTotal, kProfEnTupleFull, kProfEnWFull, kProfEnWConvert,
  kProfUnits = 16, kProfTuples, kProfCtas, kProfSlots = 20
};

// f() (a bounded wait) with its duration added to acc when PROF.
template <bool PROF, class F>
__device__ __forceinline__ bool prof_wait(long long &acc, F f) {
  if constexpr (PROF) {
    const long long t = clock64();
    const bool r = f();
    acc += clock64() - t;
    return r;
  } else {
    return f();
  }
}

__device__ __forceinline__ void prof_add(unsigned long long *prof, int slot, long long v) {
  atomicAdd(prof + slot, (unsigned long long)v);
}

__device__ __forceinline__ int energy_rank(int warp, int lane) {
  return ((warp < 4 ? warp - 2 : warp - 6) << 5) | lane;
}

// W cells live in global memory (two tuple parities x passes x three group
// buffers per CTA): one 8-byte cell per element and group, {int32 level-0
// sum, float rest}, stored by the epilogue without reading; the energy warps
// add the three groups into the FP64 value.  The
// epilogue warps fill buffer k % 2 for tuple k while the energy warps read
// buffer (k-1) % 2, so the tensor-core work of one tuple overlaps the FP64
// energy evaluation of the previous one.
// F16 (transposed variant only): FP16 digits of radix 2^11.  Level 0 is
// then an FP32 sum of products up to 2^20 -- rounded, not exact, but an
// integer below 2^31 for K < 2048, so the int32 cell format still holds it.
template <int S, int NP, bool SPLIT0, bool WSMEM, bool TV, bool MSHARE = false, bool F16 = false,
          bool MULTI = false, bool PROF = false>
__global__ void __launch_bounds__(kThreads, 1)
    triples_split_kernel(const __grid_constant__ SplitMaps maps, const SplitArgs g) {
  using K = typename std::conditional<TV, KernelShapeT<S, MSHARE>, KernelShape<S, NP, SPLIT0>>::type;
  constexpr float kInvRadix = F16 ? 1.f / 2048.f : 1.f / 256.f;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *ring = smem;
  // layout sizes (the largest system of a multi-system launch); the roles
  // shadow No, No2, No3 and npass with the values of the tuple at hand
  const int No = g.no_lay, No2 = No * No, No3 = No2 * No;
  const size_t WP = (size_t)No3;  // pitch of one group's W cells
  const int kStages = g.nstages;
  unsigned char *mring = ring + kStages * g.stage_bytes;  // MSHARE slots
  unsigned char *tail = mring + (MSHARE ? kMSlots * g.mslot_bytes : 0);
  // W buffers: [tuple parity][pass] per CTA, pass 1 = J intermediates
  const int npass = g.npass_lay;
  const int npL = npass;
  // W buffers: [tuple parity][pass][group] per CTA; each group's items
  // store their contribution to every cell (no read-modify-write), the
  // energy warps add the three groups
  double *Wbase = reinterpret_cast<double *>(g.wglobal) + (size_t)blockIdx.x * 2 * npass * 3 * No3;
  uint64_t *full = reinterpret_cast<uint64_t *>(tail);
  uint64_t *empty = full + kMaxStages;
  uint64_t *accf = empty + kMaxStages;
  uint64_t *acce = accf + 2;
  uint64_t *tfull = acce + 2;
  uint64_t *tempty = tfull + kTupleSlots;
  uint64_t *wfull = tempty + kTupleSlots;
  uint64_t *wfree = wfull + 2;
  uint64_t *mfull = wfree + 2;  // MSHARE slot barriers
  uint64_t *mempty = mfull + kMSlots;
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(mempty + kMSlots);
  TupleSlot *tslot = reinterpret_cast<TupleSlot *>(tail + 264);
  double *ta = reinterpret_cast<double *>(tail + 384);
  double *tb = ta + 64;
  double *tc = tb + 64;
  double *red = tc + 64;        // [kEnergyWarps]
  double *Vsm = red + 16 + 64;  // the singles' 3 No x No blocks (g.vsm)
  double *Wsm = Vsm + (g.vsm ? 3 * No2 : 0);  // FP64 copy of W for the energy loop (WSMEM)
  float *stg = reinterpret_cast<float *>(Wsm + (WSMEM ? No3 : 0));  // TV epilogue staging

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 128);
      mbar_init(&wfull[b], 1);
      mbar_init(&wfree[b], 1);
      mbar_init(&mfull[b], 1);
      mbar_init(&mempty[b], 1);
    }
    for (int s = 0; s < kTupleSlots; ++s) {
      mbar_init(&tfull[s], 1);
      mbar_init(&tempty[s], 3);
    }
    fence_mbar_init();
  }
  if (threadIdx.x == 0 && !MULTI) {
    prefetch_tensormap(&maps.TaN);
    prefetch_tensormap(&maps.TaT);
    prefetch_tensormap(&maps.VhN);
    prefetch_tensormap(&maps.VhT);
    prefetch_tensormap(&maps.Vp);
    prefetch_tensormap(&maps.TpN);
    prefetch_tensormap(&maps.TpT);
    if (g.use_j) {
      prefetch_tensormap(&maps.JhN);
      prefetch_tensormap(&maps.JhT);
      prefetch_tensormap(&maps.Jp);
    }
  }
  // rows of the A stage tiles past No*jt are never written by TMA: zero them
  for (int i = threadIdx.x;
       i < (kStages * g.stage_bytes + (MSHARE ? kMSlots * g.mslot_bytes : 0)) / 16;
       i += kThreads)
    reinterpret_cast<uint4 *>(ring)[i] = make_uint4(0, 0, 0, 0);
  if (warp == 1) {
    tmem_alloc(tmem_holder, K::kAllocCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  if (warp == 0) {
    // ------------------------------------------------------ TMA producer
    if (lane == 0 && !g.unpublished) {
      const long long c_start = PROF ? clock64() : 0;
      long long c_empty = 0, c_tempty = 0;
      uint32_t mcount = 0;
      int pst = 0;          // ring slot of the next unit
      uint32_t puse = 0;    // completed passes over the ring
      unsigned char *sbase = ring;
      // multi-system launch: the system of the previous tuple, its queue
      // range and values (the positions one CTA draws only grow, so a new
      // system is looked for only past the end of the current one)
      int cur = -1;
      unsigned long long cur_lo = 0, cur_hi = 0;
      SysRef P = sys_ref<MULTI, TV>(g, maps, 0);
      const unsigned long long total = MULTI ? (unsigned long long)g.prefix[g.nsys]
                                             : (unsigned long long)(g.t_end - g.t_begin);
      bool alive = true;
      for (uint32_t k = 0;; ++k) {
        const int ts = k % kTupleSlots;
        const uint32_t tuse = k / kTupleSlots;
        if (tuse > 0 && !prof_wait<PROF>(c_tempty, [&] {
              return mbar_wait(&tempty[ts], (tuse - 1) & 1, g.status, kErrTimeoutEmpty, g.wait_cycles);
            }))
          alive = false;
        const unsigned long long q = alive ? atomicAdd(g.queue, 1ull) : ~0ull;
        const bool stop = !alive || q >= total || *reinterpret_cast<volatile int *>(g.status) != 0;
        TupleSlot s;
        s.a = s.b = s.c = 0;
        s.s = 0;
        if (stop) {
          s.t = -1;
        } else if constexpr (MULTI) {
          if (q >= cur_hi) {
            int lo = cur < 0 ? 0 : cur;
            while (lo + 1 < g.nsys && (unsigned long long)g.prefix[lo + 1] <= q) ++lo;
            cur = lo;
            cur_lo = (unsigned long long)g.prefix[lo];
            cur_hi = (unsigned long long)g.prefix[lo + 1];
            // first tuple of another system: its values and maps, once
            P = sys_ref<MULTI, TV>(g, maps, lo);
            const SplitMaps &M = *P.maps;
            tensormap_acquire(&M.TaN2);
            tensormap_acquire(&M.TaT2);
            tensormap_acquire(&M.VhN2);
            tensormap_acquire(&M.VhT2);
            tensormap_acquire(&M.Vp2);
            tensormap_acquire(&M.TpN2);
            tensormap_acquire(&M.TpT2);
            if (P.use_j) {
              tensormap_acquire(&M.JhN2);
              tensormap_acquire(&M.JhT2);
              tensormap_acquire(&M.Jp2);
            }
          }
          s.s = cur;
          s.t = P.t_begin + (int64_t)(q - cur_lo);
        } else {
          s.t = g.t_begin + (g.order ? (int64_t)g.order[q] : (int64_t)q);
        }
        if (!stop) {
          const uint32_t pk = P.tuples[s.t];
          s.a = pk & 0x3ff;
          s.b = (pk >> 10) & 0x3ff;
          s.c = (pk >> 20) & 0x3ff;
        }
        tslot[ts] = s;
        mbar_arrive(&tfull[ts]);  // release: the slot is visible to the waiters
        if (stop) break;
        // this tuple's system: its sizes (its tensor maps through P.maps)
        const int No = P.No, jt = P.jt, ntiles = P.ntiles, kch = P.kch;
        const int npass = P.use_j ? 2 : 1, a_bytes = 128 * No * jt;
        for (int gi = 0; gi < 3 * npass && alive; ++gi)
          for (int mt = 0; mt < ntiles && alive; ++mt) {
            const int j0 = mt * jt, grp = gi % 3, pass = gi / 3;
            for (int pt = 0; pt < 4 && alive; ++pt) {
              const Part p = part_of(*P.maps, grp, pt, s.a, s.b, s.c, pass, TV);
              const int nch = p.particle ? kch : 1;
              if (g.prefetch) {
                // the next part of this tuple: its (p,q)-row tiles (the
                // slabs of T and V_hhhp, the large operands) into L2 while
                // this part streams; only boxes wholly inside the tensor
                int ngi = gi, nmt = mt, npt = pt + 1;
                if (npt == 4) { npt = 0; if (++nmt == ntiles) { nmt = 0; ++ngi; } }
                const int nj0 = nmt * jt;
                if (ngi < 3 * npass && nj0 + jt <= No) {
                  const Part np = part_of(*P.maps, ngi % 3, npt, s.a, s.b, s.c, ngi / 3, TV);
                  const int nnch = np.particle ? kch : 1;
                  for (int ch = 0; ch < nnch; ++ch)
                    for (int sa = 0; sa < S; ++sa)
                      tma_prefetch_5d(np.amap, ch * kKChunk, 0, nj0, np.ax, sa);
                }
              }
              for (int ch = 0; ch < nch && alive; ++ch)
                for (int sa = 0; sa < S; ++sa) {
                  if constexpr (MSHARE) {
                    if (sa == 0) {
                      // one M-side stack per K chunk: slices -(S-1) .. S-1
                      // (the negative ones read as zeros); slice unit sa
                      // uses the 128 rows from row block S-1-sa
                      const int ms = mcount % kMSlots;
                      const uint32_t muse = mcount / kMSlots;
                      if (muse > 0 &&
                          !mbar_wait(&mempty[ms], (muse - 1) & 1, g.status, kErrTimeoutEmpty, g.wait_cycles)) {
                        alive = false;
                        break;
                      }
                      mbar_arrive_expect_tx(&mfull[ms], 128 * (2 * S - 1) * No);
                      tma_load_5d(mring + ms * g.mslot_bytes, p.bmap3, &mfull[ms], ch * kKChunk,
                                  0, p.bz, p.by, -(S - 1));
                      ++mcount;
                    }
                  }
                  const int st = pst;
                  if (puse > 0 && !prof_wait<PROF>(c_empty, [&] {
                        return mbar_wait(&empty[st], (puse - 1) & 1, g.status, kErrTimeoutEmpty,
                                         g.wait_cycles);
                      })) {
                    alive = false;
                    break;
                  }
                  if constexpr (MSHARE) {
                    mbar_arrive_expect_tx(&full[st], a_bytes);
                    tma_load_5d(sbase, p.amap, &full[st], ch * kKChunk, 0, j0, p.ax, sa);
                  } else if constexpr (TV) {
                    // M side: slices -sa .. S-1-sa of the r-column operand
                    // (those below 0 read as zeros), so row block j always
                    // holds level j = sa + sb; N side: (p,q) rows, slice sa
                    mbar_arrive_expect_tx(&full[st], 128 * S * No + a_bytes);
                    tma_load_5d(sbase, p.bmap, &full[st], ch * kKChunk, 0, p.bz, p.by, -sa);
                    tma_load_5d(sbase + P.b_off, p.amap, &full[st], ch * kKChunk, 0, j0, p.ax, sa);
                  } else {
                    const int nb = S - sa;
                    mbar_arrive_expect_tx(&full[st], a_bytes + nb * NP * 128);
                    tma_load_5d(sbase, p.amap, &full[st], ch * kKChunk, 0, j0, p.ax, sa);
                    for (int sb = 0; sb < nb; ++sb)
                      tma_load_5d(sbase + kATileBytes + sb * K::kBTile, p.bmap, &full[st],
                                  ch * kKChunk, 0, p.bz, p.by, sb);
                  }
                  if (++pst == kStages) {
                    pst = 0;
                    ++puse;
                    sbase = ring;
                  } else {
                    sbase += g.stage_bytes;
                  }
                }
            }
          }
      }
      if constexpr (PROF) {
        prof_add(g.prof, kProfProdTotal, clock64() - c_start);
        prof_add(g.prof, kProfProdEmpty, c_empty);
        prof_add(g.prof, kProfProdTupleEmpty, c_tempty);
        prof_add(g.prof, kProfCtas, 1);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // -------------------------------------------------------- MMA issuer
    if (lane == 0) {
      // the issuer is a single thread: keep its per-unit work to a few
      // additions (incremental ring slot, phase and descriptor offset; no
      // divisions), so the tensor pipe's short instruction queue stays fed
      const long long c_start = PROF ? clock64() : 0;
      long long c_tfull = 0, c_acce = 0, c_full = 0, n_units = 0, n_tuples = 0;
      uint32_t item_count = 0, mcount = 0;
      int st = 0;           // ring slot of the next unit
      uint32_t ph = 0;      // its full-barrier phase parity
      uint32_t st_off = 0;  // its descriptor offset (bytes >> 4)
      const uint64_t ring_desc = sdesc_sw128(smem_u32(ring));
      const uint32_t stage_step = (uint32_t)g.stage_bytes >> 4;
      int cur = -1;  // system of the previous tuple (multi-system launch)
      SysRef P = sys_ref<MULTI, TV>(g, maps, 0);
      bool alive = true;
      for (uint32_t k = 0;; ++k) {
        const int ts = k % kTupleSlots;
        if (!prof_wait<PROF>(c_tfull, [&] {
              return mbar_wait(&tfull[ts], (k / kTupleSlots) & 1, g.status, kErrTimeoutFull,
                               g.wait_cycles);
            }))
          break;
        const int64_t t = tslot[ts].t;
        const int sys = tslot[ts].s;
        mbar_arrive(&tempty[ts]);
        if (t < 0) break;
        ++n_tuples;
        if (MULTI && sys != cur) {  // another system: its values, once
          cur = sys;
          P = sys_ref<MULTI, TV>(g, maps, sys);
        }
        const int No = P.No, ntiles = P.ntiles, kch = P.kch, npass = P.use_j ? 2 : 1;
        const uint32_t b_step = (uint32_t)P.b_off >> 4;
        const uint32_t id_tv = F16 ? idesc_f16_f32(128, P.nmma) : idesc_bf16_f32(128, P.nmma);
        for (int it = 0; it < 3 * npass * ntiles && alive; ++it) {
          const int buf = item_count % K::kNbuf;
          const uint32_t use = item_count / K::kNbuf;
          if (use > 0 && !prof_wait<PROF>(c_acce, [&] {
                return mbar_wait(&acce[buf], (use - 1) & 1, g.status, kErrTimeoutAccEmpty,
                                 g.wait_cycles);
              })) {
            alive = false;
            break;
          }
          tc_fence_after();
          bool fresh_main = true, fresh_tr0 = true;
          const uint32_t dbase = tmem + buf * K::kBufCols;
          for (int pt = 0; pt < 4 && alive; ++pt) {
            const int nch = (pt & 1) == 0 ? kch : 1;
            for (int ch = 0; ch < nch && alive; ++ch) {
              // K steps of 16 that hold data: the zero padding past Nv (last
              // particle chunk) and past No (hole chunk) is skipped
              const int kvalid = (pt & 1) == 0 ? min(kKChunk, P.Nv - ch * kKChunk) : No;
              const int nkk = (kvalid + 15) / 16;
              const int ms = mcount % kMSlots;
              for (int sa = 0; sa < S; ++sa) {
                if constexpr (MSHARE) {
                  if (sa == 0 &&
                      !mbar_wait(&mfull[ms], (mcount / kMSlots) & 1, g.status, kErrTimeoutFull, g.wait_cycles)) {
                    alive = false;
                    break;
                  }
                }
                ++n_units;
                if (!prof_wait<PROF>(c_full, [&] {
                      return mbar_wait(&full[st], ph, g.status, kErrTimeoutFull, g.wait_cycles);
                    })) {
                  alive = false;
                  break;
                }
                tc_fence_after();
                // descriptors: the ring's base descriptor plus the stage
                // offset (shared-memory addresses stay below 2^18, so the
                // 14-bit address field never carries)
                const uint64_t sdesc = ring_desc + st_off;
                // MSHARE: A = the chunk's shared stack from row block S-1-sa
                // (No % 8 == 0 keeps the start on a 1024-byte swizzle atom)
                const uint64_t adesc =
                    MSHARE ? sdesc_sw128(smem_u32(mring + ms * g.mslot_bytes) +
                                         (uint32_t)((S - 1 - sa) * No * 128))
                           : sdesc;
                const uint64_t bdesc = sdesc + b_step;
                // A slice sa against B slices 0 .. S-1-sa in one MMA: the
                // result columns are the level accumulators sa .. S-1, which
                // sit side by side in TMEM.  (Transposed variant: the stacked
                // slices are the M rows, the (p,q) pairs the N columns.)
                if constexpr (TV) {
#pragma unroll
                  for (int kk = 0; kk < kKChunk / 16; ++kk)
                    if (kk < nkk)
                      mma_bf16(dbase, adesc + 2 * kk, bdesc + 2 * kk, id_tv,
                               (fresh_main && kk == 0) ? 0u : 1u);
                  fresh_main = false;
                } else if (SPLIT0 && pt >= 2 && sa == 0) {
                  // level 0 of the transposed half has its own accumulator
#pragma unroll
                  for (int kk = 0; kk < kKChunk / 16; ++kk)
                    if (kk < nkk)
                      mma_bf16(dbase + S * NP, adesc + 2 * kk, bdesc + 2 * kk,
                               idesc_bf16_f32(128, NP), (fresh_tr0 && kk == 0) ? 0u : 1u);
                  fresh_tr0 = false;
                  if (S > 1) {
                    const uint64_t bdesc1 = sdesc + ((uint32_t)(kATileBytes + K::kBTile) >> 4);
#pragma unroll
                    for (int kk = 0; kk < kKChunk / 16; ++kk)
                      if (kk < nkk)
                        mma_bf16(dbase + NP, adesc + 2 * kk, bdesc1 + 2 * kk,
                                 idesc_bf16_f32(128, (S - 1) * NP), 1u);
                  }
                } else {
                  const uint32_t id = idesc_bf16_f32(128, (S - sa) * NP);
#pragma unroll
                  for (int kk = 0; kk < kKChunk / 16; ++kk)
                    if (kk < nkk)
                      mma_bf16(dbase + sa * NP, adesc + 2 * kk, bdesc + 2 * kk, id,
                               (fresh_main && kk == 0) ? 0u : 1u);
                  fresh_main = false;
                }
                mma_commit(&empty[st]);
                if (++st == kStages) {
                  st = 0;
                  ph ^= 1u;
                  st_off = 0;
                } else {
                  st_off += stage_step;
                }
                if constexpr (MSHARE) {
                  if (sa == S - 1) {
                    mma_commit(&mempty[ms]);  // the stack is free once these MMAs end
                    ++mcount;
                  }
                }
              }
            }
          }
          mma_commit(&accf[buf]);
          ++item_count;
        }
        if (!alive) break;
      }
      if constexpr (PROF) {
        prof_add(g.prof, kProfMmaTotal, clock64() - c_start);
        prof_add(g.prof, kProfMmaTupleFull, c_tfull);
        prof_add(g.prof, kProfMmaAccEmpty, c_acce);
        prof_add(g.prof, kProfMmaFull, c_full);
        prof_add(g.prof, kProfUnits, n_units);
        prof_add(g.prof, kProfTuples, n_tuples);
      }
    }
    __syncwarp();
  } else if (warp >= 4 && warp < 8) {
    // ------------------------------------------------ epilogue (4 warps)
    // warp % 4 selects the 32-lane TMEM quarter this warp may read
    const int quarter = warp - 4;
    const int l = quarter * 32 + lane;
    const long long c_start = PROF ? clock64() : 0;
    long long c_tfull = 0, c_wfree = 0, c_accf = 0;
    uint32_t item_count = 0;
    int cur = -1;  // system of the previous tuple (multi-system launch)
    SysRef P = sys_ref<MULTI, TV>(g, maps, 0);
    bool alive = true;
    for (uint32_t k = 0;; ++k) {
      const int ts = k % kTupleSlots;
      bool ok = prof_wait<PROF>(c_tfull, [&] {
        return mbar_wait(&tfull[ts], (k / kTupleSlots) & 1, g.status, kErrTimeoutFull, g.wait_cycles);
      });
      const int64_t t = tslot[ts].t;
      const int sys = tslot[ts].s;
      // agree on ok so that every epilogue thread leaves (or stays) together
      ok = named_bar_and(1, 128, ok);
      if (threadIdx.x == 128) mbar_arrive(&tempty[ts]);
      if (!ok || t < 0) break;
      if (MULTI && sys != cur) {  // another system: its values, once
        cur = sys;
        P = sys_ref<MULTI, TV>(g, maps, sys);
      }
      const int No = P.No, jt = P.jt, ntiles = P.ntiles;
      const int npass = P.use_j ? 2 : 1;
      const int wb = k & 1;
      const uint32_t wuse = k >> 1;
      ok = wuse == 0 || prof_wait<PROF>(c_wfree, [&] {
             return mbar_wait(&wfree[wb], (wuse - 1) & 1, g.status, kErrTimeoutEmpty, g.wait_cycles);
           });
      for (int it = 0; it < 3 * npass * ntiles; ++it) {
        const int gi = it / ntiles, mt = it % ntiles, grp = gi % 3, pass = gi / 3;
        int2 *Wc = reinterpret_cast<int2 *>(Wbase + (size_t)((wb * npL + pass) * 3 + grp) * WP);
        const int buf = item_count % K::kNbuf;
        const uint32_t use = item_count / K::kNbuf;
        bool okw = ok && alive && prof_wait<PROF>(c_accf, [&] {
                     return mbar_wait(&accf[buf], use & 1, g.status, kErrTimeoutAccFull, g.wait_cycles);
                   });
        // tcgen05.ld is warp-collective: agree; a failed wait skips the
        // loads but meets the same barriers as the other epilogue warps
        okw = __all_sync(0xffffffffu, okw);
        if (!okw) alive = false;
        tc_fence_after();
        if constexpr (TV) {
          // accumulator: lane s No + r = level s of column r, TMEM column n
          // = (p,q) pair p + No (q - q0); the four warps stage 64 columns at
          // a time in shared memory, then each thread recombines the levels
          // of its (r, column) cells and stores them into the group's W
          const bool okall = named_bar_and(3, 128, okw);
          if (!okall) alive = false;
          const int q0 = mt * jt;
          const int nvalid = No * min(jt, No - q0);
          const int t128 = threadIdx.x - 128, cc = t128 & (kStageCols - 1);
          const int rq = t128 / kStageCols;  // 0 or 1
          // floor(x / No) = (x * mno) >> 20 exactly for x < 2^12, No <= 64
          const uint32_t mno = ((1u << 20) + (uint32_t)No - 1) / (uint32_t)No;
          const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + buf * K::kBufCols;
          for (int c0 = 0; c0 < nvalid && okall; c0 += kStageCols) {
            // only the S No level rows are staged (rows past them hold
            // products with whatever follows the stack in shared memory)
            float *row = stg + l * kStagePitch;
#pragma unroll
            for (int h = 0; h < kStageCols / 16; ++h) {
              float v[16];
              tmem_ld16(tbase + c0 + 16 * h, v);
              tmem_wait_ld();
              if (l < S * No) {
#pragma unroll
                for (int x = 0; x < 16; ++x) row[16 * h + x] = v[x];
              }
            }
            named_bar_sync(1, 128);
            // cells (r, column): groups 0 and 1 walk the columns across a
            // warp (W index consecutive in p), group 2 walks r (its W index
            // is consecutive in r), so every warp store coalesces
            if (grp != 2) {
              // one column per thread, rows rq, rq + 2, ...: the column's
              // (p, q) and the W index of row 0 once, then a fixed stride
              const int n = c0 + cc;
              if (n < nvalid) {
                const int nq = (int)(((uint32_t)n * mno) >> 20);
                const int f = n - nq * No, sl = q0 + nq;
                // group 0: (i, j, k) = (f, sl, r); group 1: (f, r, sl)
                const int base = grp == 0 ? f + No * sl : f + No * No * sl;
                const int rstep = grp == 0 ? No * No : No;
                const float *col = stg + cc;
                for (int r = rq; r < No; r += 2) {
                  const int lev0 = __float2int_rn(col[r * kStagePitch]);
                  float rr = 0.f;
#pragma unroll
                  for (int q = S - 1; q >= 1; --q)
                    rr = rr * kInvRadix + col[(q * No + r) * kStagePitch];
                  __stcg(&Wc[base + r * rstep], make_int2(lev0, __float_as_int(rr * kInvRadix)));
                }
              }
            } else {
              const int ncells = No * kStageCols;
              for (int id = t128; id < ncells; id += 128) {
                const int ccu = (int)(((uint32_t)id * mno) >> 20);
                const int r = id - ccu * No;
                const int n = c0 + ccu;
                if (n >= nvalid) continue;
                const int lev0 = __float2int_rn(stg[r * kStagePitch + ccu]);
                float rr = 0.f;
#pragma unroll
                for (int q = S - 1; q >= 1; --q)
                  rr = rr * kInvRadix + stg[(q * No + r) * kStagePitch + ccu];
                const int nq = (int)(((uint32_t)n * mno) >> 20);
                const int f = n - nq * No, sl = q0 + nq;
                // group 2: (i, j, k) = (r, f, sl)
                __stcg(&Wc[r + No * (f + No * sl)],
                       make_int2(lev0, __float_as_int(rr * kInvRadix)));
              }
            }
            named_bar_sync(1, 128);  // the staging buffer is reused
          }
        } else {
          const int j0 = mt * jt;
          const int rows = No * min(jt, No - j0);
          const bool valid = l < rows;
          const int f = l % No, sl = j0 + l / No;
          const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + buf * K::kBufCols;
          for (int c0 = 0; c0 < NP && okw; c0 += 16) {
            float v[K::kNacc][16];
#pragma unroll
            for (int q = 0; q < K::kNacc; ++q) tmem_ld16(tbase + q * NP + c0, v[q]);
            tmem_wait_ld();
            if (valid) {
              // level-0 integer and weighted rest of the 16 columns
              int lev0[16];
              float rest[16];
#pragma unroll
              for (int cc = 0; cc < 16; ++cc) {
                lev0[cc] = __float2int_rn(v[0][cc]);
                if (SPLIT0) lev0[cc] += __float2int_rn(v[S][cc]);
                float r = 0.f;
#pragma unroll
                for (int q = S - 1; q >= 1; --q) r = r * kInvRadix + v[q][cc];
                rest[cc] = r * kInvRadix;
              }
              // the 16 cells are distinct elements of W: issue every load
              // before any store so the round trips to L2 overlap
              int idx[16];
#pragma unroll
              for (int cc = 0; cc < 16; ++cc) {
                const int col = c0 + cc;
                int i, jj, kx;
                if (grp == 0) { i = f; jj = sl; kx = col; }
                else if (grp == 1) { i = f; kx = sl; jj = col; }
                else { jj = f; kx = sl; i = col; }
                idx[cc] = col < No ? i + No * (jj + No * kx) : -1;
              }
#pragma unroll
              for (int cc = 0; cc < 16; ++cc)
                if (idx[cc] >= 0)
                  __stcg(&Wc[idx[cc]], make_int2(lev0[cc], __float_as_int(rest[cc])));
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acce[buf]);
        named_bar_sync(1, 128);  // orders the scatters of consecutive items
        ++item_count;
      }
      // W of tuple k complete: hand it to the energy warps
      __threadfence_block();
      named_bar_sync(1, 128);
      if (threadIdx.x == 128) mbar_arrive(&wfull[wb]);
    }
    if (PROF && threadIdx.x == 128) {
      prof_add(g.prof, kProfEpiTotal, clock64() - c_start);
      prof_add(g.prof, kProfEpiTupleFull, c_tfull);
      prof_add(g.prof, kProfEpiWFree, c_wfree);
      prof_add(g.prof, kProfEpiAccFull, c_accf);
    }
    __syncwarp();
  } else if (warp < 16) {
    // ------------------------------------------------ energy (10 warps)
    const int er = energy_rank(warp, lane);
    const long long c_start = PROF ? clock64() : 0;
    long long c_tfull = 0, c_wfull = 0, c_conv = 0, c_t0 = 0;
    int cur = -1;  // system of the previous tuple (multi-system launch)
    SysRef P = sys_ref<MULTI, TV>(g, maps, 0);
    for (uint32_t k = 0;; ++k) {
      const int ts = k % kTupleSlots;
      bool ok = prof_wait<PROF>(c_tfull, [&] {
        return mbar_wait(&tfull[ts], (k / kTupleSlots) & 1, g.status, kErrTimeoutFull, g.wait_cycles);
      });
      const TupleSlot s = tslot[ts];
      ok = named_bar_and(2, kEnergyThreads, ok);  // leave together
      if (er == 0) mbar_arrive(&tempty[ts]);
      if (!ok || s.t < 0) break;
      if (MULTI && s.s != cur) {  // another system: its values, once
        cur = s.s;
        P = sys_ref<MULTI, TV>(g, maps, s.s);
      }
      const int No = P.No, No2 = No * No, No3 = No2 * No;
      const int64_t Nv = P.Nv;
      // W, Z and the singles are carried in units of unit (W cell = level-0
      // integer + rest), the (cT) T in units of unit_j; both are powers of
      // two, so the tuple energies scale back exactly at the end
      const double inv_unit = 1.0 / P.unit;
      const int a = s.a, b = s.b, c = s.c;
      if (er < No) {
        // in units of the W cells (a power of two: exact)
        ta[er] = g.tai_sign * P.tai[a + er * Nv] * inv_unit;
        tb[er] = g.tai_sign * P.tai[b + er * Nv] * inv_unit;
        tc[er] = g.tai_sign * P.tai[c + er * Nv] * inv_unit;
      }
      if (g.vsm) {
        // the singles' blocks into shared memory while the MMAs of this
        // tuple run (visible to all after the W conversion's barrier)
        const double *Vbc = P.Vhh + ((int64_t)b * Nv + c) * No2;
        const double *Vac = P.Vhh + ((int64_t)a * Nv + c) * No2;
        const double *Vab = P.Vhh + ((int64_t)a * Nv + b) * No2;
        for (int i = er; i < No2; i += kEnergyThreads) {
          Vsm[i] = Vbc[i];
          Vsm[No2 + i] = Vac[i];
          Vsm[2 * No2 + i] = Vab[i];
        }
      }
      const int wb = k & 1;
      ok = prof_wait<PROF>(c_wfull, [&] {
        return mbar_wait(&wfull[wb], (k >> 1) & 1, g.status, kErrTimeoutAccFull, g.wait_cycles);
      });
      if constexpr (PROF) c_t0 = clock64();
      double *Wg = Wbase + (size_t)(wb * npL) * 3 * WP;
      const int2 *Wc0 = reinterpret_cast<const int2 *>(Wg);
      const int2 *Wc1 = Wc0 + WP, *Wc2 = Wc1 + WP;
      // W / unit = level-0 integer + rest in FP64 from the three group
      // cells (integer parts exact, rests added in group order): copied into
      // shared memory (the buffers go back to the epilogue at once), or,
      // when it does not fit, written in place over group 0's cells
      double *Wd = WSMEM ? Wsm : Wg;
      // level-0 parts: each below 2^24 (BF16 digits) or 2^31 (FP16 digits),
      // so their sum fits int32 or int64 respectively
      auto lev0 = [](int2 c0, int2 c1, int2 c2) {
        return i64_to_f64_exact((long long)c0.x + c1.x + c2.x);
      };
      // four elements per thread in flight: the cells come from L2
      constexpr int kU = 6;
      for (int i0 = er; i0 < No3; i0 += kU * kEnergyThreads) {
        int2 c[kU][3];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int i = i0 + u * kEnergyThreads;
          if (i < No3) {
            c[u][0] = Wc0[i];
            c[u][1] = Wc1[i];
            c[u][2] = Wc2[i];
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int i = i0 + u * kEnergyThreads;
          if (i < No3) {
            const float rest = (__int_as_float(c[u][0].y) + __int_as_float(c[u][1].y)) +
                               __int_as_float(c[u][2].y);
            Wd[i] = lev0(c[u][0], c[u][1], c[u][2]) + f32_to_f64_exact(rest);
          }
        }
      }
      __threadfence_block();
      named_bar_sync(2, kEnergyThreads);
      if constexpr (PROF) c_conv += clock64() - c_t0;
      if (WSMEM && !P.use_j && er == 0) mbar_arrive(&wfree[wb]);

      int cls = 0;  // src/atrip/Atrip.cxx:640-642
      if (a == b) cls++;
      if (b == c) cls--;
      const bool distinct = cls == 0;
      const double epsabc = P.epsa[a] + P.epsa[b] + P.epsa[c];
      // the singles' No x No blocks of V_hhpp: the shared copy, or read in
      // place (L1 / L2) where shared memory is left to the operand ring
      const double *Vbc = g.vsm ? Vsm : P.Vhh + ((int64_t)b * Nv + c) * No2;
      const double *Vac = g.vsm ? Vsm + No2 : P.Vhh + ((int64_t)a * Nv + c) * No2;
      const double *Vab = g.vsm ? Vsm + 2 * No2 : P.Vhh + ((int64_t)a * Nv + b) * No2;
      auto W = [&](int i, int j, int kx) { return Wd[i + No * (j + No * kx)]; };
      auto Zv = [&](int i, int j, int kx) {
        double z = W(i, j, kx);
        z += ta[i] * Vbc[j + kx * No];
        z += tb[j] * Vac[i + kx * No];
        z += tc[kx] * Vab[i + j * No];
        return z;
      };
      // one tuple energy (src/atrip/Equations.cxx:101-238) with T values
      // from Tv and Z = W + singles; reduced over the energy warps
      auto tuple_energy = [&](auto &&Tv) {
        double sum = 0.0;
        for (int n = er; n < P.n_triples && ok; n += kEnergyThreads) {
          const uint32_t tp = P.triples[n];
          const double2 ef = P.tri_ef[n];
          const int i = tp & 0xff, j = (tp >> 8) & 0xff, kx = (tp >> 16) & 0xff;
          const double denominator = epsabc - ef.x;
          double value;
          if (distinct) {
            const double U = Zv(i, j, kx), V = Zv(i, kx, j), Wv = Zv(j, i, kx),
                         X = Zv(j, kx, i), Y = Zv(kx, i, j), Z = Zv(kx, j, i);
            const double A = Tv(i, j, kx), B = Tv(i, kx, j), C = Tv(j, i, kx), D = Tv(j, kx, i),
                         E = Tv(kx, i, j), F = Tv(kx, j, i);
            const double UXY = U + (X + Y), VWZ = V + (Wv + Z), ADE = A + (D + E),
                         BCF = B + (C + F);
            const double first = A * U + (B * V + (C * Wv + (D * X + (E * Y + F * Z))));
            value = 3.0 * first + ((UXY - 2.0 * VWZ) * ADE + (VWZ - 2.0 * UXY) * BCF);
          } else {
            const double U = Zv(i, j, kx), V = Zv(j, kx, i), Wv = Zv(kx, i, j);
            const double A = Tv(i, j, kx), B = Tv(j, kx, i), C = Tv(kx, i, j);
            value = 3.0 * ((A * U + B * V) + C * Wv) - (A + (B + C)) * (U + (V + Wv));
          }
          sum = fma(value, recip_nr(denominator) * ef.y, sum);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) red[er >> 5] = sum;
        named_bar_sync(2, kEnergyThreads);
        double e = 0.0;
        for (int w = 0; w < kEnergyWarps; ++w) e += red[w];
        named_bar_sync(2, kEnergyThreads);  // red is reused
        return e;
      };
      const double e = (P.unit * P.unit) * tuple_energy(W);
      double ect = e;
      if (P.use_j) {
        // (cT): T from the J pass, Z as above (src/atrip/Atrip.cxx:928-963)
        const int2 *WJ0 = reinterpret_cast<const int2 *>(Wbase + (size_t)(wb * npL + 1) * 3 * WP);
        const int2 *WJ1 = WJ0 + WP, *WJ2 = WJ1 + WP;
        ect = (P.unit * P.unit_j) * tuple_energy([&](int i, int j, int kx) {
          const int x = i + No * (j + No * kx);
          const int2 c0 = WJ0[x], c1 = WJ1[x], c2 = WJ2[x];
          const float rest = (__int_as_float(c0.y) + __int_as_float(c1.y)) + __int_as_float(c2.y);
          return lev0(c0, c1, c2) + f32_to_f64_exact(rest);
        });
      }
      if (er == 0) {
        P.e[s.t] = e;
        P.ect[s.t] = ect;
      }
      // no zeroing: every group of the next tuple that uses these buffers
      // stores all of its cells
      named_bar_sync(2, kEnergyThreads);  // Wsm is reused by the next tuple
      if ((!WSMEM || P.use_j) && er == 0) mbar_arrive(&wfree[wb]);
    }
    if (PROF && er == 0) {
      prof_add(g.prof, kProfEnTotal, clock64() - c_start);
      prof_add(g.prof, kProfEnTupleFull, c_tfull);
      prof_add(g.prof, kProfEnWFull, c_wfull);
      prof_add(g.prof, kProfEnWConvert, c_conv);
    }
    __syncwarp();
  }

  // Leave only after every tcgen05 op of this CTA has completed: the
  // epilogue has drained every accumulator it was handed.
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, K::kAllocCols);
}

// ------------------------------------------------------------------ host

struct SplitImpl {
  int S = 0, No = 0, Nv = 0, Ep = 0;
  __nv_bfloat16 *TaS = nullptr, *TaST = nullptr, *VhS = nullptr, *VhST = nullptr,
                *VpS = nullptr, *TpS = nullptr, *TpTS = nullptr;
  __nv_bfloat16 *JhS = nullptr, *JhST = nullptr, *JpS = nullptr;  // (cT), cut on demand
  bool has_j = false;
  int eT = 0;
  double unit = 1.0, unit_j = 1.0;
  float *wglobal = nullptr;
  size_t wglobal_floats = 0;
  int *d_status = nullptr;
  int stage_cap = 0;  // operand ring depth limit (0 = as many as fit)
  bool w_global = false;
  int variant = 0;    // 2: transposed kernel where eligible
  int bits = 8;       // digit radix 2^bits: 8 = BF16 slices, 11 = FP16 slices
  double2 *tri_ef = nullptr;  // per-triple denominator part and weight
  int tri_n = 0;
  unsigned long long *d_prof = nullptr;  // role profile of the last profiled launch
  SplitMaps maps;
};

void free_impl(SplitImpl *p) {
  if (!p) return;
  cudaFree(p->TaS);
  cudaFree(p->TaST);
  cudaFree(p->VhS);
  cudaFree(p->VhST);
  cudaFree(p->VpS);
  cudaFree(p->TpS);
  cudaFree(p->TpTS);
  cudaFree(p->JhS);
  cudaFree(p->JhST);
  cudaFree(p->JpS);
  cudaFree(p->wglobal);
  cudaFree(p->d_status);
  cudaFree(p->tri_ef);
  cudaFree(p->d_prof);
  delete p;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 5-D BF16 tensor map: dims[0] fastest (K, padded: the row pitch),
// 128-byte swizzle.  kext (if nonzero) is the K extent the map declares:
// the zero padding between kext and the pitch is then filled by TMA
// instead of being read from memory.
int make_map(CUtensorMap *m, const void *base, const uint64_t dims[5], const uint32_t box[5],
             uint64_t kext = 0) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled not available from the driver");
    return ATRIP_ERR_CUDA;
  }
  uint64_t strides[4];
  uint64_t s = dims[0] * 2;
  for (int i = 0; i < 4; ++i) {
    strides[i] = s;
    s *= dims[i + 1];
  }
  const uint32_t estr[5] = {1, 1, 1, 1, 1};
  const uint64_t ext[5] = {kext ? kext : dims[0], dims[1], dims[2], dims[3], dims[4]};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(base), ext, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r));
    return ATRIP_ERR_CUDA;
  }
  return ATRIP_OK;
}

int exponent_of(double maxabs) {
  if (!(maxabs > 0.0)) return 0;
  return std::ilogb(maxabs) + 1;  // maxabs < 2^e
}

int absmax(const double *x, int64_t n, unsigned long long *d_tmp, cudaStream_t st, double *out) {
  ATRIP_CUDA_TRY(cudaMemsetAsync(d_tmp, 0, sizeof(unsigned long long), st));
  if (n > 0) {
    absmax_kernel<<<152 * 8, 256, 0, st>>>(x, n, d_tmp);
    ATRIP_CUDA_TRY(cudaGetLastError());
  }
  unsigned long long h = 0;
  ATRIP_CUDA_TRY(cudaMemcpyAsync(&h, d_tmp, sizeof(h), cudaMemcpyDeviceToHost, st));
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  double v;
  std::memcpy(&v, &h, sizeof(v));
  *out = v;
  return ATRIP_OK;
}

int run_slices(SliceJob j, cudaStream_t st) {
  int64_t blocks = (j.nrows * j.Kp + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  slice_kernel<<<(int)blocks, 256, 0, st>>>(j);
  return cudaGetLastError() == cudaSuccess ? ATRIP_OK : ATRIP_ERR_CUDA;
}

int prepare(SplitImpl *p, const DeviceTensors &dt, int No, int Nv, int S, int bits,
            cudaStream_t st, int64_t *launches) {
  p->S = S;
  p->bits = bits;
  p->No = No;
  p->Nv = Nv;
  p->Ep = (Nv + kKChunk - 1) / kKChunk * kKChunk;
  const int64_t No2 = (int64_t)No * No, Ep = p->Ep;
  unsigned long long *d_tmp = nullptr;
  ATRIP_CUDA_TRY(cudaMalloc(&d_tmp, sizeof(unsigned long long)));
  double mT = 0, mVp = 0, mVh = 0;
  int rc = absmax(dt.Ta, (int64_t)Nv * No2 * Nv, d_tmp, st, &mT);
  if (rc == ATRIP_OK) rc = absmax(dt.Vpt, (int64_t)Nv * Nv * No * Nv, d_tmp, st, &mVp);
  if (rc == ATRIP_OK) rc = absmax(dt.Vht, (int64_t)Nv * No2 * No, d_tmp, st, &mVh);
  cudaFree(d_tmp);
  if (rc != ATRIP_OK) return rc;
  *launches += 3;
  const int eT = exponent_of(mT), eV = exponent_of(mVp > mVh ? mVp : mVh);
  p->eT = eT;
  // x = 2^(e-bits+1) sum_s q_s 2^(-bits s): level-0 products carry
  // 2^(eT+eV-2(bits-1))
  p->unit = std::ldexp(1.0, eT + eV - 2 * (bits - 1));
  const double sT = std::ldexp(1.0, bits - 1 - eT), sV = std::ldexp(1.0, bits - 1 - eV);

  const size_t nTa = (size_t)S * Nv * No2 * Ep, nVh = (size_t)S * Nv * No2 * kHoleK,
               nVp = (size_t)S * Nv * Nv * No * Ep, nTp = (size_t)S * Nv * Nv * No * kHoleK;
  ATRIP_CUDA_TRY(cudaMalloc(&p->TaS, 2 * nTa));
  ATRIP_CUDA_TRY(cudaMalloc(&p->TaST, 2 * nTa));
  ATRIP_CUDA_TRY(cudaMalloc(&p->VhS, 2 * nVh));
  ATRIP_CUDA_TRY(cudaMalloc(&p->VhST, 2 * nVh));
  ATRIP_CUDA_TRY(cudaMalloc(&p->VpS, 2 * nVp));
  ATRIP_CUDA_TRY(cudaMalloc(&p->TpS, 2 * nTp));
  ATRIP_CUDA_TRY(cudaMalloc(&p->TpTS, 2 * nTp));
  ATRIP_CUDA_TRY(cudaMalloc(&p->d_status, sizeof(int)));

  // rows (o, r1, r2) and source strides of each slice tensor
  SliceJob j;
  j.S = S;
  j.bits = bits;
  j.sign = 1.0;
  // TaS[s][x][q][p][E] = T[x,E,p,q] from Ta[x][q][p][E]
  j.src = dt.Ta; j.dst = p->TaS; j.nrows = Nv * No2; j.n1 = No; j.n2 = No;
  j.so = No2 * Nv; j.s1 = No * Nv; j.s2 = Nv; j.sk = 1; j.K = Nv; j.Kp = (int)Ep; j.scale = sT;
  if ((rc = run_slices(j, st))) return rc;
  // TaST[s][x][p][q][E]: rows with q fastest
  j.dst = p->TaST; j.s1 = Nv; j.s2 = No * Nv;
  if ((rc = run_slices(j, st))) return rc;
  // VhS[s][w][q][p][L] = Vh[p,q,L,w] from Vht[w][q][p][L]
  j.src = dt.Vht; j.dst = p->VhS; j.nrows = Nv * No2; j.n1 = No; j.n2 = No;
  j.so = No2 * No; j.s1 = No2; j.s2 = No; j.sk = 1; j.K = No; j.Kp = kHoleK; j.scale = sV;
  if ((rc = run_slices(j, st))) return rc;
  j.dst = p->VhST; j.s1 = No; j.s2 = No2;
  if ((rc = run_slices(j, st))) return rc;
  // VpS[s][y][z][r][E] = Vp[y,z,E,r] from Vpt[y][z][r][E]
  j.src = dt.Vpt; j.dst = p->VpS; j.nrows = (int64_t)Nv * Nv * No; j.n1 = Nv; j.n2 = No;
  j.so = (int64_t)Nv * No * Nv; j.s1 = (int64_t)No * Nv; j.s2 = Nv; j.sk = 1; j.K = Nv;
  j.Kp = (int)Ep; j.scale = sV;
  if ((rc = run_slices(j, st))) return rc;
  // TpS[s][u][v][r][L] = -T[u,v,L,r] = -Tp[u][v][r][L]
  j.src = dt.Tp; j.dst = p->TpS; j.nrows = (int64_t)Nv * Nv * No; j.n1 = Nv; j.n2 = No;
  j.so = (int64_t)Nv * No2; j.s1 = No2; j.s2 = No; j.sk = 1; j.K = No; j.Kp = kHoleK;
  j.scale = sT; j.sign = -1.0;
  if ((rc = run_slices(j, st))) return rc;
  // TpTS[s][u][v][r][L] = -T[u,v,r,L] = -Tp[u][v][L][r]
  j.dst = p->TpTS; j.s2 = 1; j.sk = No;
  if ((rc = run_slices(j, st))) return rc;
  *launches += 7;
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));

  // tensor maps (all 5-D, K-dim fastest); boxes: A (64, No, jt), B (64, NP)
  const int jt = 128 / No;
  const int NP = No <= 16 ? 16 : No <= 32 ? 32 : No <= 48 ? 48 : 64;
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt, 1, 1};
    if ((rc = make_map(&p->maps.TaN, p->TaS, d, box, (uint64_t)Nv))) return rc;
    if ((rc = make_map(&p->maps.TaT, p->TaST, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt, 1, 1};
    if ((rc = make_map(&p->maps.VhN, p->VhS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.VhT, p->VhST, d, box, (uint64_t)No))) return rc;
  }
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)NP, 1, 1, 1};
    if ((rc = make_map(&p->maps.Vp, p->VpS, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)NP, 1, 1, 1};
    if ((rc = make_map(&p->maps.TpN, p->TpS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.TpT, p->TpTS, d, box, (uint64_t)No))) return rc;
  }
  // transposed variant: (p,q)-row boxes of jt2 row groups, r-column boxes
  // of all S slices (loaded from slice -sa, the rows below 0 read as zeros)
  const int jt2 = 256 / No;
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt2, 1, 1};
    if ((rc = make_map(&p->maps.TaN2, p->TaS, d, box, (uint64_t)Nv))) return rc;
    if ((rc = make_map(&p->maps.TaT2, p->TaST, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt2, 1, 1};
    if ((rc = make_map(&p->maps.VhN2, p->VhS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.VhT2, p->VhST, d, box, (uint64_t)No))) return rc;
  }
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)S};
    if ((rc = make_map(&p->maps.Vp2, p->VpS, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)S};
    if ((rc = make_map(&p->maps.TpN2, p->TpS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.TpT2, p->TpTS, d, box, (uint64_t)No))) return rc;
  }
  // shared M stacks: 2S-1 slices from slice -(S-1)
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)(2 * S - 1)};
    if ((rc = make_map(&p->maps.Vp3, p->VpS, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)(2 * S - 1)};
    if ((rc = make_map(&p->maps.TpN3, p->TpS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.TpT3, p->TpTS, d, box, (uint64_t)No))) return rc;
  }
  p->maps.JhN = p->maps.VhN;
  p->maps.JhT = p->maps.VhT;
  p->maps.Jp = p->maps.Vp;
  p->maps.JhN2 = p->maps.VhN2;
  p->maps.JhT2 = p->maps.VhT2;
  p->maps.Jp2 = p->maps.Vp2;
  p->maps.Jp3 = p->maps.Vp3;
  return ATRIP_OK;
}

// Digit slices and maps of the (cT) intermediates, with their own scale.
int prepare_j(SplitImpl *p, const DeviceTensors &dt, cudaStream_t st, int64_t *launches) {
  const int No = p->No, Nv = p->Nv, S = p->S;
  const int64_t No2 = (int64_t)No * No, Ep = p->Ep;
  unsigned long long *d_tmp = nullptr;
  ATRIP_CUDA_TRY(cudaMalloc(&d_tmp, sizeof(unsigned long long)));
  double mJp = 0, mJh = 0;
  int rc = absmax(dt.Jpt, (int64_t)Nv * Nv * No * Nv, d_tmp, st, &mJp);
  if (rc == ATRIP_OK) rc = absmax(dt.Jht, (int64_t)Nv * No2 * No, d_tmp, st, &mJh);
  cudaFree(d_tmp);
  if (rc != ATRIP_OK) return rc;
  *launches += 2;
  const int eJ = exponent_of(mJp > mJh ? mJp : mJh);
  p->unit_j = std::ldexp(1.0, p->eT + eJ - 2 * (p->bits - 1));
  const double sJ = std::ldexp(1.0, p->bits - 1 - eJ);
  const size_t nVh = (size_t)S * Nv * No2 * kHoleK, nVp = (size_t)S * Nv * Nv * No * Ep;
  ATRIP_CUDA_TRY(cudaMalloc(&p->JhS, 2 * nVh));
  ATRIP_CUDA_TRY(cudaMalloc(&p->JhST, 2 * nVh));
  ATRIP_CUDA_TRY(cudaMalloc(&p->JpS, 2 * nVp));
  SliceJob j;
  j.S = S;
  j.bits = p->bits;
  j.sign = 1.0;
  j.src = dt.Jht; j.dst = p->JhS; j.nrows = Nv * No2; j.n1 = No; j.n2 = No;
  j.so = No2 * No; j.s1 = No2; j.s2 = No; j.sk = 1; j.K = No; j.Kp = kHoleK; j.scale = sJ;
  if ((rc = run_slices(j, st))) return rc;
  j.dst = p->JhST; j.s1 = No; j.s2 = No2;
  if ((rc = run_slices(j, st))) return rc;
  j.src = dt.Jpt; j.dst = p->JpS; j.nrows = (int64_t)Nv * Nv * No; j.n1 = Nv; j.n2 = No;
  j.so = (int64_t)Nv * No * Nv; j.s1 = (int64_t)No * Nv; j.s2 = Nv; j.sk = 1; j.K = Nv;
  j.Kp = (int)Ep; j.scale = sJ;
  if ((rc = run_slices(j, st))) return rc;
  *launches += 3;
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  const int jt = 128 / No;
  const int NP = No <= 16 ? 16 : No <= 32 ? 32 : No <= 48 ? 48 : 64;
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt, 1, 1};
    if ((rc = make_map(&p->maps.JhN, p->JhS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.JhT, p->JhST, d, box, (uint64_t)No))) return rc;
  }
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)NP, 1, 1, 1};
    if ((rc = make_map(&p->maps.Jp, p->JpS, d, box, (uint64_t)Nv))) return rc;
  }
  const int jt2 = 256 / No;
  {
    const uint64_t d[5] = {kHoleK, (uint64_t)No, (uint64_t)No, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, (uint32_t)jt2, 1, 1};
    if ((rc = make_map(&p->maps.JhN2, p->JhS, d, box, (uint64_t)No))) return rc;
    if ((rc = make_map(&p->maps.JhT2, p->JhST, d, box, (uint64_t)No))) return rc;
  }
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)S};
    if ((rc = make_map(&p->maps.Jp2, p->JpS, d, box, (uint64_t)Nv))) return rc;
  }
  {
    const uint64_t d[5] = {(uint64_t)Ep, (uint64_t)No, (uint64_t)Nv, (uint64_t)Nv, (uint64_t)S};
    const uint32_t box[5] = {kKChunk, (uint32_t)No, 1, 1, (uint32_t)(2 * S - 1)};
    if ((rc = make_map(&p->maps.Jp3, p->JpS, d, box, (uint64_t)Nv))) return rc;
  }
  p->has_j = true;
  return ATRIP_OK;
}

template <int S, int NP, bool SPLIT0, bool WSMEM>
int launch_shape(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  using K = KernelShape<S, NP, SPLIT0>;
  const size_t No3 = (size_t)a.No * a.No * a.No;
  const size_t vsm_bytes = sizeof(double) * 3 * (size_t)a.No * a.No;
  size_t vbytes = sizeof(double) * (WSMEM ? No3 : 0);
  // the singles' blocks go to shared memory where three stages still fit
  const bool vsm = kSmemLimit - 1024 - kTailBytes - vbytes >= vsm_bytes + 3 * K::kStageBytes;
  if (vsm) vbytes += vsm_bytes;
  const size_t avail = kSmemLimit - 1024 - kTailBytes - vbytes;
  int nst = (int)(avail / K::kStageBytes);
  if (nst > kMaxStages) nst = kMaxStages;
  if (p->stage_cap >= 2 && nst > p->stage_cap) nst = p->stage_cap;
  if (nst < 2) {
    set_error("split form: shared memory too small for No=" + std::to_string(a.No));
    return ATRIP_ERR_UNSUPPORTED;
  }
  SplitArgs args = a;
  args.nstages = nst;
  args.stage_bytes = K::kStageBytes;
  args.b_off = kATileBytes;
  args.vsm = vsm ? 1 : 0;
  const size_t smem = 1024 + (size_t)nst * K::kStageBytes + kTailBytes + vbytes;
  auto kern = triples_split_kernel<S, NP, SPLIT0, WSMEM, false>;
  ATRIP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const int64_t n = a.t_end - a.t_begin;
  const int grid = (int)(n < sm_count ? n : sm_count);
  kern<<<grid, kThreads, smem, st>>>(p->maps, args);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}

template <int S, int NP>
int launch_np(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  const bool split0 = 2 * (a.Nv + a.No) > 1024;
  // the FP64 copy of W fits next to three operand stages up to No = 24
  const bool wsmem = a.No <= 24 && !p->w_global;
  if (wsmem)
    return split0 ? launch_shape<S, NP, true, true>(p, a, sm_count, st)
                  : launch_shape<S, NP, false, true>(p, a, sm_count, st);
  return split0 ? launch_shape<S, NP, true, false>(p, a, sm_count, st)
                : launch_shape<S, NP, false, false>(p, a, sm_count, st);
}

// Transposed variant (S No <= 128, K = 2 (Nv + No) <= 1024).  The FP64 copy
// of W goes to shared memory when at least three operand stages still fit.
// One shared M slot: (S-1) No + 128 rows of 128 bytes (the MMA of slice
// unit sa reads 128 rows from row (S-1-sa) No), on 1024-byte atoms.
size_t mslot_bytes_for(int S, int No) {
  return ((size_t)((S - 1) * No + 128) * 128 + 1023) / 1024 * 1024;
}

// Epilogue staging of the transposed kernel: the S No level rows of one
// 64-column round (rows past them are never read).
size_t staging_bytes_t(int S, int No) {
  return ((size_t)S * No * kStagePitch * 4 + 15) / 16 * 16;
}

// One ring stage of the transposed kernel: the M-side stack (S No rows,
// rounded to a 1024-byte swizzle atom) followed directly by the N-side tile
// (nmma rows).  The MMA reads 128 stack rows; the rows past S No are the
// first rows of the N-side tile, which only feed accumulator rows the
// epilogue never reads.  A stage is at least those 128 rows (16 KB).  With
// the stacks in their own slots (MSHARE) a stage is the N-side tile alone.
struct TStage {
  size_t bytes, b_off;
};
TStage t_stage(int S, int No, bool mshare) {
  const int jt2 = 256 / No;
  const size_t b = (size_t)((No * jt2 + 15) / 16 * 16) * 128;  // nmma rows, 2 KB multiple
  if (mshare) return {b, 0};
  const size_t a = ((size_t)S * No * 128 + 1023) / 1024 * 1024;
  return {a + b < 16384 ? 16384 : a + b, a};
}

template <int S, bool WSMEM, bool MSHARE, bool F16>
int launch_shape_t(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  const TStage ts = t_stage(S, a.No, MSHARE);
  const size_t No3 = (size_t)a.No * a.No * a.No;
  const size_t mslots = MSHARE ? kMSlots * mslot_bytes_for(S, a.No) : 0;
  const size_t vsm_bytes = sizeof(double) * 3 * (size_t)a.No * a.No;
  size_t vbytes = sizeof(double) * (WSMEM ? No3 : 0) + staging_bytes_t(S, a.No) + mslots;
  // the singles' blocks go to shared memory where three stages still fit
  // beside them (at No = 56 they would leave two)
  const bool vsm = kSmemLimit - 1024 - kTailBytes - vbytes >= vsm_bytes + 3 * ts.bytes;
  if (vsm) vbytes += vsm_bytes;
  const size_t avail = kSmemLimit - 1024 - kTailBytes - vbytes;
  int nst = (int)(avail / ts.bytes);
  if (nst > kMaxStages) nst = kMaxStages;
  if (p->stage_cap >= 2 && nst > p->stage_cap) nst = p->stage_cap;
  if (nst < 2) {
    set_error("split form (transposed): shared memory too small for No=" + std::to_string(a.No));
    return ATRIP_ERR_UNSUPPORTED;
  }
  SplitArgs args = a;
  args.nstages = nst;
  args.mslot_bytes = MSHARE ? (int)mslot_bytes_for(S, a.No) : 0;
  args.stage_bytes = (int)ts.bytes;
  args.b_off = (int)ts.b_off;
  args.vsm = vsm ? 1 : 0;
  const size_t smem = 1024 + (size_t)nst * ts.bytes + kTailBytes + vbytes;
  auto kern = triples_split_kernel<S, 16, false, WSMEM, true, MSHARE, F16>;
  if (a.prof) {
    // the role profile is built for the two-slice transposed kernel only
    if constexpr (S == 2 && !MSHARE) {
      kern = triples_split_kernel<S, 16, false, WSMEM, true, false, F16, false, true>;
    } else {
      set_error("split form: the role profile needs 2 slices and the transposed kernel (variant 2)");
      return ATRIP_ERR_UNSUPPORTED;
    }
  }
  ATRIP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const int64_t n = a.t_end - a.t_begin;
  const int grid = (int)(n < sm_count ? n : sm_count);
  kern<<<grid, kThreads, smem, st>>>(p->maps, args);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}

// S slices of No rows fit the 128 M rows, level 0 stays exact (BF16
// digits, K = 2 (Nv + No) <= 1024) or within int32 (FP16 digits, K < 2048),
// and two operand stages fit next to the epilogue staging.
bool transposed_eligible(int S, int No, int Nv, bool f16 = false) {
  if (S * No > 128 || 2 * (Nv + No) > (f16 ? 2047 : 1024)) return false;
  const size_t fixed = 1024 + kTailBytes + staging_bytes_t(S, No);
  return fixed + 2 * t_stage(S, No, false).bytes <= (size_t)kSmemLimit;
}

template <int S, bool F16>
int launch_t(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  const size_t No3 = (size_t)a.No * a.No * a.No;
  const size_t fixed =
      1024 + kTailBytes + staging_bytes_t(S, a.No);
  // variant 3: one M stack per K chunk shared by the S slice units, where
  // its row blocks start on swizzle atoms (No % 8 == 0) and 2 ring stages fit
  if (p->variant == 3 && a.No % 8 == 0 &&
      fixed + kMSlots * mslot_bytes_for(S, a.No) + 2 * t_stage(S, a.No, true).bytes <=
          (size_t)kSmemLimit)
    return launch_shape_t<S, false, true, F16>(p, a, sm_count, st);
  const bool wsmem = !p->w_global && fixed + sizeof(double) * No3 +
                                         3 * t_stage(S, a.No, false).bytes <=
                                         (size_t)kSmemLimit;
  return wsmem ? launch_shape_t<S, true, false, F16>(p, a, sm_count, st)
               : launch_shape_t<S, false, false, F16>(p, a, sm_count, st);
}

// FP16 digits: the transposed kernel only (variant 3 where chosen).
int launch_f16(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  if (p->S != 2 || !transposed_eligible(2, a.No, a.Nv, true)) {
    set_error("split FP16 form: needs 2 slices, No <= 64 and 2 (Nv + No) < 2048 (No=" +
              std::to_string(a.No) + ", Nv=" + std::to_string(a.Nv) + ")");
    return ATRIP_ERR_UNSUPPORTED;
  }
  return launch_t<2, true>(p, a, sm_count, st);
}

template <int S>
int launch_s(SplitImpl *p, const SplitArgs &a, int sm_count, cudaStream_t st) {
  if (p->variant >= 2 && transposed_eligible(S, a.No, a.Nv))
    return launch_t<S, false>(p, a, sm_count, st);
  if (a.prof) {
    set_error("split form: the role profile needs 2 slices and the transposed kernel (variant 2)");
    return ATRIP_ERR_UNSUPPORTED;
  }
  const int No = a.No;
  if (No <= 16) return launch_np<S, 16>(p, a, sm_count, st);
  if (No <= 32) return launch_np<S, 32>(p, a, sm_count, st);
  if (No <= 48) return launch_np<S, 48>(p, a, sm_count, st);
  return launch_np<S, 64>(p, a, sm_count, st);
}

// Multi-system launch of the transposed kernel, layout of the largest system.
template <int S, bool WSMEM, bool F16>
int launch_multi(const SplitMultiBuffers &b, const SplitArgs &a, int grid, cudaStream_t st) {
  auto kern = triples_split_kernel<S, 16, false, WSMEM, true, false, F16, true>;
  ATRIP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)b.smem));
  SplitMaps none;
  std::memset(&none, 0, sizeof(none));
  kern<<<grid, kThreads, b.smem, st>>>(none, a);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}

template <int S>
int launch_multi_s(const SplitMultiBuffers &b, const SplitArgs &a, int grid, cudaStream_t st) {
  if (b.f16) return b.wsmem ? launch_multi<S, true, true>(b, a, grid, st)
                            : launch_multi<S, false, true>(b, a, grid, st);
  return b.wsmem ? launch_multi<S, true, false>(b, a, grid, st)
                 : launch_multi<S, false, false>(b, a, grid, st);
}

}  // namespace

void split_multi_free(SplitMultiBuffers &b) {
  cudaFreeHost(b.h_desc);
  cudaFree(b.d_desc);
  cudaFreeHost(b.h_prefix);
  cudaFree(b.d_prefix);
  cudaFree(b.wglobal);
  cudaFree(b.d_status);
  cudaFree(b.d_queue);
  b = SplitMultiBuffers();
}

int split_multi_prepare(const SplitMultiSystem *sys, int n, int slices, bool f16, int sm_count,
                        SplitMultiBuffers &b) {
  if (n < 1 || slices < 2 || slices > 4 || (f16 && slices != 2)) return ATRIP_ERR_UNSUPPORTED;
  int no_lay = 0, npass = 1;
  size_t stage = 0;
  for (int k = 0; k < n; ++k) {
    const SplitMultiSystem &m = sys[k];
    auto *p = static_cast<SplitImpl *>(m.state->impl);
    if (!m.state->valid || !p || p->S != slices || p->bits != (f16 ? 11 : 8) ||
        (m.use_j && !p->has_j) || p->tri_n != m.n_triples ||
        !transposed_eligible(slices, m.No, m.Nv, f16))
      return ATRIP_ERR_UNSUPPORTED;
    no_lay = std::max(no_lay, m.No);
    if (m.use_j) npass = 2;
    stage = std::max(stage, t_stage(slices, m.No, false).bytes);
  }
  const size_t L3 = (size_t)no_lay * no_lay * no_lay;
  const size_t fixed = 1024 + kTailBytes + staging_bytes_t(slices, no_lay);
  const bool wsmem = fixed + sizeof(double) * L3 + 3 * stage <= (size_t)kSmemLimit;
  size_t vfix = fixed + (wsmem ? sizeof(double) * L3 : 0);
  const size_t vsm_bytes = sizeof(double) * 3 * (size_t)no_lay * no_lay;
  const bool vsm = vfix + vsm_bytes + 3 * stage <= (size_t)kSmemLimit;
  if (vsm) vfix += vsm_bytes;
  if (vfix >= (size_t)kSmemLimit) return ATRIP_ERR_UNSUPPORTED;
  int nst = (int)(((size_t)kSmemLimit - vfix) / stage);
  if (nst > kMaxStages) nst = kMaxStages;
  if (nst < 2) return ATRIP_ERR_UNSUPPORTED;
  // buffers: descriptor tables, prefix sums, W cells of the largest system
  if (b.cap < n) {
    cudaFreeHost(b.h_desc);
    cudaFree(b.d_desc);
    cudaFreeHost(b.h_prefix);
    cudaFree(b.d_prefix);
    b.h_desc = b.d_desc = nullptr;
    b.h_prefix = b.d_prefix = nullptr;
    b.cap = 0;
    ATRIP_CUDA_TRY(cudaMallocHost(&b.h_desc, sizeof(SysDesc) * n));
    ATRIP_CUDA_TRY(cudaMalloc(&b.d_desc, sizeof(SysDesc) * n));
    ATRIP_CUDA_TRY(cudaMallocHost(&b.h_prefix, sizeof(int64_t) * (n + 1)));
    ATRIP_CUDA_TRY(cudaMalloc(&b.d_prefix, sizeof(int64_t) * (n + 1)));
    b.cap = n;
  }
  if (!b.d_status) ATRIP_CUDA_TRY(cudaMalloc(&b.d_status, sizeof(int)));
  if (!b.d_queue) ATRIP_CUDA_TRY(cudaMalloc(&b.d_queue, sizeof(unsigned long long)));
  const size_t need = (size_t)sm_count * 2 * npass * 3 * 2 * L3;  // floats
  if (need > b.wglobal_floats) {
    cudaFree(b.wglobal);
    b.wglobal = nullptr;
    b.wglobal_floats = 0;
    ATRIP_CUDA_TRY(cudaMalloc(&b.wglobal, sizeof(float) * need));
    b.wglobal_floats = need;
  }
  SysDesc *h = static_cast<SysDesc *>(b.h_desc);
  b.h_prefix[0] = 0;
  for (int k = 0; k < n; ++k) {
    const SplitMultiSystem &m = sys[k];
    auto *p = static_cast<SplitImpl *>(m.state->impl);
    SysDesc d;
    std::memset(&d, 0, sizeof(d));
    d.maps = p->maps;
    d.epsa = m.dt->epsa;
    d.tai = m.dt->tai;
    d.Vhh = m.dt->Vhh;
    d.tuples = m.tuples;
    d.triples = m.triples;
    d.tri_ef = p->tri_ef;
    d.e = m.e;
    d.ect = m.ect;
    d.unit = p->unit;
    d.unit_j = p->unit_j;
    d.t_begin = m.t_begin;
    d.No = m.No;
    d.Nv = m.Nv;
    d.jt2 = 256 / m.No;
    d.ntiles2 = (m.No + d.jt2 - 1) / d.jt2;
    d.nmma = (m.No * d.jt2 + 15) / 16 * 16;
    d.kch = p->Ep / kKChunk;
    d.b_off = (int)t_stage(slices, m.No, false).b_off;
    d.n_triples = m.n_triples;
    d.use_j = m.use_j ? 1 : 0;
    h[k] = d;
    b.h_prefix[k + 1] = b.h_prefix[k] + std::max<int64_t>(0, m.t_end - m.t_begin);
  }
  b.n = n;
  b.slices = slices;
  b.f16 = f16 ? 1 : 0;
  b.no_lay = no_lay;
  b.npass_lay = npass;
  b.nstages = nst;
  b.wsmem = wsmem ? 1 : 0;
  b.vsm = vsm ? 1 : 0;
  b.stage_bytes = stage;
  b.smem = vfix + (size_t)nst * stage;
  return ATRIP_OK;
}

int split_multi_enqueue(const SplitMultiBuffers &b, double tai_sign, int sm_count,
                        cudaStream_t st, int64_t *launches) {
  if (b.n < 1) {
    set_error("split form: multi-system launch not prepared");
    return ATRIP_ERR_STATE;
  }
  ATRIP_CUDA_TRY(cudaMemcpyAsync(b.d_desc, b.h_desc, sizeof(SysDesc) * b.n,
                                 cudaMemcpyHostToDevice, st));
  ATRIP_CUDA_TRY(cudaMemcpyAsync(b.d_prefix, b.h_prefix, sizeof(int64_t) * (b.n + 1),
                                 cudaMemcpyHostToDevice, st));
  ATRIP_CUDA_TRY(cudaMemsetAsync(b.d_queue, 0, sizeof(unsigned long long), st));
  ATRIP_CUDA_TRY(cudaMemsetAsync(b.d_status, 0, sizeof(int), st));
  const int64_t total = b.h_prefix[b.n];
  if (total == 0) return ATRIP_OK;
  SplitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.No = b.no_lay;
  a.nstages = b.nstages;
  a.stage_bytes = (int)b.stage_bytes;
  a.tai_sign = tai_sign;
  a.queue = b.d_queue;
  a.status = b.d_status;
  a.wglobal = b.wglobal;
  a.wait_cycles = kWaitCycles;
  a.sys = static_cast<const SysDesc *>(b.d_desc);
  a.prefix = b.d_prefix;
  a.nsys = b.n;
  a.no_lay = b.no_lay;
  a.npass_lay = b.npass_lay;
  a.vsm = b.vsm;
  const int grid = (int)std::min<int64_t>(total, sm_count);
  int rc;
  switch (b.slices) {
    case 2: rc = launch_multi_s<2>(b, a, grid, st); break;
    case 3: rc = launch_multi_s<3>(b, a, grid, st); break;
    default: rc = launch_multi_s<4>(b, a, grid, st); break;
  }
  if (rc != ATRIP_OK) return rc;
  *launches += 1;
  return ATRIP_OK;
}

int split_profile_read(const SplitState &s, unsigned long long *out, int n) {
  auto *p = static_cast<const SplitImpl *>(s.impl);
  if (!p || !p->d_prof) {
    set_error("split form: no profiled run on this context");
    return ATRIP_ERR_STATE;
  }
  ATRIP_CUDA_TRY(cudaMemcpy(out, p->d_prof, sizeof(unsigned long long) * std::min(n, (int)kProfSlots),
                            cudaMemcpyDeviceToHost));
  return ATRIP_OK;
}

void split_invalidate(SplitState &s) { s.valid = false; }

void split_free(SplitState &s) {
  free_impl(static_cast<SplitImpl *>(s.impl));
  s.impl = nullptr;
  s.valid = false;
  s.generation++;
}

int split_prepare(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
                  bool use_j, int slices, const uint32_t *triples, int n_triples,
                  cudaStream_t st, int64_t *launches) {
  if (slices < 2 || slices > 4) {
    set_error("split form: slices must be 2, 3 or 4");
    return ATRIP_ERR_ARGUMENT;
  }
  const int bits = s.f16 ? 11 : 8;
  if (s.f16 && slices != 2) {
    set_error("split FP16 form: slices must be 2");
    return ATRIP_ERR_ARGUMENT;
  }
  if (!s.valid || s.slices != slices || !s.impl ||
      static_cast<SplitImpl *>(s.impl)->bits != bits) {
    split_free(s);
    auto *p = new SplitImpl();
    s.impl = p;
    int rc = prepare(p, dt, No, Nv, slices, bits, st, launches);
    if (rc == ATRIP_OK && n_triples > 0) {
      if (cudaMalloc(&p->tri_ef, sizeof(double2) * n_triples) != cudaSuccess) {
        set_error("split form: allocating the triple table failed");
        rc = ATRIP_ERR_CUDA;
      } else {
        triple_table_kernel<<<(n_triples + 255) / 256, 256, 0, st>>>(triples, n_triples,
                                                                     dt.epsi, p->tri_ef);
        rc = cudaGetLastError() == cudaSuccess ? ATRIP_OK : ATRIP_ERR_CUDA;
        p->tri_n = n_triples;
        *launches += 1;
      }
    }
    if (rc != ATRIP_OK) {
      split_free(s);
      return rc;
    }
    s.valid = true;
    s.slices = slices;
  }
  auto *p = static_cast<SplitImpl *>(s.impl);
  if (use_j && !p->has_j) {
    s.generation++;
    const int rc = prepare_j(p, dt, st, launches);
    if (rc != ATRIP_OK) return rc;
  }
  // W buffers (one double per element): two tuple parities x passes per CTA
  const size_t need = (size_t)sm_count * 2 * (use_j ? 2 : 1) * 3 * 2 * No * No * No;  // floats
  if (need > p->wglobal_floats) {
    s.generation++;
    cudaFree(p->wglobal);
    p->wglobal = nullptr;
    ATRIP_CUDA_TRY(cudaMalloc(&p->wglobal, sizeof(float) * need));
    p->wglobal_floats = need;
  }
  return ATRIP_OK;
}

int split_enqueue(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
                  const uint32_t *tuples, const uint32_t *triples, int n_triples, int64_t t_begin,
                  int64_t t_end, const uint32_t *order, double tai_sign, bool use_j,
                  unsigned long long *queue, double *e, double *ect, cudaStream_t st,
                  int64_t *launches) {
  auto *p = static_cast<SplitImpl *>(s.impl);
  if (!s.valid || !p || (use_j && !p->has_j)) {
    set_error("split form: operands not prepared");
    return ATRIP_ERR_STATE;
  }
  const size_t need = (size_t)sm_count * 2 * (use_j ? 2 : 1) * 3 * 2 * No * No * No;
  if (need > p->wglobal_floats) {
    set_error("split form: W buffers prepared for fewer CTAs");
    return ATRIP_ERR_STATE;
  }
  if (p->tri_n != n_triples) {
    set_error("split form: triple table prepared for another list");
    return ATRIP_ERR_STATE;
  }
  p->stage_cap = s.stage_cap;
  p->w_global = s.w_global;
  p->variant = s.variant;
  // no clearing of the W buffers: every cell a tuple's energy reads is
  // stored by that tuple's groups before the energy warps get it
  ATRIP_CUDA_TRY(cudaMemsetAsync(p->d_status, 0, sizeof(int), st));
  SplitArgs a;
  a.prof = nullptr;
  if (s.profile) {
    if (!p->d_prof)
      ATRIP_CUDA_TRY(cudaMalloc(&p->d_prof, sizeof(unsigned long long) * kProfSlots));
    ATRIP_CUDA_TRY(cudaMemsetAsync(p->d_prof, 0, sizeof(unsigned long long) * kProfSlots, st));
    a.prof = p->d_prof;
  }
  a.No = No;
  a.Nv = Nv;
  a.jt = 128 / No;
  a.ntiles = (No + a.jt - 1) / a.jt;
  a.prefetch = s.prefetch ? 1 : 0;
  a.unpublished = s.unpublished ? 1 : 0;
  a.sys = nullptr;
  a.prefix = nullptr;
  a.nsys = 0;
  a.no_lay = No;
  a.npass_lay = use_j ? 2 : 1;
  a.wait_cycles = s.wait_cycles > 0 ? s.wait_cycles : kWaitCycles;
  a.jt2 = 256 / No;
  a.ntiles2 = (No + a.jt2 - 1) / a.jt2;
  a.nmma = (No * a.jt2 + 15) / 16 * 16;
  a.kch = p->Ep / kKChunk;
  a.epsi = dt.epsi;
  a.epsa = dt.epsa;
  a.tai = dt.tai;
  a.Vhh = dt.Vhh;
  a.tuples = tuples;
  a.triples = triples;
  a.tri_ef = p->tri_ef;
  a.n_triples = n_triples;
  a.t_begin = t_begin;
  a.t_end = t_end;
  a.order = order;
  a.queue = queue;
  a.tai_sign = tai_sign;
  a.unit = p->unit;
  a.unit_j = p->unit_j;
  a.use_j = use_j ? 1 : 0;
  a.e = e;
  a.ect = ect;
  a.status = p->d_status;
  a.wglobal = p->wglobal;
  int rc;
  if (p->bits == 11) {
    rc = launch_f16(p, a, sm_count, st);
    if (rc != ATRIP_OK) return rc;
    *launches += 1;
    return ATRIP_OK;
  }
  switch (s.slices) {
    case 2: rc = launch_s<2>(p, a, sm_count, st); break;
    case 3: rc = launch_s<3>(p, a, sm_count, st); break;
    default: rc = launch_s<4>(p, a, sm_count, st); break;
  }
  if (rc != ATRIP_OK) return rc;
  *launches += 1;
  return ATRIP_OK;
}

const int *split_status_ptr(const SplitState &s) {
  auto *p = static_cast<SplitImpl *>(s.impl);
  return p ? p->d_status : nullptr;
}

int split_status_check(int status) {
  if (status != 0) {
    set_error("split kernel: a bounded wait gave up (code " + std::to_string(status) + ")");
    return ATRIP_ERR_TIMEOUT;
  }
  return ATRIP_OK;
}

int split_run(SplitState &s, const DeviceTensors &dt, int No, int Nv, int sm_count,
              const uint32_t *tuples, const uint32_t *triples, int n_triples, int64_t t_begin,
              int64_t t_end, const uint32_t *order, double tai_sign, bool use_j, int slices,
              unsigned long long *queue, double *e, double *ect, cudaStream_t st,
              int64_t *launches) {
  int rc = split_prepare(s, dt, No, Nv, sm_count, use_j, slices, triples, n_triples, st,
                         launches);
  if (rc != ATRIP_OK) return rc;
  rc = split_enqueue(s, dt, No, Nv, sm_count, tuples, triples, n_triples, t_begin, t_end, order,
                     tai_sign, use_j, queue, e, ect, st, launches);
  if (rc != ATRIP_OK) return rc;
  int status = 0;
  ATRIP_CUDA_TRY(cudaMemcpyAsync(&status, split_status_ptr(s), sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
  ATRIP_CUDA_TRY(cudaStreamSynchronize(st));
  return split_status_check(status);
}

}  // namespace atrip_gb300
