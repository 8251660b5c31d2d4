/*
 * CPU oracle for the CCSD(T) triples hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of atrip's per-(a,b,c) triples kernels, used by the
 * test-suite as the parity checker and by bench.py as the timed CPU
 * baseline.  Product code never calls it.  It is pinned against the atrip
 * reference's own sources compiled one-rank with shims (oracle/Makefile,
 * oracle/ref_harness.cxx) and against the committed fixtures in
 * tests/golden/, which that build produced.
 *
 * Input layout: column-major FP64 exactly as atrip's CTF tensors hand them
 * to read_all (first index fastest):
 *   epsi[No], epsa[Nv], Tai[a + i Nv], Tabij[a,b,i,j], Vabij[a,b,i,j],
 *   Vijka[i,j,k,a], Vabci[a,b,e,i] (+ optional Jijka, Jabci like V*).
 *
 * Two evaluation routes, which must agree with each other and with the
 * reference:
 *   - "naive": the BLAS-free loops of src/atrip/Equations.cxx:685-726,
 *     reading straight from the full tensors through the slice maps of
 *     src/atrip/Unions.hpp:77-278;
 *   - "port": the DGEMM route of src/atrip/Equations.cxx:492-684 (12 GEMMs
 *     into a buffer, each followed by a permuted accumulation), with the
 *     operand slices cut once up front as atrip's SliceUnion::init does.
 *     dgemm comes from an ILP64 OpenBLAS if one is registered
 *     (oracle_set_blas), otherwise from the loops in this file.
 * Tuples are split over pthreads in contiguous blocks, like atrip's NAIVE
 * distribution over ranks (src/atrip/Tuples.cxx:89-120).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int No, Nv;
  const double *epsi, *epsa, *Tai, *Tabij, *Vabij, *Vijka, *Vabci, *Jijka, *Jabci;
} oracle_inputs;

/* ------------------------------------------------------------------ tuples */

/* Number of a <= b <= c tuples without a == b == c (src/atrip/Tuples.cxx:93). */
int64_t oracle_n_tuples(int Nv) {
  const int64_t n = Nv;
  return n * (n + 1) * (n + 2) / 6 - n;
}

/* Lexicographic tuple list (src/atrip/Tuples.cxx:122-134). */
void oracle_tuple_list(int Nv, int32_t *abc) {
  int64_t u = 0;
  for (int a = 0; a < Nv; ++a)
    for (int b = a; b < Nv; ++b)
      for (int c = b; c < Nv; ++c) {
        if (a == b && b == c) continue;
        abc[3 * u + 0] = a;
        abc[3 * u + 1] = b;
        abc[3 * u + 2] = c;
        ++u;
      }
}

/* ----------------------------------------------------- naive-loop doubles */

/* Tijk for tuple (a,b,c); src/atrip/Equations.cxx:685-726 with the operand
 * slices read in place:
 *   TXphh[E + i Nv + j Nv No] = T[x,E,i,j]   (Unions.hpp:97-110)
 *   VhhhX[i + j No + k No^2]  = Vh[i,j,k,x]  (Unions.hpp:137-148)
 *   VXYph[E + k Nv]           = Vp[x,y,E,k]  (Unions.hpp:181-195)
 *   TXYhh[i + j No]           = T[x,y,i,j]   (Unions.hpp:261-276)   */
void oracle_doubles_naive(const oracle_inputs *in, int a, int b, int c,
                          const double *Vh, const double *Vp, double *Tijk) {
  const int64_t No = in->No, Nv = in->Nv, NoNo = No * No, NvNv = Nv * Nv;
  const double *T = in->Tabij;
#define TPH(x, e, i, j) T[(x) + (e) * Nv + (i) * NvNv + (j) * NvNv * No]
#define THH(x, y, i, j) T[(x) + (y) * Nv + (i) * NvNv + (j) * NvNv * No]
#define VHHH(i, j, k, x) Vh[(i) + (j) * No + (k) * NoNo + (x) * NoNo * No]
#define VPPH(x, y, e, k) Vp[(x) + (y) * Nv + (e) * NvNv + (k) * NvNv * Nv]
  for (int64_t k = 0; k < No; k++)
    for (int64_t j = 0; j < No; j++)
      for (int64_t i = 0; i < No; i++) {
        double t = 0.0;
        for (int64_t L = 0; L < No; L++) {
          t -= THH(a, b, L, j) * VHHH(i, k, L, c);
          t -= THH(a, b, i, L) * VHHH(j, k, L, c);
          t -= THH(a, c, L, k) * VHHH(i, j, L, b);
          t -= THH(a, c, i, L) * VHHH(k, j, L, b);
          t -= THH(b, c, L, k) * VHHH(j, i, L, a);
          t -= THH(b, c, j, L) * VHHH(k, i, L, a);
        }
        for (int64_t E = 0; E < Nv; E++) {
          t += TPH(a, E, i, j) * VPPH(b, c, E, k);
          t += TPH(a, E, i, k) * VPPH(c, b, E, j);
          t += TPH(c, E, k, i) * VPPH(a, b, E, j);
          t += TPH(c, E, k, j) * VPPH(b, a, E, i);
          t += TPH(b, E, j, i) * VPPH(a, c, E, k);
          t += TPH(b, E, j, k) * VPPH(c, a, E, i);
        }
        Tijk[i + j * No + k * NoNo] = t;
      }
#undef TPH
#undef THH
#undef VHHH
#undef VPPH
}

/* Z += t1 (x) Vpphh; src/atrip/Equations.cxx:387-426 (Tai possibly negated
 * for ijkabc, src/atrip/Atrip.cxx:183-187). */
void oracle_singles(const oracle_inputs *in, int a, int b, int c, const double *Tai,
                    double *Zijk) {
  const int64_t No = in->No, Nv = in->Nv, NoNo = No * No, NvNv = Nv * Nv;
  const double *V = in->Vabij;
#define VHH(x, y, i, j) V[(x) + (y) * Nv + (i) * NvNv + (j) * NvNv * No]
  for (int64_t k = 0; k < No; k++)
    for (int64_t i = 0; i < No; i++)
      for (int64_t j = 0; j < No; j++) {
        const int64_t ijk = i + j * No + k * NoNo;
        Zijk[ijk] += Tai[a + i * Nv] * VHH(b, c, j, k);
        Zijk[ijk] += Tai[b + j * Nv] * VHH(a, c, i, k);
        Zijk[ijk] += Tai[c + k * Nv] * VHH(a, b, i, j);
      }
#undef VHH
}

/* ------------------------------------------------------------------ energy */

/* get_energy_distinct, src/atrip/Equations.cxx:101-180 (ATRIP_NEW_ENERGY). */
double oracle_energy_distinct(double epsabc, int No_, const double *epsi,
                              const double *Tijk, const double *Zijk) {
  const int64_t No = No_, bs = 16;
  double energy = 0.0;
  for (int64_t kk = 0; kk < No; kk += bs) {
    const int64_t kend = kk + bs < No ? kk + bs : No;
    for (int64_t jj = kk; jj < No; jj += bs) {
      const int64_t jend = jj + bs < No ? jj + bs : No;
      for (int64_t ii = jj; ii < No; ii += bs) {
        const int64_t iend = ii + bs < No ? ii + bs : No;
        for (int64_t k = kk; k < kend; k++) {
          const double ek = epsi[k];
          for (int64_t j = (jj > k ? jj : k); j < jend; j++) {
            const double ej = epsi[j], facjk = j == k ? 0.5 : 1.0;
            for (int64_t i = (ii > j ? ii : j); i < iend; i++) {
              const double ei = epsi[i], facij = i == j ? 0.5 : 1.0;
              const double denominator = epsabc - ((ei + ej) + ek);
              const double U = Zijk[i + No * j + No * No * k], V = Zijk[i + No * k + No * No * j],
                           W = Zijk[j + No * i + No * No * k], X = Zijk[j + No * k + No * No * i],
                           Y = Zijk[k + No * i + No * No * j], Z = Zijk[k + No * j + No * No * i];
              const double A = Tijk[i + No * j + No * No * k], B = Tijk[i + No * k + No * No * j],
                           C = Tijk[j + No * i + No * No * k], D = Tijk[j + No * k + No * No * i],
                           E = Tijk[k + No * i + No * No * j], F = Tijk[k + No * j + No * No * i];
              const double UXY = U + (X + Y), VWZ = V + (W + Z), ADE = A + (D + E),
                           BCF = B + (C + F);
              const double first = A * U + (B * V + (C * W + (D * X + (E * Y + F * Z))));
              const double second = (UXY - 2.0 * VWZ) * ADE;
              const double third = (VWZ - 2.0 * UXY) * BCF;
              const double value = 3.0 * first + (second + third);
              energy += (2.0 * value / denominator) * (facjk * facij);
            }
          }
        }
      }
    }
  }
  return energy;
}

/* get_energy_same, src/atrip/Equations.cxx:182-238. */
double oracle_energy_same(double epsabc, int No_, const double *epsi, const double *Tijk,
                          const double *Zijk) {
  const int64_t No = No_, bs = 16;
  double energy = 0.0;
  for (int64_t kk = 0; kk < No; kk += bs) {
    const int64_t kend = kk + bs < No ? kk + bs : No;
    for (int64_t jj = kk; jj < No; jj += bs) {
      const int64_t jend = jj + bs < No ? jj + bs : No;
      for (int64_t ii = jj; ii < No; ii += bs) {
        const int64_t iend = ii + bs < No ? ii + bs : No;
        for (int64_t k = kk; k < kend; k++) {
          const double ek = epsi[k];
          for (int64_t j = (jj > k ? jj : k); j < jend; j++) {
            const double facjk = j == k ? 0.5 : 1.0, ej = epsi[j];
            for (int64_t i = (ii > j ? ii : j); i < iend; i++) {
              const double ei = epsi[i], facij = i == j ? 0.5 : 1.0;
              const double denominator = epsabc - ((ei + ej) + ek);
              const double U = Zijk[i + No * j + No * No * k], V = Zijk[j + No * k + No * No * i],
                           W = Zijk[k + No * i + No * No * j];
              const double A = Tijk[i + No * j + No * No * k], B = Tijk[j + No * k + No * No * i],
                           C = Tijk[k + No * i + No * No * j];
              const double value = 3.0 * ((A * U + B * V) + C * W) - (A + (B + C)) * (U + (V + W));
              energy += (2.0 * value / denominator) * (facjk * facij);
            }
          }
        }
      }
    }
  }
  return energy;
}

/* Classification of src/atrip/Atrip.cxx:640-642. */
static double tuple_energy(const oracle_inputs *in, int a, int b, int c, const double *T,
                           const double *Z) {
  int distinct = 0;
  if (a == b) distinct++;
  if (b == c) distinct--;
  const double epsabc = in->epsa[a] + in->epsa[b] + in->epsa[c];
  return distinct == 0 ? oracle_energy_distinct(epsabc, in->No, in->epsi, T, Z)
                       : oracle_energy_same(epsabc, in->No, in->epsi, T, Z);
}

/* -------------------------------------------------------------- dgemm hook */

typedef void (*dgemm64_fn)(const char *, const char *, const int64_t *, const int64_t *,
                           const int64_t *, const double *, const double *, const int64_t *,
                           const double *, const int64_t *, const double *, double *,
                           const int64_t *);
static dgemm64_fn g_dgemm64 = 0;

/* Register an ILP64 BLAS (e.g. numpy's bundled OpenBLAS).  Returns 1 if a
 * dgemm was found, 0 otherwise (the loops below are used then). */
int oracle_set_blas(const char *path, const char *dgemm_symbol, const char *threads_symbol) {
  void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 0;
  g_dgemm64 = (dgemm64_fn)dlsym(h, dgemm_symbol);
  if (threads_symbol && *threads_symbol) {
    void (*set_threads)(int) = (void (*)(int))dlsym(h, threads_symbol);
    if (set_threads) set_threads(1);
  }
  return g_dgemm64 != 0;
}

/* Column-major C(m x n) = alpha op(A) op(B) + beta C, loops for when no BLAS
 * was registered. */
static void dgemm_loops(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                        const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                        double *C, int64_t ldc) {
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < m; ++i) C[i + j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + j * ldc];
    for (int64_t l = 0; l < k; ++l) {
      const double bl = alpha * (tb == 'N' ? B[l + j * ldb] : B[j + l * ldb]);
      if (ta == 'N')
        for (int64_t i = 0; i < m; ++i) C[i + j * ldc] += A[i + l * lda] * bl;
      else
        for (int64_t i = 0; i < m; ++i) C[i + j * ldc] += A[l + i * lda] * bl;
    }
  }
}

static void xgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                  const double *A, int64_t lda, const double *B, int64_t ldb, double *C,
                  int64_t ldc) {
  const double beta = 0.0;
  if (g_dgemm64)
    g_dgemm64(&ta, &tb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc);
  else
    dgemm_loops(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

/* ------------------------------------------------------- DGEMM-route port */

/* Operand slices cut once, laid out as atrip's SliceUnion sources hold them
 * (src/atrip/Unions.hpp:77-278). */
typedef struct {
  int No, Nv;
  double *Ta;  /* [x][ E + i Nv + j Nv No ]  = T[x,E,i,j]  */
  double *Vp;  /* [x + y Nv][ E + k Nv ]     = Vp[x,y,E,k] */
  double *Jp;  /* same for Jabci (or NULL) */
  double *Tab; /* [x + y Nv][ i + j No ]     = T[x,y,i,j]  */
  double *Vab; /* [x + y Nv][ i + j No ]     = V[x,y,i,j]  */
} port_slices;

static void cut_slices(const oracle_inputs *in, port_slices *s) {
  const int64_t No = in->No, Nv = in->Nv, NvNv = Nv * Nv;
  s->No = in->No;
  s->Nv = in->Nv;
  s->Ta = (double *)malloc(sizeof(double) * Nv * Nv * No * No);
  s->Vp = (double *)malloc(sizeof(double) * Nv * Nv * Nv * No);
  s->Jp = in->Jabci ? (double *)malloc(sizeof(double) * Nv * Nv * Nv * No) : 0;
  s->Tab = (double *)malloc(sizeof(double) * Nv * Nv * No * No);
  s->Vab = (double *)malloc(sizeof(double) * Nv * Nv * No * No);
  for (int64_t j = 0; j < No; ++j)
    for (int64_t i = 0; i < No; ++i)
      for (int64_t e = 0; e < Nv; ++e)
        for (int64_t x = 0; x < Nv; ++x) {
          const int64_t src = x + e * Nv + i * NvNv + j * NvNv * No;
          s->Ta[x * Nv * No * No + e + i * Nv + j * Nv * No] = in->Tabij[src];
          /* the same element, read as T[x',y',i,j] with x' = x, y' = e */
          s->Tab[(x + e * Nv) * No * No + i + j * No] = in->Tabij[src];
          s->Vab[(x + e * Nv) * No * No + i + j * No] = in->Vabij[src];
        }
  for (int64_t k = 0; k < No; ++k)
    for (int64_t e = 0; e < Nv; ++e)
      for (int64_t y = 0; y < Nv; ++y)
        for (int64_t x = 0; x < Nv; ++x) {
          const int64_t src = x + y * Nv + e * NvNv + k * NvNv * Nv;
          s->Vp[(x + y * Nv) * Nv * No + e + k * Nv] = in->Vabci[src];
          if (s->Jp) s->Jp[(x + y * Nv) * Nv * No + e + k * Nv] = in->Jabci[src];
        }
}

static void free_slices(port_slices *s) {
  free(s->Ta);
  free(s->Vp);
  free(s->Jp);
  free(s->Tab);
  free(s->Vab);
}

/* Tijk[idx(i,j,k)] += from[perm(i,j,k)], the six reorder<> kernels of
 * src/atrip/Equations.cxx:27-83. */
enum { IJK, IKJ, JIK, JKI, KIJ, KJI };
static void reorder_add(int kind, int64_t n, double *to, const double *from) {
  for (int64_t k = 0, idx = 0; k < n; k++)
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++, idx++) {
        int64_t f;
        switch (kind) {
        case IJK: f = i + j * n + k * n * n; break;
        case IKJ: f = i + k * n + j * n * n; break;
        case JIK: f = j + i * n + k * n * n; break;
        case JKI: f = j + k * n + i * n * n; break;
        case KIJ: f = k + i * n + j * n * n; break;
        default: f = k + j * n + i * n * n; break;
        }
        to[idx] += from[f];
      }
}

/* doubles_contribution, DGEMM route (src/atrip/Equations.cxx:581-680). */
static void doubles_port(const port_slices *s, const double *Vh, const double *Vp, int a, int b,
                         int c, double *Tijk, double *tbuf) {
  const int64_t No = s->No, Nv = s->Nv, NoNo = No * No, NoNoNo = NoNo * No, slab = Nv * No;
  const double *VABph = Vp + (a + b * Nv) * slab, *VACph = Vp + (a + c * Nv) * slab,
               *VBCph = Vp + (b + c * Nv) * slab, *VBAph = Vp + (b + a * Nv) * slab,
               *VCAph = Vp + (c + a * Nv) * slab, *VCBph = Vp + (c + b * Nv) * slab;
  const double *VhhhA = Vh + a * NoNoNo, *VhhhB = Vh + b * NoNoNo, *VhhhC = Vh + c * NoNoNo;
  const double *TAphh = s->Ta + a * slab * No, *TBphh = s->Ta + b * slab * No,
               *TCphh = s->Ta + c * slab * No;
  const double *TABhh = s->Tab + (a + b * Nv) * NoNo, *TAChh = s->Tab + (a + c * Nv) * NoNo,
               *TBChh = s->Tab + (b + c * Nv) * NoNo;
  memset(Tijk, 0, sizeof(double) * NoNoNo);
#define HOLES(A, B, TR, R)                                                  \
  xgemm('N', TR, NoNo, No, No, -1.0, A, NoNo, B, No, tbuf, NoNo);           \
  reorder_add(R, No, Tijk, tbuf)
#define PARTICLES(A, B, R)                                                  \
  xgemm('T', 'N', NoNo, No, Nv, 1.0, A, Nv, B, Nv, tbuf, NoNo);             \
  reorder_add(R, No, Tijk, tbuf)
  /* the conjugating copies of V_hhh are plain copies for real F */
  HOLES(VhhhC, TABhh, 'N', IKJ);
  HOLES(VhhhC, TABhh, 'T', JKI);
  HOLES(VhhhB, TAChh, 'N', IJK);
  HOLES(VhhhB, TAChh, 'T', KJI);
  HOLES(VhhhA, TBChh, 'N', JIK);
  HOLES(VhhhA, TBChh, 'T', KIJ);
  PARTICLES(TAphh, VBCph, IJK);
  PARTICLES(TAphh, VCBph, IKJ);
  PARTICLES(TCphh, VABph, KIJ);
  PARTICLES(TCphh, VBAph, KJI);
  PARTICLES(TBphh, VACph, JIK);
  PARTICLES(TBphh, VCAph, JKI);
#undef HOLES
#undef PARTICLES
}

/* ------------------------------------------------------------ tuple loops */

typedef struct {
  const oracle_inputs *in;
  const port_slices *s;
  const int32_t *abc;
  int64_t t0, t1;
  int ijkabc, use_j, route;
  double *e, *ect;
} worker_args;

static void *worker(void *p) {
  worker_args *w = (worker_args *)p;
  const oracle_inputs *in = w->in;
  const int64_t No = in->No, Nv = in->Nv, n3 = No * No * No;
  double *T = (double *)malloc(sizeof(double) * n3), *Z = (double *)malloc(sizeof(double) * n3),
         *tb = (double *)malloc(sizeof(double) * n3),
         *Tai = (double *)malloc(sizeof(double) * Nv * No);
  for (int64_t x = 0; x < Nv * No; ++x) Tai[x] = w->ijkabc ? -in->Tai[x] : in->Tai[x];
  const int with_j = w->use_j && in->Jijka && in->Jabci;
  for (int64_t t = w->t0; t < w->t1; ++t) {
    const int a = w->abc[3 * t], b = w->abc[3 * t + 1], c = w->abc[3 * t + 2];
    if (w->route == 0)
      oracle_doubles_naive(in, a, b, c, in->Vijka, in->Vabci, T);
    else
      doubles_port(w->s, in->Vijka, w->s->Vp, a, b, c, T, tb);
    memcpy(Z, T, sizeof(double) * n3);
    oracle_singles(in, a, b, c, Tai, Z);
    w->e[t] = tuple_energy(in, a, b, c, T, Z);
    if (with_j) {
      if (w->route == 0)
        oracle_doubles_naive(in, a, b, c, in->Jijka, in->Jabci, T);
      else
        doubles_port(w->s, in->Jijka, w->s->Jp, a, b, c, T, tb);
      w->ect[t] = tuple_energy(in, a, b, c, T, Z);
    } else {
      w->ect[t] = w->e[t];
    }
  }
  free(T);
  free(Z);
  free(tb);
  free(Tai);
  return 0;
}

/* Per-tuple energies e[t], ect[t] for lexicographic tuples t in [t0, t1).
 * route 0 = naive loops, 1 = DGEMM-route port.  The (cT) energy uses the J
 * intermediates when use_j and both are present, else equals e
 * (src/atrip/Atrip.cxx:925-963).  Returns 0 on success. */
int oracle_tuple_energies(const oracle_inputs *in, int64_t t0, int64_t t1, int ijkabc, int use_j,
                          int route, int nthreads, double *e, double *ect) {
  const int64_t n = oracle_n_tuples(in->Nv);
  if (t0 < 0 || t1 > n || t0 > t1 || nthreads < 1) return 1;
  int32_t *abc = (int32_t *)malloc(sizeof(int32_t) * 3 * (n > 0 ? n : 1));
  oracle_tuple_list(in->Nv, abc);
  port_slices s;
  memset(&s, 0, sizeof(s));
  if (route == 1) cut_slices(in, &s);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  worker_args *args = (worker_args *)malloc(sizeof(worker_args) * nthreads);
  const int64_t total = t1 - t0, per = (total + nthreads - 1) / nthreads;
  int started = 0;
  for (int r = 0; r < nthreads; ++r) {
    worker_args w = {in, &s, abc, t0 + r * per, t0 + (r + 1) * per, ijkabc, use_j, route,
                     e - t0, ect - t0};
    if (w.t0 > t1) w.t0 = t1;
    if (w.t1 > t1) w.t1 = t1;
    args[r] = w;
    if (nthreads == 1) {
      worker(&args[r]);
    } else {
      pthread_create(&th[r], 0, worker, &args[r]);
      started++;
    }
  }
  for (int r = 0; r < started; ++r) pthread_join(th[r], 0);
  free(th);
  free(args);
  if (route == 1) free_slices(&s);
  free(abc);
  return 0;
}

/* Prepared DGEMM-route port: slices cut once, then timed tuple ranges
 * (bench.py's CPU baseline times oracle_port_run only). */
typedef struct {
  oracle_inputs in;
  port_slices s;
  int32_t *abc;
} oracle_port;

void *oracle_port_prepare(const oracle_inputs *in) {
  oracle_port *p = (oracle_port *)calloc(1, sizeof(oracle_port));
  p->in = *in;
  cut_slices(in, &p->s);
  const int64_t n = oracle_n_tuples(in->Nv);
  p->abc = (int32_t *)malloc(sizeof(int32_t) * 3 * (n > 0 ? n : 1));
  oracle_tuple_list(in->Nv, p->abc);
  return p;
}

int oracle_port_run(void *h, int64_t t0, int64_t t1, int ijkabc, int use_j, int nthreads,
                    double *e, double *ect) {
  oracle_port *p = (oracle_port *)h;
  const int64_t n = oracle_n_tuples(p->in.Nv);
  if (!p || t0 < 0 || t1 > n || t0 > t1 || nthreads < 1) return 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  worker_args *args = (worker_args *)malloc(sizeof(worker_args) * nthreads);
  const int64_t per = (t1 - t0 + nthreads - 1) / nthreads;
  for (int r = 0; r < nthreads; ++r) {
    worker_args w = {&p->in, &p->s, p->abc, t0 + r * per, t0 + (r + 1) * per, ijkabc, use_j, 1,
                     e - t0, ect - t0};
    if (w.t0 > t1) w.t0 = t1;
    if (w.t1 > t1) w.t1 = t1;
    args[r] = w;
    pthread_create(&th[r], 0, worker, &args[r]);
  }
  for (int r = 0; r < nthreads; ++r) pthread_join(th[r], 0);
  free(th);
  free(args);
  return 0;
}

void oracle_port_free(void *h) {
  oracle_port *p = (oracle_port *)h;
  if (!p) return;
  free_slices(&p->s);
  free(p->abc);
  free(p);
}

/* Tijk and Zijk of one tuple through the naive route (element-wise checks). */
int oracle_tuple_arrays(const oracle_inputs *in, int a, int b, int c, int ijkabc, double *Tijk,
                        double *Zijk) {
  const int64_t No = in->No, Nv = in->Nv, n3 = No * No * No;
  double *Tai = (double *)malloc(sizeof(double) * Nv * No);
  for (int64_t x = 0; x < Nv * No; ++x) Tai[x] = ijkabc ? -in->Tai[x] : in->Tai[x];
  oracle_doubles_naive(in, a, b, c, in->Vijka, in->Vabci, Tijk);
  memcpy(Zijk, Tijk, sizeof(double) * n3);
  oracle_singles(in, a, b, c, Tai, Zijk);
  free(Tai);
  return 0;
}

/* Sum of tuple energies in tuple order with the final sign of
 * src/atrip/Atrip.cxx:1108-1111 (E = -sum unless ijkabc). */
double oracle_total(const double *e, int64_t n, int ijkabc) {
  double s = 0.0;
  for (int64_t t = 0; t < n; ++t) s += e[t];
  return ijkabc ? s : -s;
}
