/* CPU oracle for the complex field (atrip's run<Complex>) -- TEST
 * INFRASTRUCTURE ONLY (used by tests/ as the checker, never by the product).
 *
 * Plain-C restatement of the reference's Complex instantiation on the
 * configure-default route (ATRIP_USE_DGEMM, configure.ac:96-102):
 *   doubles   src/atrip/Equations.cxx:599-665: every hole term uses the
 *             conjugated V_hhhp slice (MAYBE_CONJ of VhhhA/B/C before the
 *             hole GEMMs, Operations.hpp:28-44), particle terms use the
 *             slices as they are;
 *   singles   src/atrip/Equations.cxx:387-426, no conjugation;
 *   energy    src/atrip/Equations.cxx:101-238 with A..F = conj(Tijk),
 *             U..Z = Zijk, the complex sum's real part per tuple; epsabc is
 *             the real part of eps_a + eps_b + eps_c as a complex number
 *             (src/atrip/Atrip.cxx:643-646), eps_i stays complex.
 * (The reference's BLAS-free loops, Equations.cxx:685-726, skip the hole
 * conjugation, so its two routes disagree for complex input; the default
 * route is the one restated here.)
 *
 * All tensors are interleaved (re, im) FP64, column-major -- what
 * CTF::Tensor<Complex>::read_all returns.  Complex products and quotients
 * are C99 `double complex` arithmetic, the same compiler built-ins that
 * std::complex<double> uses.
 */
#include <complex.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zd;

typedef struct {
  int No, Nv;
  const double *epsi, *epsa, *Tai, *Tabij, *Vabij, *Vijka, *Vabci, *Jijka, *Jabci;
} oracle_z_inputs;

static inline zd ld(const double *p, int64_t i) { return p[2 * i] + I * p[2 * i + 1]; }

/* Tijk of tuple (a,b,c) (index i + j No + k No^2), terms in the order of
 * src/atrip/Equations.cxx:599-665. */
void oracle_z_doubles(const oracle_z_inputs *in, int a, int b, int c, const double *Vh,
                      const double *Vp, double *Tijk) {
  const int64_t No = in->No, Nv = in->Nv, NoNo = No * No, NvNv = Nv * Nv;
  const double *T = in->Tabij;
#define TPH(x, e, i, j) ld(T, (x) + (e) * Nv + (i) * NvNv + (j) * NvNv * No)
#define THH(x, y, i, j) ld(T, (x) + (y) * Nv + (i) * NvNv + (j) * NvNv * No)
#define VHC(i, j, k, x) conj(ld(Vh, (i) + (j) * No + (k) * NoNo + (x) * NoNo * No))
#define VPPH(x, y, e, k) ld(Vp, (x) + (y) * Nv + (e) * NvNv + (k) * NvNv * Nv)
  for (int64_t k = 0; k < No; k++)
    for (int64_t j = 0; j < No; j++)
      for (int64_t i = 0; i < No; i++) {
        zd t = 0.0;
        for (int64_t L = 0; L < No; L++) {
          t -= THH(a, b, L, j) * VHC(i, k, L, c);
          t -= THH(a, b, i, L) * VHC(j, k, L, c);
          t -= THH(a, c, L, k) * VHC(i, j, L, b);
          t -= THH(a, c, i, L) * VHC(k, j, L, b);
          t -= THH(b, c, L, k) * VHC(j, i, L, a);
          t -= THH(b, c, j, L) * VHC(k, i, L, a);
        }
        for (int64_t E = 0; E < Nv; E++) {
          t += TPH(a, E, i, j) * VPPH(b, c, E, k);
          t += TPH(a, E, i, k) * VPPH(c, b, E, j);
          t += TPH(c, E, k, i) * VPPH(a, b, E, j);
          t += TPH(c, E, k, j) * VPPH(b, a, E, i);
          t += TPH(b, E, j, i) * VPPH(a, c, E, k);
          t += TPH(b, E, j, k) * VPPH(c, a, E, i);
        }
        const int64_t o = i + j * No + k * NoNo;
        Tijk[2 * o] = creal(t);
        Tijk[2 * o + 1] = cimag(t);
      }
#undef TPH
#undef THH
#undef VHC
#undef VPPH
}

/* Z += t1 (x) Vpphh (src/atrip/Equations.cxx:387-426). */
static void singles(const oracle_z_inputs *in, int a, int b, int c, const zd *Tai, zd *Z) {
  const int64_t No = in->No, Nv = in->Nv, NoNo = No * No, NvNv = Nv * Nv;
  const double *V = in->Vabij;
#define VHH(x, y, i, j) ld(V, (x) + (y) * Nv + (i) * NvNv + (j) * NvNv * No)
  for (int64_t k = 0; k < No; k++)
    for (int64_t i = 0; i < No; i++)
      for (int64_t j = 0; j < No; j++) {
        const int64_t ijk = i + j * No + k * NoNo;
        Z[ijk] += Tai[a + i * Nv] * VHH(b, c, j, k);
        Z[ijk] += Tai[b + j * Nv] * VHH(a, c, i, k);
        Z[ijk] += Tai[c + k * Nv] * VHH(a, b, i, j);
      }
#undef VHH
}

/* get_energy_distinct / get_energy_same for Complex: conj(T) against Z,
 * blocked loop order of src/atrip/Equations.cxx:101-238, real part. */
static double energy(int distinct, zd epsabc, int64_t No, const zd *epsi, const zd *T,
                     const zd *Z) {
  const int64_t bs = 16;
  zd acc = 0.0;
  for (int64_t kk = 0; kk < No; kk += bs) {
    const int64_t kend = kk + bs < No ? kk + bs : No;
    for (int64_t jj = kk; jj < No; jj += bs) {
      const int64_t jend = jj + bs < No ? jj + bs : No;
      for (int64_t ii = jj; ii < No; ii += bs) {
        const int64_t iend = ii + bs < No ? ii + bs : No;
        for (int64_t k = kk; k < kend; k++)
          for (int64_t j = (jj > k ? jj : k); j < jend; j++) {
            const double facjk = j == k ? 0.5 : 1.0;
            for (int64_t i = (ii > j ? ii : j); i < iend; i++) {
              const double facij = i == j ? 0.5 : 1.0;
              const zd denominator = epsabc - ((epsi[i] + epsi[j]) + epsi[k]);
#define IX(p, q, r) ((p) + No * (q) + No * No * (r))
              zd value;
              if (distinct) {
                const zd U = Z[IX(i, j, k)], V = Z[IX(i, k, j)], W = Z[IX(j, i, k)],
                         X = Z[IX(j, k, i)], Y = Z[IX(k, i, j)], ZZ = Z[IX(k, j, i)];
                const zd A = conj(T[IX(i, j, k)]), B = conj(T[IX(i, k, j)]),
                         C = conj(T[IX(j, i, k)]), D = conj(T[IX(j, k, i)]),
                         E = conj(T[IX(k, i, j)]), F = conj(T[IX(k, j, i)]);
                const zd UXY = U + (X + Y), VWZ = V + (W + ZZ), ADE = A + (D + E),
                         BCF = B + (C + F);
                const zd first = A * U + (B * V + (C * W + (D * X + (E * Y + F * ZZ))));
                value = 3.0 * first + ((UXY - 2.0 * VWZ) * ADE + (VWZ - 2.0 * UXY) * BCF);
              } else {
                const zd U = Z[IX(i, j, k)], V = Z[IX(j, k, i)], W = Z[IX(k, i, j)];
                const zd A = conj(T[IX(i, j, k)]), B = conj(T[IX(j, k, i)]),
                         C = conj(T[IX(k, i, j)]);
                value = 3.0 * ((A * U + B * V) + C * W) - (A + (B + C)) * (U + (V + W));
              }
#undef IX
              acc += (2.0 * value / denominator) * (facjk * facij);
            }
          }
      }
    }
  }
  return creal(acc);
}

/* Tijk, Zijk (interleaved) and the energies of one tuple. */
static void tuple(const oracle_z_inputs *in, int a, int b, int c, int ijkabc, int use_j,
                  double *e, double *ect, double *Tout, double *Zout) {
  const int64_t No = in->No, Nv = in->Nv, n3 = No * No * No;
  double *Tb = malloc(sizeof(double) * 2 * n3);
  zd *T = malloc(sizeof(zd) * n3), *Z = malloc(sizeof(zd) * n3);
  zd *Tai = malloc(sizeof(zd) * Nv * No), *epsi = malloc(sizeof(zd) * No);
  for (int64_t x = 0; x < Nv * No; ++x) Tai[x] = (ijkabc ? -1.0 : 1.0) * ld(in->Tai, x);
  for (int64_t x = 0; x < No; ++x) epsi[x] = ld(in->epsi, x);
  oracle_z_doubles(in, a, b, c, in->Vijka, in->Vabci, Tb);
  for (int64_t x = 0; x < n3; ++x) T[x] = Z[x] = Tb[2 * x] + I * Tb[2 * x + 1];
  singles(in, a, b, c, Tai, Z);
  int cls = 0;
  if (a == b) cls++;
  if (b == c) cls--;
  const zd epsabc = creal(ld(in->epsa, a) + ld(in->epsa, b) + ld(in->epsa, c));
  *e = energy(cls == 0, epsabc, No, epsi, T, Z);
  if (Tout) memcpy(Tout, Tb, sizeof(double) * 2 * n3);
  if (Zout)
    for (int64_t x = 0; x < n3; ++x) {
      Zout[2 * x] = creal(Z[x]);
      Zout[2 * x + 1] = cimag(Z[x]);
    }
  if (use_j && in->Jijka && in->Jabci) {
    oracle_z_doubles(in, a, b, c, in->Jijka, in->Jabci, Tb);
    for (int64_t x = 0; x < n3; ++x) T[x] = Tb[2 * x] + I * Tb[2 * x + 1];
  }
  *ect = energy(cls == 0, epsabc, No, epsi, T, Z);
  free(Tb);
  free(T);
  free(Z);
  free(Tai);
  free(epsi);
}

int oracle_z_tuple_arrays(const oracle_z_inputs *in, int a, int b, int c, int ijkabc, double *T,
                          double *Z) {
  double e, ect;
  tuple(in, a, b, c, ijkabc, 0, &e, &ect, T, Z);
  return 0;
}

typedef struct {
  const oracle_z_inputs *in;
  const int32_t *abc;
  int64_t t0, t1, stride, first;
  int ijkabc, use_j;
  double *e, *ect;
} zjob;

static void *zworker(void *p) {
  zjob *j = p;
  for (int64_t t = j->first; t < j->t1; t += j->stride)
    tuple(j->in, j->abc[3 * t], j->abc[3 * t + 1], j->abc[3 * t + 2], j->ijkabc, j->use_j,
          &j->e[t - j->t0], &j->ect[t - j->t0], 0, 0);
  return 0;
}

/* Per-tuple energies of list positions t0 .. t1-1 (lexicographic list,
 * src/atrip/Tuples.cxx:122-134) on nthreads host threads. */
int oracle_z_tuple_energies(const oracle_z_inputs *in, const int32_t *abc, int64_t t0, int64_t t1,
                            int ijkabc, int use_j, int nthreads, double *e, double *ect) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  zjob jobs[256];
  for (int w = 0; w < nthreads; ++w) {
    jobs[w] = (zjob){in, abc, t0, t1, nthreads, t0 + w, ijkabc, use_j, e, ect};
    if (pthread_create(&th[w], 0, zworker, &jobs[w]) != 0) {
      zworker(&jobs[w]);
      th[w] = 0;
    }
  }
  for (int w = 0; w < nthreads; ++w)
    if (th[w]) pthread_join(th[w], 0);
  return 0;
}
