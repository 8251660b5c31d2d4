/* Driver that runs the UNMODIFIED atrip reference sources as a one-rank CPU
 * oracle (test infrastructure only; never linked into the product).
 *
 * Inputs: a directory holding meta.txt ("No Nv hasJ [complex]") and
 * column-major .bin files epsi, epsa, Tai, Tabij, Vabij, Vijka, Vabci
 * [, Jijka, Jabci] -- exactly the arrays CTF's read_all would return for
 * atrip's input tensors (src/atrip/Atrip.hpp:68-107): FP64, or interleaved
 * (re, im) FP64 pairs when the complex flag is 1, in which case every mode
 * runs the reference's Complex instantiation (src/atrip/Atrip.cxx:1136).
 *
 * Modes
 *   run  [maxit] [ijkabc] [usej] [group]
 *                                 -> Atrip::init + Atrip::run<double>
 *                                    (src/atrip/Atrip.cxx:66-1133)
 *   tuples N [ijkabc] [usej]      -> per-tuple energies of the first N
 *                                    lexicographic tuples, calling the
 *                                    reference's doubles_contribution /
 *                                    singles_contribution / get_energy_*
 *                                    directly with slices cut as in
 *                                    src/atrip/Unions.hpp:77-278
 *   dump t                        -> Tijk and Zijk of tuple t
 * Output lines start with RESULT / TUPLE / TIJK / ZIJK for easy parsing
 * (complex Tijk/Zijk values print as "re im").
 */
#include <atrip.hpp>
#include <atrip/Equations.hpp>
#include <atrip/Tuples.hpp>

#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

using atrip::Atrip;

template <typename F>
static std::vector<F> load(const std::string &dir, const char *name, size_t n) {
  std::vector<F> v(n);
  std::string path = dir + "/" + name + ".bin";
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path.c_str()); std::exit(2); }
  if (std::fread(v.data(), sizeof(F), n, f) != n) {
    std::fprintf(stderr, "short read %s\n", path.c_str()); std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <typename F>
struct Inputs {
  int No = 0, Nv = 0, hasJ = 0;
  std::vector<F> epsi, epsa, Tai, Tabij, Vabij, Vijka, Vabci, Jijka, Jabci;
};

template <typename F>
static Inputs<F> read_inputs(const std::string &dir, int No, int Nv, int hasJ) {
  Inputs<F> in;
  in.No = No;
  in.Nv = Nv;
  in.hasJ = hasJ;
  const size_t o = No, v = Nv;
  in.epsi = load<F>(dir, "epsi", o);
  in.epsa = load<F>(dir, "epsa", v);
  in.Tai = load<F>(dir, "Tai", v * o);
  in.Tabij = load<F>(dir, "Tabij", v * v * o * o);
  in.Vabij = load<F>(dir, "Vabij", v * v * o * o);
  in.Vijka = load<F>(dir, "Vijka", o * o * o * v);
  in.Vabci = load<F>(dir, "Vabci", v * v * v * o);
  if (in.hasJ) {
    in.Jijka = load<F>(dir, "Jijka", o * o * o * v);
    in.Jabci = load<F>(dir, "Jabci", v * v * v * o);
  }
  return in;
}

template <typename F>
static CTF::Tensor<F> *make(std::vector<int> lens, const std::vector<F> &v) {
  auto *t = new CTF::Tensor<F>((int)lens.size(), lens.data());
  std::copy(v.begin(), v.end(), t->data);
  return t;
}

static void print_value(const char *tag, double x) { std::printf("%s %.17g\n", tag, x); }
static void print_value(const char *tag, const std::complex<double> &x) {
  std::printf("%s %.17g %.17g\n", tag, x.real(), x.imag());
}

template <typename F>
static int mode_run(const Inputs<F> &in, size_t maxit, bool ijkabc, bool usej, bool group) {
  const int No = in.No, Nv = in.Nv;
  Atrip::init(MPI_COMM_WORLD);
  auto *ei = make({No}, in.epsi), *ea = make({Nv}, in.epsa),
       *Tph = make({Nv, No}, in.Tai), *Tpphh = make({Nv, Nv, No, No}, in.Tabij),
       *Vpphh = make({Nv, Nv, No, No}, in.Vabij),
       *Vhhhp = make({No, No, No, Nv}, in.Vijka),
       *Vppph = make({Nv, Nv, Nv, No}, in.Vabci);
  CTF::Tensor<F> *Jhhhp = nullptr, *Jppph = nullptr;
  auto input = Atrip::Input<F>()
                   .with_epsilon_i(ei)
                   .with_epsilon_a(ea)
                   .with_Tai(Tph)
                   .with_Tabij(Tpphh)
                   .with_Vabij(Vpphh)
                   .with_Vijka(Vhhhp)
                   .with_Vabci(Vppph)
                   .with_max_iterations(maxit)
                   .with_ijkabc(ijkabc)
                   .with_read_checkpoint_if_exists(false)
                   .with_checkpoint_at_every_iteration(~size_t(0) >> 1)
                   .with_checkpoint_path("/dev/null");
  if (group)
    input.with_tuples_distribution(Atrip::Input<F>::TuplesDistribution::GROUP_AND_SORT);
  if (usej && in.hasJ) {
    Jhhhp = make({No, No, No, Nv}, in.Jijka);
    Jppph = make({Nv, Nv, Nv, No}, in.Jabci);
    input.with_Jijka(Jhhhp).with_Jabci(Jppph);
  }
  auto t0 = std::chrono::steady_clock::now();
  Atrip::Output out = Atrip::run<F>(input);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("RESULT %.17g %.17g %.6f\n", out.energy, out.ct_energy, secs);
  return 0;
}

template <typename F>
struct SliceSet {
  std::vector<F> V[6], Vh[3], Ta[3], Tab[3];
};

template <typename F>
static void cut(const Inputs<F> &in, const std::vector<F> &Vp, const std::vector<F> &Vh,
                size_t a, size_t b, size_t c, SliceSet<F> &s) {
  const size_t No = in.No, Nv = in.Nv;
  const size_t pairs[6][2] = {{a, b}, {a, c}, {b, c}, {b, a}, {c, a}, {c, b}};
  for (int p = 0; p < 6; ++p) {
    s.V[p].resize(Nv * No);
    for (size_t k = 0; k < No; ++k)
      for (size_t e = 0; e < Nv; ++e)
        s.V[p][e + k * Nv] = Vp[pairs[p][0] + pairs[p][1] * Nv + e * Nv * Nv + k * Nv * Nv * Nv];
  }
  const size_t xs[3] = {a, b, c};
  for (int x = 0; x < 3; ++x) {
    s.Vh[x].assign(Vh.begin() + xs[x] * No * No * No, Vh.begin() + (xs[x] + 1) * No * No * No);
    s.Ta[x].resize(Nv * No * No);
    for (size_t j = 0; j < No; ++j)
      for (size_t i = 0; i < No; ++i)
        for (size_t e = 0; e < Nv; ++e)
          s.Ta[x][e + i * Nv + j * Nv * No] =
              in.Tabij[xs[x] + e * Nv + i * Nv * Nv + j * Nv * Nv * No];
  }
  const size_t tp[3][2] = {{a, b}, {a, c}, {b, c}};
  for (int p = 0; p < 3; ++p) {
    s.Tab[p].resize(No * No);
    for (size_t j = 0; j < No; ++j)
      for (size_t i = 0; i < No; ++i)
        s.Tab[p][i + j * No] = in.Tabij[tp[p][0] + tp[p][1] * Nv + i * Nv * Nv + j * Nv * Nv * No];
  }
}

template <typename F>
static void doubles(const Inputs<F> &in, SliceSet<F> &s, F *Tijk, F *tb, F *vh) {
  atrip::doubles_contribution<F>(in.No, in.Nv,
      s.V[0].data(), s.V[1].data(), s.V[2].data(), s.V[3].data(), s.V[4].data(), s.V[5].data(),
      s.Vh[0].data(), s.Vh[1].data(), s.Vh[2].data(),
      s.Ta[0].data(), s.Ta[1].data(), s.Ta[2].data(),
      s.Tab[0].data(), s.Tab[1].data(), s.Tab[2].data(), Tijk, tb, vh);
}

/* One tuple through the reference's own kernels, in the order of
 * src/atrip/Atrip.cxx:855-963. */
template <typename F>
static void tuple_energy(const Inputs<F> &in, size_t a, size_t b, size_t c, bool ijkabc,
                         bool usej, double &e, double &ect, std::vector<F> *dumpT = nullptr,
                         std::vector<F> *dumpZ = nullptr) {
  const size_t No = in.No, Nv = in.Nv, n3 = No * No * No;
  std::vector<F> Tijk(n3), Zijk(n3), tb(n3), vh(n3), Tai(in.Tai);
  if (ijkabc) for (auto &x : Tai) x = -x;
  std::vector<F> epsi(in.epsi);
  SliceSet<F> s;
  cut(in, in.Vabci, in.Vijka, a, b, c, s);
  doubles(in, s, Tijk.data(), tb.data(), vh.data());
  Zijk = Tijk;
  std::vector<F> VAB(No * No), VAC(No * No), VBC(No * No);
  for (size_t j = 0; j < No; ++j)
    for (size_t i = 0; i < No; ++i) {
      const size_t o = i * Nv * Nv + j * Nv * Nv * No;
      VAB[i + j * No] = in.Vabij[a + b * Nv + o];
      VAC[i + j * No] = in.Vabij[a + c * Nv + o];
      VBC[i + j * No] = in.Vabij[b + c * Nv + o];
    }
  atrip::singles_contribution<F>(No, Nv, a, b, c, Tai.data(), VAB.data(), VAC.data(),
                                 VBC.data(), Zijk.data());
  if (dumpT) *dumpT = Tijk;
  if (dumpZ) *dumpZ = Zijk;
  // src/atrip/Atrip.cxx:640-646: real part of the sum, as a field value
  const F epsabc{std::real(in.epsa[a] + in.epsa[b] + in.epsa[c])};
  int distinct = 0;
  if (a == b) distinct++;
  if (b == c) distinct--;
  auto energy = [&](F *T) {
    double r = 0.0;
    if (distinct == 0)
      atrip::get_energy_distinct<F>(epsabc, No, epsi.data(), T, Zijk.data(), &r);
    else
      atrip::get_energy_same<F>(epsabc, No, epsi.data(), T, Zijk.data(), &r);
    return r;
  };
  e = energy(Tijk.data());
  if (usej && in.hasJ) {
    SliceSet<F> sj;
    cut(in, in.Jabci, in.Jijka, a, b, c, sj);
    doubles(in, sj, Tijk.data(), tb.data(), vh.data());
  }
  ect = energy(Tijk.data());
}

template <typename F>
static int main_t(const std::string &dir, const std::string &mode, int No, int Nv, int hasJ,
                  int argc, char **argv) {
  Inputs<F> in = read_inputs<F>(dir, No, Nv, hasJ);
  auto arg = [&](int i, long dflt) { return argc > i ? std::atol(argv[i]) : dflt; };
  if (mode == "run")
    return mode_run(in, (size_t)arg(3, 0), arg(4, 0) != 0, arg(5, 1) != 0, arg(6, 0) != 0);
  if (mode == "tuples") {
    const size_t n = (size_t)arg(3, 10);
    const bool ijkabc = arg(4, 0) != 0, usej = arg(5, 1) != 0;
    auto all = atrip::get_all_tuples_list(in.Nv);
    for (size_t t = 0; t < n && t < all.size(); ++t) {
      double e, ect;
      tuple_energy(in, all[t][0], all[t][1], all[t][2], ijkabc, usej, e, ect);
      std::printf("TUPLE %zu %zu %zu %zu %.17g %.17g\n", t, all[t][0], all[t][1], all[t][2], e,
                  ect);
    }
    return 0;
  }
  if (mode == "dump") {
    const size_t t = (size_t)arg(3, 0);
    auto all = atrip::get_all_tuples_list(in.Nv);
    std::vector<F> T, Z;
    double e, ect;
    tuple_energy(in, all[t][0], all[t][1], all[t][2], false, false, e, ect, &T, &Z);
    for (const F &x : T) print_value("TIJK", x);
    for (const F &x : Z) print_value("ZIJK", x);
    std::printf("TUPLE %zu %zu %zu %zu %.17g %.17g\n", t, all[t][0], all[t][1], all[t][2], e, ect);
    return 0;
  }
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s DIR run|tuples|dump ...\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1], mode = argv[2];
  int No = 0, Nv = 0, hasJ = 0, cplx = 0;
  {
    std::ifstream meta(dir + "/meta.txt");
    meta >> No >> Nv >> hasJ;
    if (!(meta >> cplx)) cplx = 0;
  }
  try {
    if (cplx) return main_t<atrip::Complex>(dir, mode, No, Nv, hasJ, argc, argv);
    return main_t<double>(dir, mode, No, Nv, hasJ, argc, argv);
  } catch (const char *m) {
    std::fprintf(stderr, "reference threw: %s\n", m);
    return 3;
  } catch (const std::string &m) {
    std::fprintf(stderr, "reference threw: %s\n", m.c_str());
    return 3;
  }
}
