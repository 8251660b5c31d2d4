// Compiles unchanged atrip-style driver code against the drop-in header
// (include/atrip.hpp) and runs it.  Test infrastructure: the MPI and CTF
// stand-ins come from oracle/ref_shims.  Reads the seeded inputs from a
// directory written by atrip_gb300.synth.write_bin_dir (real or complex,
// per its meta.txt) and prints "RESULT energy ct_energy".
#include <atrip.hpp>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

template <typename F>
static std::vector<F> load(const std::string &dir, const char *name, size_t n) {
  std::vector<F> v(n);
  FILE *f = std::fopen((dir + "/" + name + ".bin").c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(F), n, f) != n) std::exit(2);
  std::fclose(f);
  return v;
}

template <typename F>
static CTF::Tensor<F> *tensor(std::vector<int> lens, const std::vector<F> &v) {
  auto *t = new CTF::Tensor<F>((int)lens.size(), lens.data());
  std::copy(v.begin(), v.end(), t->data);
  return t;
}

template <typename F>
static int drive(const std::string &dir, int No, int Nv, int hasJ, int form) {
  const size_t o = No, v = Nv;
  auto *ei = tensor<F>({No}, load<F>(dir, "epsi", o));
  auto *ea = tensor<F>({Nv}, load<F>(dir, "epsa", v));
  auto *Tai = tensor<F>({Nv, No}, load<F>(dir, "Tai", v * o));
  auto *Tabij = tensor<F>({Nv, Nv, No, No}, load<F>(dir, "Tabij", v * v * o * o));
  auto *Vabij = tensor<F>({Nv, Nv, No, No}, load<F>(dir, "Vabij", v * v * o * o));
  auto *Vijka = tensor<F>({No, No, No, Nv}, load<F>(dir, "Vijka", o * o * o * v));
  auto *Vabci = tensor<F>({Nv, Nv, Nv, No}, load<F>(dir, "Vabci", v * v * v * o));
  atrip::Atrip::init(MPI_COMM_WORLD);
  auto in = typename atrip::Atrip::template Input<F>()
                .with_epsilon_i(ei)
                .with_epsilon_a(ea)
                .with_Tai(Tai)
                .with_Tabij(Tabij)
                .with_Vabij(Vabij)
                .with_Vijka(Vijka)
                .with_Vabci(Vabci)
                .with_read_checkpoint_if_exists(false)
                .with_form(form)
                .with_slices(form == ATRIP_FORM_SPLIT_F16 ? 2 : 3);
  if (hasJ)
    in.with_Jijka(tensor<F>({No, No, No, Nv}, load<F>(dir, "Jijka", o * o * o * v)))
        .with_Jabci(tensor<F>({Nv, Nv, Nv, No}, load<F>(dir, "Jabci", v * v * v * o)));
  try {
    atrip::Atrip::Output out = atrip::Atrip::run(in);
    std::printf("RESULT %.17g %.17g\n", out.energy, out.ct_energy);
  } catch (const std::string &m) {
    std::fprintf(stderr, "atrip error: %s\n", m.c_str());
    return 3;
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string dir = argv[1];
  const int form = std::atoi(argv[2]);
  int No = 0, Nv = 0, hasJ = 0, cplx = 0;
  std::ifstream meta(dir + "/meta.txt");
  meta >> No >> Nv >> hasJ;
  if (!(meta >> cplx)) cplx = 0;
  return cplx ? drive<atrip::Complex>(dir, No, Nv, hasJ, form)
              : drive<double>(dir, No, Nv, hasJ, form);
}
