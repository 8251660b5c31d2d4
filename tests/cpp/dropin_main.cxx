// Compiles unchanged atrip-style driver code against the drop-in header
// (include/atrip.hpp) and runs it.  Test infrastructure: the MPI and CTF
// stand-ins come from oracle/ref_shims.  Reads the seeded inputs from a
// directory written by atrip_gb300.synth.write_bin_dir and prints
// "RESULT energy ct_energy".
#include <atrip.hpp>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

static std::vector<double> load(const std::string &dir, const char *name, size_t n) {
  std::vector<double> v(n);
  FILE *f = std::fopen((dir + "/" + name + ".bin").c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(double), n, f) != n) std::exit(2);
  std::fclose(f);
  return v;
}

static CTF::Tensor<double> *tensor(std::vector<int> lens, const std::vector<double> &v) {
  auto *t = new CTF::Tensor<double>((int)lens.size(), lens.data());
  std::copy(v.begin(), v.end(), t->data);
  return t;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string dir = argv[1];
  const int form = std::atoi(argv[2]);
  int No, Nv, hasJ;
  std::ifstream(dir + "/meta.txt") >> No >> Nv >> hasJ;
  const size_t o = No, v = Nv;
  auto *ei = tensor({No}, load(dir, "epsi", o));
  auto *ea = tensor({Nv}, load(dir, "epsa", v));
  auto *Tai = tensor({Nv, No}, load(dir, "Tai", v * o));
  auto *Tabij = tensor({Nv, Nv, No, No}, load(dir, "Tabij", v * v * o * o));
  auto *Vabij = tensor({Nv, Nv, No, No}, load(dir, "Vabij", v * v * o * o));
  auto *Vijka = tensor({No, No, No, Nv}, load(dir, "Vijka", o * o * o * v));
  auto *Vabci = tensor({Nv, Nv, Nv, No}, load(dir, "Vabci", v * v * v * o));
  atrip::Atrip::init(MPI_COMM_WORLD);
  auto in = atrip::Atrip::Input<double>()
                .with_epsilon_i(ei)
                .with_epsilon_a(ea)
                .with_Tai(Tai)
                .with_Tabij(Tabij)
                .with_Vabij(Vabij)
                .with_Vijka(Vijka)
                .with_Vabci(Vabci)
                .with_read_checkpoint_if_exists(false)
                .with_form(form)
                .with_slices(3);
  if (hasJ)
    in.with_Jijka(tensor({No, No, No, Nv}, load(dir, "Jijka", o * o * o * v)))
        .with_Jabci(tensor({Nv, Nv, Nv, No}, load(dir, "Jabci", v * v * v * o)));
  try {
    atrip::Atrip::Output out = atrip::Atrip::run(in);
    std::printf("RESULT %.17g %.17g\n", out.energy, out.ct_energy);
  } catch (const std::string &m) {
    std::fprintf(stderr, "atrip error: %s\n", m.c_str());
    return 3;
  }
  // the complex field is declared and reports that it is not built
  try {
    atrip::Atrip::run(atrip::Atrip::Input<atrip::Complex>());
    return 4;
  } catch (const std::string &) {
  }
  return 0;
}
