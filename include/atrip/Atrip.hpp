// atrip_gb300 -- source-compatible drop-in for atrip's public C++ API
// (src/atrip/Atrip.hpp:41-140 of the reference).
//
// Code written against atrip (cc4s-style drivers, atrip's own bench/main.cxx)
// includes <atrip.hpp>, fills an Atrip::Input<F> with CTF tensors and calls
// Atrip::run<F>.  This header keeps those names, members, builder methods and
// defaults; Atrip::run gathers each tensor with read_all and hands it to the
// GB300 engine through the C ABI in <atrip_gb300.h>.  Link with
// -latrip_gb300.  Like atrip, it needs <mpi.h> and <ctf.hpp> on the include
// path (real ones, or any stand-ins that provide MPI_Comm and
// CTF::Tensor<F>{lens, read_all}).
//
// Differences a caller can see:
//  * one process drives one GPU; Atrip::rank is 0 and Atrip::np is 1;
//  * TuplesDistribution is accepted, and both values map to the on-device
//    work queue over atrip's lexicographic tuple list;
//  * checkpoints keep atrip's YAML format and resume semantics; when atrip
//    would write one every iteration (checkpoint modulus 0,
//    src/atrip/Atrip.cxx:588-591, 713) they are written between tuple chunks
//    of the device queue (checkpoint_chunks per run);
//  * extra attributes select the arithmetic form and device (form: an
//    atrip_form value -- FP64, BF16 or FP16 split, auto; slices; device);
//  * F = std::complex<double> runs the FP64 form only.
#ifndef ATRIP_GB300_ATRIP_HPP_
#define ATRIP_GB300_ATRIP_HPP_

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iomanip>
#include <map>
#include <string>
#include <vector>

#include <mpi.h>
#include <ctf.hpp>

#include <atrip_gb300.h>
#include <atrip/Chrono.hpp>
#include <atrip/Complex.hpp>
#include <atrip/Debug.hpp>

#define ATRIP_GB300_ADD_ATTRIBUTE(_type, _name, _default)                     \
  _type _name = _default;                                                      \
  Input &with_##_name(_type i) {                                               \
    _name = i;                                                                 \
    return *this;                                                              \
  }

namespace atrip {

// src/atrip/Checkpoint.hpp:27-79
struct Checkpoint {
  size_t no = 0, nv = 0;
  size_t nranks = 1;
  size_t nnodes = 1;
  double energy = 0.0;
  size_t iteration = 0;
  bool rank_round_robin = false;
};

inline void write_checkpoint(Checkpoint const &c, std::string const &filepath) {
  std::ofstream out(filepath);
  out << "No: " << c.no << "\n"
      << "Nv: " << c.nv << "\n"
      << "Nranks: " << c.nranks << "\n"
      << "Nnodes: " << c.nnodes << "\n"
      << "Energy: " << std::setprecision(19) << c.energy << "\n"
      << "Iteration: " << c.iteration << "\n"
      << "RankRoundRobin: " << (c.rank_round_robin ? "true" : "false") << "\n";
}

inline Checkpoint read_checkpoint(std::ifstream &in) {
  Checkpoint c;
  auto trim = [](std::string &s, const char *chars) {
    s.erase(0, s.find_first_not_of(chars));
    s.erase(s.find_last_not_of(chars) + 1);
  };
  for (std::string header, value; std::getline(in, header, ':');) {
    std::getline(in, value, '\n');
    trim(value, " \t");
    trim(header, " \t");
    if (header == "No") c.no = std::atoi(value.c_str());
    else if (header == "Nv") c.nv = std::atoi(value.c_str());
    else if (header == "Nranks") c.nranks = std::atoi(value.c_str());
    else if (header == "Nnodes") c.nnodes = std::atoi(value.c_str());
    else if (header == "Energy") c.energy = std::atof(value.c_str());
    else if (header == "Iteration") c.iteration = std::atoi(value.c_str());
    else if (header == "RankRoundRobin") c.rank_round_robin = (!value.empty() && value[0] == 't');
  }
  return c;
}

inline Checkpoint read_checkpoint(std::string const &filepath) {
  std::ifstream in(filepath);
  return read_checkpoint(in);
}

struct Atrip {
  // src/atrip/Atrip.hpp:43-47: process-wide state read by drivers
  // (atrip's bench prints the energy where rank == 0)
  inline static size_t rank = 0;
  inline static size_t np = 1;
  inline static Timings chrono;
  inline static MPI_Comm communicator = MPI_COMM_WORLD;

  // src/atrip/Atrip.cxx:54-63.  One process drives one GPU; with several
  // ranks each runs a contiguous share of the tuple list on its own GPU
  // (device attribute + rank, modulo the GPUs it sees) and the energies are
  // merged at the end.
  static void init(MPI_Comm c) {
    int r = 0, n = 1;
    MPI_Comm_rank(c, &r);
    MPI_Comm_size(c, &n);
    communicator = c;
    rank = (size_t)r;
    np = (size_t)n;
  }

  template <typename F = double>
  struct Input {
    CTF::Tensor<F> *ei = nullptr, *ea = nullptr, *Tph = nullptr, *Tpphh = nullptr,
                   *Vpphh = nullptr, *Vhhhp = nullptr, *Vppph = nullptr, *Jppph = nullptr,
                   *Jhhhp = nullptr;
    Input &with_epsilon_i(CTF::Tensor<F> *t) { ei = t; return *this; }
    Input &with_epsilon_a(CTF::Tensor<F> *t) { ea = t; return *this; }
    Input &with_Tai(CTF::Tensor<F> *t) { Tph = t; return *this; }
    Input &with_Tabij(CTF::Tensor<F> *t) { Tpphh = t; return *this; }
    Input &with_Vabij(CTF::Tensor<F> *t) { Vpphh = t; return *this; }
    Input &with_Vijka(CTF::Tensor<F> *t) { Vhhhp = t; return *this; }
    Input &with_Vabci(CTF::Tensor<F> *t) { Vppph = t; return *this; }
    Input &with_Jijka(CTF::Tensor<F> *t) { Jhhhp = t; return *this; }
    Input &with_Jabci(CTF::Tensor<F> *t) { Jppph = t; return *this; }
    enum TuplesDistribution { NAIVE, GROUP_AND_SORT };

    ATRIP_GB300_ADD_ATTRIBUTE(bool, delete_Vppph, false)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, rank_round_robin, false)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, chrono, false)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, barrier, false)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, blocking, false)
    ATRIP_GB300_ADD_ATTRIBUTE(size_t, max_iterations, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(int, iteration_mod, -1)
    ATRIP_GB300_ADD_ATTRIBUTE(int, percentage_mod, -1)
    ATRIP_GB300_ADD_ATTRIBUTE(TuplesDistribution, tuples_distribution, NAIVE)
    ATRIP_GB300_ADD_ATTRIBUTE(std::string, checkpoint_path, "atrip-checkpoint.yaml")
    ATRIP_GB300_ADD_ATTRIBUTE(bool, read_checkpoint_if_exists, true)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, writeCheckpoint, true)
    ATRIP_GB300_ADD_ATTRIBUTE(float, checkpoint_at_percentage, 10)
    ATRIP_GB300_ADD_ATTRIBUTE(size_t, checkpoint_at_every_iteration, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(bool, ijkabc, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(size_t, ooo_threads, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(size_t, ooo_blocks, 0)
    // GPU attributes (no counterpart in the reference)
    ATRIP_GB300_ADD_ATTRIBUTE(int, form, ATRIP_FORM_FP64)
    ATRIP_GB300_ADD_ATTRIBUTE(int, slices, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(int, device, 0)
    ATRIP_GB300_ADD_ATTRIBUTE(size_t, checkpoint_chunks, 100)
  };

  struct Output {
    double energy;
    double ct_energy;
  };

  template <typename F = double>
  static Output run(Input<F> const &in);

 private:
  template <typename F>
  static Output run_field(Input<F> const &in, int32_t field);
};

namespace detail {

inline void check(int status) {
  if (status != ATRIP_OK) throw std::string(atrip_gpu_last_error());
}

template <typename F>
inline std::vector<F> gather(CTF::Tensor<F> *t, size_t expected) {
  std::vector<F> buf(expected);
  t->read_all(buf.data());
  return buf;
}

struct ContextGuard {
  atrip_gpu_context *c = nullptr;
  ~ContextGuard() { atrip_gpu_destroy(c); }
};

inline void neumaier(double &s, double &c, double x) {
  const double t = s + x;
  c += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
  s = t;
}

// Rank `Atrip::rank`'s contiguous share of tuples first .. end-1 (sizes
// differ by at most one), then every rank's compensated sums gathered and
// merged in rank order -- the role of atrip's final MPI_Reduce
// (src/atrip/Atrip.cxx:1094-1107); every rank returns the total.
// Checkpoints are read but not written across ranks.
inline Atrip::Output run_share(atrip_gpu_context *ctx, atrip_run_options o, size_t first,
                               size_t end, double start_energy, bool ijkabc);

}  // namespace detail

inline Atrip::Output detail::run_share(atrip_gpu_context *ctx, atrip_run_options o, size_t first,
                                       size_t end, double start_energy, bool ijkabc) {
  const size_t n = end > first ? end - first : 0, P = Atrip::np, R = Atrip::rank;
  const size_t base = n / P, extra = n % P;
  const size_t t0 = first + R * base + std::min(R, extra);
  const size_t t1 = t0 + base + (R < extra ? 1 : 0);
  double local[4] = {0.0, 0.0, 0.0, 0.0};
  if (t1 > t0) {
    atrip_result r{};
    if (t1 == 1 && end > 1) {
      // max_iterations = 0 would mean "every tuple": run two, keep the first
      o.first_iteration = 0;
      o.max_iterations = 1;
      check(atrip_gpu_run(ctx, &o, &r));
      check(atrip_gpu_tuple_energies(ctx, 0, 1, &local[0], &local[2]));
    } else {
      o.first_iteration = (int64_t)t0;
      o.max_iterations = (int64_t)t1 - 1;
      check(atrip_gpu_run(ctx, &o, &r));
      check(atrip_gpu_last_sums(ctx, local));
    }
  }
  std::vector<double> all(4 * P);
  MPI_Allgather(local, 4, MPI_DOUBLE, all.data(), 4, MPI_DOUBLE, Atrip::communicator);
  double se = 0, ce = 0, sc = 0, cc = 0;
  for (size_t p = 0; p < P; ++p) {
    neumaier(se, ce, all[4 * p + 0]);
    neumaier(se, ce, all[4 * p + 1]);
    neumaier(sc, cc, all[4 * p + 2]);
    neumaier(sc, cc, all[4 * p + 3]);
  }
  neumaier(se, ce, -start_energy);  // src/atrip/Atrip.cxx:612-616
  const double sign = ijkabc ? 1.0 : -1.0;
  return {sign * (se + ce), sign * (sc + cc)};
}

namespace detail {

}  // namespace detail

// src/atrip/Atrip.cxx:66-1133 on one GPU, for F = double or Complex
// (std::complex<double> is laid out as (re, im), what the C ABI takes for
// ATRIP_FIELD_COMPLEX).
template <typename F>
inline Atrip::Output Atrip::run_field(Atrip::Input<F> const &in, int32_t field) {
  using clock = std::chrono::steady_clock;
  const auto t_start = clock::now();
  if (!in.ei || !in.ea || !in.Tph || !in.Tpphh || !in.Vpphh || !in.Vhhhp || !in.Vppph)
    throw std::string("atrip_gb300: Atrip::run needs ei, ea, Tai, Tabij, Vabij, Vijka, Vabci");
  const size_t No = in.ei->lens[0], Nv = in.ea->lens[0];
  int32_t device = in.device;
  if (np > 1) {
    int32_t count = 0;
    if (atrip_gpu_device_count(&count) == ATRIP_OK && count > 0)
      device = (int32_t)((in.device + rank) % (size_t)count);
  }
  atrip_dims dims{(int32_t)No, (int32_t)Nv, device, field};
  detail::ContextGuard g;
  detail::check(atrip_gpu_create(&dims, &g.c));
  struct Slot {
    CTF::Tensor<F> *t;
    int id;
    size_t n;
  } slots[] = {
      {in.ei, ATRIP_EPSI, No},
      {in.ea, ATRIP_EPSA, Nv},
      {in.Tph, ATRIP_TAI, Nv * No},
      {in.Tpphh, ATRIP_TABIJ, Nv * Nv * No * No},
      {in.Vpphh, ATRIP_VABIJ, Nv * Nv * No * No},
      {in.Vhhhp, ATRIP_VIJKA, No * No * No * Nv},
      {in.Vppph, ATRIP_VABCI, Nv * Nv * Nv * No},
      {in.Jhhhp, ATRIP_JIJKA, No * No * No * Nv},
      {in.Jppph, ATRIP_JABCI, Nv * Nv * Nv * No},
  };
  for (auto &s : slots) {
    if (!s.t) continue;
    std::vector<F> buf = detail::gather(s.t, s.n);
    detail::check(
        atrip_gpu_upload(g.c, s.id, reinterpret_cast<const double *>(buf.data()), (int64_t)s.n));
  }
  if (in.delete_Vppph) delete in.Vppph;  // src/atrip/Atrip.cxx:310

  const size_t n = (size_t)atrip_gpu_n_tuples((int32_t)Nv);
  size_t first = 0;
  double start_energy = 0.0;
  if (in.read_checkpoint_if_exists) {
    std::ifstream fin(in.checkpoint_path);
    if (fin.is_open()) {
      Checkpoint c = read_checkpoint(fin);
      first = c.iteration;
      start_energy = c.energy;
    }
  }
  const size_t mod = in.checkpoint_at_every_iteration != 0
                         ? in.checkpoint_at_every_iteration
                         : (size_t)(n * in.checkpoint_at_percentage / 100);
  const size_t end = in.max_iterations == 0 ? n : std::min(n, in.max_iterations + 1);
  atrip_run_options o{};
  o.form = in.form;
  o.slices = in.slices;
  o.ijkabc = in.ijkabc ? 1 : 0;
  o.use_j = 1;
  Output result{0.0, 0.0};
  atrip_result r{};
  if (np > 1) {
    result = detail::run_share(g.c, o, first, end, start_energy, in.ijkabc);
    chrono["run"].add(std::chrono::duration<double>(clock::now() - t_start).count());
    return result;
  }
  if (mod != 0) {
    o.first_iteration = (int64_t)first;
    o.max_iterations = (int64_t)in.max_iterations;
    o.start_energy = start_energy;
    detail::check(atrip_gpu_run(g.c, &o, &r));
    result = {r.energy, r.ct_energy};
  } else {
    const size_t chunks = in.checkpoint_chunks ? in.checkpoint_chunks : 1;
    const size_t chunk = end > first ? (end - first + chunks - 1) / chunks : 1;
    const double sign = in.ijkabc ? 1.0 : -1.0;
    double ck_energy = start_energy, ct_local = 0.0;
    for (size_t pos = first; pos < end;) {
      write_checkpoint({No, Nv, 1, 1, ck_energy, pos, in.rank_round_robin}, in.checkpoint_path);
      const size_t stop = std::min(end, pos + chunk);
      o.first_iteration = (int64_t)pos;
      o.max_iterations = (int64_t)stop - 1;
      o.start_energy = ck_energy;
      detail::check(atrip_gpu_run(g.c, &o, &r));
      ck_energy = in.ijkabc ? -r.energy : r.energy;
      ct_local += sign * r.ct_energy;
      pos = stop;
      if (IterationDescription::descriptor())
        IterationDescription::descriptor()(
            {pos, n, std::chrono::duration<double>(clock::now() - t_start).count()});
    }
    result = {in.ijkabc ? -ck_energy : ck_energy, sign * ct_local};
    if (end <= first) result.energy = in.ijkabc ? -start_energy : start_energy;
  }
  chrono["iterations"].add(r.device_ms / 1e3);
  chrono["run"].add(std::chrono::duration<double>(clock::now() - t_start).count());
  return result;
}

template <>
inline Atrip::Output Atrip::run<double>(Atrip::Input<double> const &in) {
  return run_field(in, ATRIP_FIELD_REAL);
}

// src/atrip/Atrip.cxx:1136: the Complex instantiation (FP64 form).
template <>
inline Atrip::Output Atrip::run<Complex>(Atrip::Input<Complex> const &in) {
  return run_field(in, ATRIP_FIELD_COMPLEX);
}

}  // namespace atrip

#undef ATRIP_GB300_ADD_ATTRIBUTE

#endif
