/* Dense, single-process stand-in for the subset of Cyclops (CTF) that the
 * atrip reference calls: World, Tensor<F>{order, lens, data, read_all,
 * slice} and the NS symmetry tag (src/atrip/SliceUnion.cxx:308-317,
 * src/atrip/Unions.hpp:21-75, src/atrip/Atrip.cxx:72-73,179-181); and what
 * atrip's own driver (bench/main.cxx) calls on top: World(argc, argv) and
 * its np, fill_random, read_dense_from_file, norm2, index-labelled
 * assignment (T["ijab"] = S["abij"]) and Transform<A, B>(f)(S["i"], T["i"]).
 *
 * Test infrastructure only.  Storage is column-major (first index fastest),
 * which is the element order CTF's read_all returns for a dense tensor and
 * the order every slice offset in src/atrip/Unions.hpp assumes.
 */
#ifndef ORACLE_CTF_SHIM_HPP
#define ORACLE_CTF_SHIM_HPP

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cmath>
#include <iostream>
#include <iomanip>
#include <sstream>
#include <fstream>
#include <functional>
#include <random>
#include <complex>
#include <mpi.h>

using namespace std; // the reference relies on a transitive `using` (src/atrip/Tuples.hpp:68)

/* CTF declares its symmetry tags at global scope. */
enum ORACLE_CTF_SYM : int { NS = 0, SY = 1, AS = 2, SH = 3 };

namespace CTF {



class World {
public:
  explicit World(MPI_Comm c = MPI_COMM_WORLD) : comm(c) {}
  World(int, char **) : comm(MPI_COMM_WORLD) {}
  MPI_Comm comm;
  int np = 1;
};

template <typename F> class Tensor;

/* A tensor with one index label per mode ("abij"): the operand of labelled
 * assignments and transforms.  Modes with equal labels are matched. */
template <typename F>
struct Idx_Tensor {
  Tensor<F> *t;
  std::string idx;
  /* this[labels] = other[labels]: a permutation of the modes */
  Idx_Tensor &operator=(const Idx_Tensor &o) {
    Tensor<F>::assign_permuted(*t, idx, *o.t, o.idx);
    return *this;
  }
};

/* Transform<A, B>(f)(S["..."], T["..."]) calls f(s, t) for every pair of
 * elements of S and T at matching labels; f updates t in place. */
template <typename A, typename B = A>
class Transform {
public:
  explicit Transform(std::function<void(A, B &)> f) : f_(f) {}
  void operator()(const Idx_Tensor<A> &s, const Idx_Tensor<B> &t) const {
    Tensor<B> &T = *t.t;
    const Tensor<A> &S = *s.t;
    std::vector<int> perm = label_map(t.idx, s.idx);
    std::vector<int> idx(T.order, 0);
    for (std::int64_t n = 0; n < T.size; ++n) {
      std::int64_t lin = 0, stride = 1;
      for (int d = 0; d < S.order; ++d) { lin += idx[perm[d]] * stride; stride *= S.lens[d]; }
      f_(S.data[lin], T.data[n]);
      for (int d = 0; d < T.order; ++d) { if (++idx[d] < T.lens[d]) break; idx[d] = 0; }
    }
  }
  /* for each mode of `src`, the mode of `dst` with the same label */
  static std::vector<int> label_map(const std::string &dst, const std::string &src) {
    std::vector<int> m(src.size());
    for (std::size_t d = 0; d < src.size(); ++d) {
      const std::size_t p = dst.find(src[d]);
      if (p == std::string::npos) throw std::string("ctf shim: unmatched index label");
      m[d] = (int)p;
    }
    return m;
  }

private:
  std::function<void(A, B &)> f_;
};

template <typename F = double>
class Tensor {
public:
  int order = 0;
  int *lens = nullptr;
  F *data = nullptr;
  std::int64_t size = 0;

  Tensor(int order_, const int *lens_, const int *, World &) { init(order_, lens_); }
  Tensor(int order_, const int *lens_) { init(order_, lens_); }
  Tensor(const Tensor &o) { init(o.order, o.lens); std::memcpy(data, o.data, sizeof(F) * size); }
  Tensor &operator=(const Tensor &) = delete;
  ~Tensor() { delete[] lens; delete[] data; }

  void read_all(F *out) const { std::memcpy(out, data, sizeof(F) * size); }

  Idx_Tensor<F> operator[](const char *idx) { return Idx_Tensor<F>{this, idx}; }

  /* uniform random values in [a, b) (a fixed-seed stream: reproducible) */
  void fill_random(F a, F b) {
    std::mt19937_64 gen(0x5eed + (std::uint64_t)size);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (std::int64_t n = 0; n < size; ++n) data[n] = a + (b - a) * F(u(gen));
  }
  /* dense column-major binary file of `size` elements */
  void read_dense_from_file(const char *path) {
    std::ifstream in(path, std::ios::binary);
    if (!in.read(reinterpret_cast<char *>(data), sizeof(F) * size))
      throw std::string("ctf shim: cannot read ") + path;
  }
  double norm2() const {
    double s = 0.0;
    for (std::int64_t n = 0; n < size; ++n) s += std::norm(data[n]);
    return std::sqrt(s);
  }
  static void assign_permuted(Tensor &dst, const std::string &di, const Tensor &src,
                              const std::string &si) {
    Transform<F, F>([](F s, F &d) { d = s; })(Idx_Tensor<F>{const_cast<Tensor *>(&src), si},
                                               Idx_Tensor<F>{&dst, di});
  }

  /* this[offsets:ends] = beta * this[offsets:ends] + alpha * A[offsets_A:ends_A].
   * Both blocks are walked in column-major order; the reference only ever
   * pairs blocks with equal element counts whose extra extents are 1. */
  void slice(const int *offsets, const int *ends, F beta, const Tensor &A,
             const int *offsets_A, const int *ends_A, F alpha) {
    std::vector<std::int64_t> dst = block_indices(order, lens, offsets, ends);
    std::vector<std::int64_t> src = block_indices(A.order, A.lens, offsets_A, ends_A);
    if (dst.size() != src.size()) throw std::string("ctf shim: slice size mismatch");
    for (std::size_t n = 0; n < dst.size(); ++n)
      data[dst[n]] = beta * data[dst[n]] + alpha * A.data[src[n]];
  }

private:
  void init(int order_, const int *lens_) {
    order = order_;
    lens = new int[order_ > 0 ? order_ : 1];
    size = 1;
    for (int d = 0; d < order_; ++d) { lens[d] = lens_[d]; size *= lens_[d]; }
    data = new F[size]();
  }
  static std::vector<std::int64_t> block_indices(int ord, const int *ln,
                                                 const int *lo, const int *up) {
    std::vector<std::int64_t> out;
    std::vector<int> idx(lo, lo + ord);
    std::int64_t total = 1;
    for (int d = 0; d < ord; ++d) total *= (up[d] - lo[d]);
    out.reserve(total);
    for (std::int64_t n = 0; n < total; ++n) {
      std::int64_t lin = 0, stride = 1;
      for (int d = 0; d < ord; ++d) { lin += idx[d] * stride; stride *= ln[d]; }
      out.push_back(lin);
      for (int d = 0; d < ord; ++d) {
        if (++idx[d] < up[d]) break;
        idx[d] = lo[d];
      }
    }
    return out;
  }
};

} // namespace CTF

#endif
