/* Dense, single-process stand-in for the subset of Cyclops (CTF) that the
 * atrip reference calls: World, Tensor<F>{order, lens, data, read_all,
 * slice} and the NS symmetry tag (src/atrip/SliceUnion.cxx:308-317,
 * src/atrip/Unions.hpp:21-75, src/atrip/Atrip.cxx:72-73,179-181).
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
#include <mpi.h>

using namespace std; // the reference relies on a transitive `using` (src/atrip/Tuples.hpp:68)

/* CTF declares its symmetry tags at global scope. */
enum ORACLE_CTF_SYM : int { NS = 0, SY = 1, AS = 2, SH = 3 };

namespace CTF {



class World {
public:
  explicit World(MPI_Comm c = MPI_COMM_WORLD) : comm(c) {}
  MPI_Comm comm;
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
