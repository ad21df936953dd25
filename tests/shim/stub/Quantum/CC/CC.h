// Stand-ins for the few Eigen and SCESS types that the C++ shim of
// INTEGRATION.md uses, so that the shim compiles, links against
// libscess_cc.so and runs in this repository's tests without Eigen or the
// SCESS sources.  Only what the shim touches is defined: dense column-major
// tensors with dimension() and data(), a vector of doubles, the cancellation
// handle and the two result types, with the call signatures of
// src/Quantum/CC/CC.h:136-158.
#pragma once
#include <array>
#include <cstddef>
#include <sstream>
#include <stdexcept>
#include <vector>

namespace Eigen {
using Index = std::ptrdiff_t;

// Dense rank-R tensor, column-major (first index fastest) like Eigen's default.
template <class T, int R>
class Tensor {
 public:
  Tensor() = default;
  template <class... I>
  explicit Tensor(I... d) : dims_{static_cast<Index>(d)...} {
    static_assert(sizeof...(I) == R, "one extent per rank");
    Index n = 1;
    for (Index x : dims_) n *= x;
    v_.assign(static_cast<size_t>(n), T(0));
  }
  Index dimension(int k) const { return dims_[k]; }
  T *data() { return v_.data(); }
  const T *data() const { return v_.data(); }

 private:
  std::array<Index, R> dims_{};
  std::vector<T> v_;
};

class VectorXd {
 public:
  explicit VectorXd(Index n = 0) : v_(static_cast<size_t>(n)) {}
  Index size() const { return static_cast<Index>(v_.size()); }
  double *data() { return v_.data(); }
  const double *data() const { return v_.data(); }

 private:
  std::vector<double> v_;
};
}  // namespace Eigen

namespace DH {
class Thread {
 public:
  bool ShouldStop() const { return stop; }
  bool stop = false;
};
}  // namespace DH

namespace SCESS::CC {
using TEITensor = Eigen::Tensor<double, 4>;
using T1Tensor = Eigen::Tensor<double, 2>;
using T2Tensor = Eigen::Tensor<double, 4>;

struct RCCSD_Wfn {
  double E_CCSD = 0.0;
  double E_F12_Coupling = 0.0;
  double E_T = 0.0;
  bool converged = false;
  T1Tensor t1;
  T2Tensor t2;
};

struct RCCSD_F12Coupling {
  T2Tensor residual;
  T2Tensor energy;
};

RCCSD_Wfn SolveRCCSD_DIIS(const TEITensor &eri, const Eigen::VectorXd &orbitalEnergies,
                          Eigen::Index nOcc, const RCCSD_F12Coupling *f12 = nullptr,
                          const DH::Thread *thread = nullptr,
                          std::stringstream *console = nullptr);
double RCCSD_TriplesCorrection(const TEITensor &eri, const Eigen::VectorXd &orbitalEnergies,
                               Eigen::Index nOcc, const T1Tensor &t1, const T2Tensor &t2,
                               const DH::Thread *thread = nullptr);
}  // namespace SCESS::CC
