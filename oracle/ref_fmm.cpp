/*
 * ref_fmm.cpp -- TEST INFRASTRUCTURE.  Builds the reference's own CPU FMM for
 * the two products of the step into oracle/_ref/libmfref_fmm.so (see
 * oracle/Makefile), so its speed and accuracy can be measured beside this
 * build's.  Compiled only where the reference sources are present.
 *
 * One product is fmmtl::kernel_matrix<E>(E{P}, points, points) * charges
 * (fmmtl_minimum/fmmtl/KernelMatrix.hpp:127-131) with the set-up of
 * magnetic_solver/magnetic_force.cu:660-672: the expansion's smoothing length
 * m_h = h, FMMOptions{h, true} (FMMOptions.hpp:55-116: the theta criterion
 * plus the 3h separation), ncrit, theta.  E is
 *   kind 0: DipoleBSpherical        (fmmtl_minimum/kernel/DipoleBSpherical.hpp)
 *   kind 1: DipoleHessianSpherical  (fmmtl_minimum/kernel/DipoleHessianSpherical.hpp)
 * in the reference's FP64 expansions and FP32 kernels, on the CPU (OpenMP).
 * Arrays are AoS float [n][3]; tensors are [n][9] glm column-major.
 */
#include "kernel/DipoleBSpherical.hpp"
#include "kernel/DipoleHessianSpherical.hpp"
#include "fmmtl/KernelMatrix.hpp"

#include <chrono>
#include <cstdint>
#include <deque>
#include <queue>
#include <vector>

// FMMTL's breadth-first traversal (fmmtl/traversal/DualTraversal.hpp:35-46)
// writes `return q.emplace(...)` in a void function, which holds only while
// std::queue::emplace returns void (before C++17); the CUDA 13 CCCL headers
// need C++17.  The queue of box pairs of the 3-D tree is given here with the
// pre-C++17 interface the traversal uses, so the reference's headers compile
// unmodified and traverse as written.
namespace std {
template <>
class queue<std::pair<fmmtl::NDTree<3>::box_type, fmmtl::NDTree<3>::box_type>,
            std::deque<std::pair<fmmtl::NDTree<3>::box_type, fmmtl::NDTree<3>::box_type>>> {
  using T = std::pair<fmmtl::NDTree<3>::box_type, fmmtl::NDTree<3>::box_type>;
  std::deque<T> d_;

 public:
  bool empty() const { return d_.empty(); }
  T& front() { return d_.front(); }
  const T& front() const { return d_.front(); }
  void pop() { d_.pop_front(); }
  void push(const T& v) { d_.push_back(v); }
  template <class... Args>
  void emplace(Args&&... args) {
    d_.emplace_back(std::forward<Args>(args)...);
  }
};
}  // namespace std

namespace {

template <class E, class Out>
int run(int64_t n, const float* pos, const float* mom, float h, int P, int ncrit, double theta, int reps, Out out,
        double* seconds) {
  typedef typename E::source_type S;
  typedef typename E::charge_type C;
  typedef typename E::result_type R;
  std::vector<S> pts(static_cast<size_t>(n));
  std::vector<C> chg(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    pts[size_t(i)] = S{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    chg[size_t(i)] = C{mom[3 * i], mom[3 * i + 1], mom[3 * i + 2]};
  }
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  fmmtl::kernel_matrix<E> A(E{P}, pts, pts);
  A.kernel().m_h = h;
  FMMOptions opts{double(h), true};
  opts.ncrit = unsigned(ncrit);
  opts.theta = theta;
  A.set_options(opts);
  std::vector<R> res = A * chg;  // the first product builds the plan
  const auto t1 = clock::now();
  for (int r = 0; r < reps; ++r) res = A * chg;
  const auto t2 = clock::now();
  seconds[0] = std::chrono::duration<double>(t1 - t0).count();
  seconds[1] = reps > 0 ? std::chrono::duration<double>(t2 - t1).count() / reps : 0.0;
  for (int64_t i = 0; i < n; ++i) out(i, res[size_t(i)]);
  return 0;
}

}  // namespace

// seconds[0]: set-up and first product (tree, lists, plan); seconds[1]: one
// further product on the same plan (mean of reps).
extern "C" int ref_fmm_field(int64_t n, const float* pos, const float* mom, float h, int P, int ncrit,
                             double theta, int reps, float* out, double* seconds) {
  return run<fmmtl::DipoleBSpherical>(n, pos, mom, h, P, ncrit, theta, reps,
                                      [&](int64_t i, const Vec<3, float>& v) {
                                        for (int k = 0; k < 3; ++k) out[3 * i + k] = float(v[k]);
                                      },
                                      seconds);
}

extern "C" int ref_fmm_hessian(int64_t n, const float* pos, const float* mom, float h, int P, int ncrit,
                               double theta, int reps, float* out9, double* seconds) {
  return run<fmmtl::DipoleHessianSpherical>(n, pos, mom, h, P, ncrit, theta, reps,
                                            [&](int64_t i, const glm::mat3& m) {
                                              for (int c = 0; c < 3; ++c)
                                                for (int r = 0; r < 3; ++r) out9[9 * i + 3 * c + r] = m[c][r];
                                            },
                                            seconds);
}
