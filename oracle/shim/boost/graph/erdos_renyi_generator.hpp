// Boost-API shim (test infrastructure for oracle/_ref). Provides the name
// sorted_erdos_renyi_iterator so the reference's graph_gen.hpp compiles: an
// input iterator over the pairs (u, v), u > v, each kept with probability p,
// visited in sorted order. Its random stream is this shim's own (a uniform
// draw per pair), so graphs from it are not Boost's; the oracle harness never
// calls it for parity data (parity runs on explicit edge lists).
#pragma once
#include <cstddef>
#include <random>
#include <utility>

namespace boost {
template <typename RandomGenerator, typename Graph>
class sorted_erdos_renyi_iterator {
 public:
  using value_type = std::pair<std::size_t, std::size_t>;
  sorted_erdos_renyi_iterator() : done_(true) {}
  sorted_erdos_renyi_iterator(RandomGenerator& gen, std::size_t n, double p)
      : gen_(&gen), n_(n), p_(p), u_(1), v_(0), done_(n < 2) {
    if (!done_ && !keep())
      advance();
  }
  value_type operator*() const { return {u_, v_}; }
  sorted_erdos_renyi_iterator& operator++() {
    advance();
    return *this;
  }
  bool operator==(sorted_erdos_renyi_iterator const& o) const {
    return done_ == o.done_ && (done_ || (u_ == o.u_ && v_ == o.v_));
  }
  bool operator!=(sorted_erdos_renyi_iterator const& o) const {
    return !(*this == o);
  }

 private:
  bool keep() {
    std::uniform_real_distribution<double> d(0.0, 1.0);
    return d(*gen_) < p_;
  }
  void step() {
    if (++v_ == u_) {
      v_ = 0;
      if (++u_ == n_)
        done_ = true;
    }
  }
  void advance() {
    do {
      step();
    } while (!done_ && !keep());
  }
  RandomGenerator* gen_ = nullptr;
  std::size_t n_ = 0;
  double p_ = 0;
  std::size_t u_ = 0, v_ = 0;
  bool done_ = true;
};
}  // namespace boost
