// Stand-in for ALPSCore's Green's-function meshes (oracle harness only).
// matsubara_positive_mesh: omega_n = (2n + zeta) pi / beta, n = 0..N-1, zeta = 1 for fermions,
// 0 for bosons.  real_frequency_mesh: points of a linear grid EMIN..EMAX with N points.
#pragma once
#include <cmath>
#include <complex>
#include <cstddef>
#include <vector>

namespace alps {
namespace gf {

namespace statistics {
enum statistics_type { BOSONIC = 0, FERMIONIC = 1 };
}

template <class Mesh>
struct generic_index {
  int i;
  explicit generic_index(int x) : i(x) {}
  int operator()() const { return i; }
};

namespace grid {
class linear_real_frequency_grid {
 public:
  linear_real_frequency_grid(double emin, double emax, int n) : emin_(emin), emax_(emax), n_(n) {}
  std::vector<double> points() const {
    std::vector<double> p(n_);
    for (int i = 0; i < n_; ++i) p[i] = emin_ + (emax_ - emin_) * i / double(n_ - 1);
    return p;
  }
 private:
  double emin_, emax_;
  int n_;
};
}  // namespace grid

class matsubara_positive_mesh {
 public:
  typedef generic_index<matsubara_positive_mesh> index_type;
  matsubara_positive_mesh(double beta, int n, statistics::statistics_type s) : beta_(beta) {
    pts_.resize(n);
    int zeta = (s == statistics::FERMIONIC) ? 1 : 0;
    for (int i = 0; i < n; ++i) pts_[i] = (2.0 * i + zeta) * M_PI / beta;
  }
  const std::vector<double> &points() const { return pts_; }
  int extent() const { return int(pts_.size()); }
 private:
  double beta_;
  std::vector<double> pts_;
};

class real_frequency_mesh {
 public:
  typedef generic_index<real_frequency_mesh> index_type;
  explicit real_frequency_mesh(const grid::linear_real_frequency_grid &g) : pts_(g.points()) {}
  const std::vector<double> &points() const { return pts_; }
  int extent() const { return int(pts_.size()); }
 private:
  std::vector<double> pts_;
};

class index_mesh {
 public:
  typedef generic_index<index_mesh> index_type;
  explicit index_mesh(int n) : pts_(n) { for (int i = 0; i < n; ++i) pts_[i] = i; }
  const std::vector<int> &points() const { return pts_; }
  int extent() const { return int(pts_.size()); }
 private:
  std::vector<int> pts_;
};

typedef index_mesh real_space_index_mesh;

}  // namespace gf
}  // namespace alps
