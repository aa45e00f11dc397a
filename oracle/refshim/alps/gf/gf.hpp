// Stand-in for ALPSCore's Green's-function containers (oracle harness only): dense row-major
// complex storage over two or three meshes, element access, scaling, sums and the max-abs
// norm() the reference tests compare with.
#pragma once
#include <algorithm>
#include <complex>
#include <ostream>
#include <vector>

#include "mesh.hpp"

namespace alps {
namespace gf {

template <typename T, class M1, class M2, class M3>
class three_index_gf {
 public:
  three_index_gf(const M1 &m1, const M2 &m2, const M3 &m3)
      : m1_(m1), m2_(m2), m3_(m3), d_(size_t(m1.extent()) * m2.extent() * m3.extent(), T(0)) {}
  T &operator()(typename M1::index_type a, typename M2::index_type b, typename M3::index_type c) {
    return d_[(size_t(a.i) * m2_.extent() + b.i) * m3_.extent() + c.i];
  }
  const T &operator()(typename M1::index_type a, typename M2::index_type b, typename M3::index_type c) const {
    return d_[(size_t(a.i) * m2_.extent() + b.i) * m3_.extent() + c.i];
  }
  three_index_gf &operator*=(double s) { for (auto &x : d_) x *= s; return *this; }
  three_index_gf &operator/=(double s) { for (auto &x : d_) x /= s; return *this; }
  three_index_gf &operator-=(const three_index_gf &o) {
    for (size_t i = 0; i < d_.size(); ++i) d_[i] -= o.d_[i];
    return *this;
  }
  three_index_gf operator+(const three_index_gf &o) const {
    three_index_gf r(*this);
    for (size_t i = 0; i < d_.size(); ++i) r.d_[i] += o.d_[i];
    return r;
  }
  double norm() const {
    double m = 0;
    for (auto &x : d_) m = std::max(m, std::abs(x));
    return m;
  }
  const M1 &mesh1() const { return m1_; }
  const M2 &mesh2() const { return m2_; }
  const M3 &mesh3() const { return m3_; }
  const std::vector<T> &data() const { return d_; }

 private:
  M1 m1_;
  M2 m2_;
  M3 m3_;
  std::vector<T> d_;
};

template <typename T, class M1, class M2>
class two_index_gf {
 public:
  two_index_gf(const M1 &m1, const M2 &m2) : m1_(m1), m2_(m2), d_(size_t(m1.extent()) * m2.extent(), T(0)) {}
  T &operator()(typename M1::index_type a, typename M2::index_type b) { return d_[size_t(a.i) * m2_.extent() + b.i]; }
  const T &operator()(typename M1::index_type a, typename M2::index_type b) const {
    return d_[size_t(a.i) * m2_.extent() + b.i];
  }
  two_index_gf &operator*=(double s) { for (auto &x : d_) x *= s; return *this; }
  two_index_gf &operator/=(double s) { for (auto &x : d_) x /= s; return *this; }
  two_index_gf &operator-=(const two_index_gf &o) {
    for (size_t i = 0; i < d_.size(); ++i) d_[i] -= o.d_[i];
    return *this;
  }
  double norm() const {
    double m = 0;
    for (auto &x : d_) m = std::max(m, std::abs(x));
    return m;
  }
  const M1 &mesh1() const { return m1_; }
  const M2 &mesh2() const { return m2_; }
  const std::vector<T> &data() const { return d_; }

 private:
  M1 m1_;
  M2 m2_;
  std::vector<T> d_;
};

}  // namespace gf
}  // namespace alps
