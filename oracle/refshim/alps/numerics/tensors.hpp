// Stand-in for ALPSCore's dense tensor (oracle harness only): row-major storage with
// operator()(i0, ..., iN-1) and shape().
#pragma once
#include <array>
#include <cstddef>
#include <vector>

namespace alps {
namespace numerics {

template <typename T, size_t N>
class tensor {
 public:
  tensor() { shape_.fill(0); }
  void reshape(const std::array<size_t, N> &s) {
    shape_ = s;
    size_t t = 1;
    for (size_t i = 0; i < N; ++i) t *= s[i];
    data_.assign(t, T(0));
  }
  const std::array<size_t, N> &shape() const { return shape_; }
  size_t size() const { return data_.size(); }
  T *data() { return data_.data(); }
  template <typename... I>
  T &operator()(I... idx) { return data_[offset(idx...)]; }
  template <typename... I>
  const T &operator()(I... idx) const { return data_[offset(idx...)]; }

 private:
  template <typename... I>
  size_t offset(I... idx) const {
    static_assert(sizeof...(I) == N, "wrong number of tensor indices");
    size_t ids[N] = {size_t(idx)...};
    size_t o = 0;
    for (size_t i = 0; i < N; ++i) o = o * shape_[i] + ids[i];
    return o;
  }
  std::array<size_t, N> shape_;
  std::vector<T> data_;
};

}  // namespace numerics
}  // namespace alps
