// Stand-in for ALPSCore's HDF5 archive (oracle harness only).  HDF5 is not available, so the
// "archive" is a plain text file holding the same dataset paths the reference reads:
//
//   data <path> <ndim> <dim_0> ... <dim_{ndim-1}> <values, row-major>
//   param <KEY> <VALUE>            (ignored here; read by the harness)
//
// Reading a path fills std::vector nests, scalars and alps::numerics::tensor objects.
#pragma once
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "numerics/tensors.hpp"

namespace alps {

template <typename T>
struct pvp_ref {
  std::string path;
  T *obj;
};

template <typename T>
pvp_ref<T> make_pvp(const std::string &path, T &obj) { return pvp_ref<T>{path, &obj}; }

namespace hdf5 {

struct dataset {
  std::vector<size_t> shape;
  std::vector<double> values;
};

class archive {
 public:
  archive() = default;
  archive(const std::string &path, const std::string &mode = "r") { open(path, mode); }
  void open(const std::string &path, const std::string &mode = "r") {
    if (mode != "r") { writable_ = true; return; }
    std::ifstream in(path.c_str());
    if (!in) throw std::runtime_error("cannot open model input " + path);
    std::string tok;
    while (in >> tok) {
      if (tok == "data") {
        std::string name; size_t nd;
        in >> name >> nd;
        dataset d;
        size_t total = 1;
        for (size_t i = 0; i < nd; ++i) { size_t s; in >> s; d.shape.push_back(s); total *= s; }
        d.values.resize(total);
        for (size_t i = 0; i < total; ++i) in >> d.values[i];
        data_[name] = d;
      } else if (tok == "param") {
        std::string k, v; in >> k >> v;
      } else if (!tok.empty() && tok[0] == '#') {
        std::string rest; std::getline(in, rest);
      } else {
        throw std::runtime_error("bad token in model input: " + tok);
      }
    }
  }
  void close() {}
  bool is_data(const std::string &p) const { return data_.count(p) != 0; }

  // write access exists only so the reference's save() members type-check; the harness never saves
  struct write_proxy {
    template <typename T>
    write_proxy &operator<<(const T &) { throw std::logic_error("archive writing is not available"); }
  };
  write_proxy operator[](const std::string &) { return write_proxy(); }

  template <typename T>
  archive &operator>>(const pvp_ref<T> &r) {
    auto it = data_.find(r.path);
    if (it == data_.end()) throw std::runtime_error("dataset not found: " + r.path);
    size_t pos = 0;
    fill(*r.obj, it->second, 0, pos);
    return *this;
  }

 private:
  template <typename T>
  static typename std::enable_if<std::is_arithmetic<T>::value>::type
  fill(T &v, const dataset &d, size_t, size_t &pos) { v = T(d.values.at(pos++)); }

  template <typename T>
  static void fill(std::vector<T> &v, const dataset &d, size_t dim, size_t &pos) {
    if (dim >= d.shape.size()) throw std::runtime_error("dataset rank mismatch");
    v.resize(d.shape[dim]);
    for (auto &x : v) fill(x, d, dim + 1, pos);
  }

  template <typename T, size_t N>
  static void fill(alps::numerics::tensor<T, N> &t, const dataset &d, size_t, size_t &pos) {
    if (d.shape.size() != N) throw std::runtime_error("tensor rank mismatch");
    std::array<size_t, N> sh;
    for (size_t i = 0; i < N; ++i) sh[i] = d.shape[i];
    t.reshape(sh);
    for (size_t i = 0; i < t.size(); ++i) t.data()[i] = T(d.values.at(pos++));
  }

  std::map<std::string, dataset> data_;
  bool writable_ = false;
};

}  // namespace hdf5
}  // namespace alps
