// Minimal stand-in for ALPSCore's parameter object, written for this project so that the
// reference EDLib headers compile unmodified in the oracle harness.  Only the surface that
// EDLib's hot path touches is provided: p["KEY"] read/write with implicit conversions,
// .as<T>(), exists(), define<T>(...).
#pragma once
#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <sstream>
#include <stdexcept>
#include <cstdlib>
#include <cstddef>

namespace alps {

class params;

class param_value {
 public:
  param_value() = default;
  bool has() const { return set_; }
  void set_str(const std::string &s) { str_ = s; set_ = true; }
  std::string str() const {
    if (!set_) throw std::runtime_error("parameter has no value");
    return str_;
  }
  double num() const {
    std::string s = str();
    if (s == "TRUE" || s == "true" || s == "True") return 1.0;
    if (s == "FALSE" || s == "false" || s == "False") return 0.0;
    char *end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) throw std::runtime_error("parameter is not numeric: " + s);
    return v;
  }

  // assignment from the scalar types the tests and headers use
  param_value &operator=(int v) { set_str(std::to_string(v)); return *this; }
  param_value &operator=(long v) { set_str(std::to_string(v)); return *this; }
  param_value &operator=(unsigned long v) { set_str(std::to_string(v)); return *this; }
  param_value &operator=(bool v) { set_str(v ? "1" : "0"); return *this; }
  param_value &operator=(double v) {
    std::ostringstream o; o.precision(17); o << v; set_str(o.str()); return *this;
  }
  param_value &operator=(const char *v) { set_str(v); return *this; }
  param_value &operator=(const std::string &v) { set_str(v); return *this; }

  operator int() const { return int(num()); }
  operator long() const { return long(num()); }
  operator unsigned long() const { return (unsigned long)(num()); }
  operator double() const { return num(); }
  operator float() const { return float(num()); }
  operator bool() const { return num() != 0.0; }
  operator std::string() const { return str(); }

  template <typename T> T as() const { return T(*this); }

  bool operator==(int v) const { return int(num()) == v; }

 private:
  std::string str_;
  bool set_ = false;
};

template <> inline std::string param_value::as<std::string>() const { return str(); }

class params {
 public:
  params() = default;
  param_value &operator[](const std::string &k) { return map_[k]; }
  const param_value &operator[](const std::string &k) const {
    auto it = map_.find(k);
    if (it == map_.end()) throw std::runtime_error("unknown parameter " + k);
    return it->second;
  }
  bool exists(const std::string &k) const {
    auto it = map_.find(k);
    return it != map_.end() && it->second.has();
  }
  template <typename T, typename D>
  params &define(const std::string &k, const D &def, const std::string &) {
    param_value &v = map_[k];
    if (!v.has()) v = def;
    return *this;
  }
  template <typename T>
  params &define(const std::string &k, const std::string &) {
    map_[k];
    return *this;
  }
 private:
  std::map<std::string, param_value> map_;
};

}  // namespace alps
