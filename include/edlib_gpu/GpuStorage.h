// EDLib Storage concept on the GB300 library: a drop-in storage for EDLib::Hamiltonian<Storage>.
//
// The reference's plug-in point is a compile-time Storage class (include/edlib/CRSStorage.h,
// SpinResolvedStorage.h, SOCRSStorage.h of the reference).  GpuStorage<Model, kind> implements the same
// members with the same meaning -- fill, reset, init, diag, eigenvalues, eigenvectors, av, a_adag, vv,
// vector_size, prepare_work_arrays, finalize, zero_eigenapair -- on top of the C ABI in edgpu.h, so
//
//   typedef EDLib::Hamiltonian<EDLib::Storage::GpuSpinResolvedStorage<EDLib::Model::HubbardModel<double>>> Ham;
//
// drives the reference's own Hamiltonian, GreensFunction, ChiLoc and StaticObservables templates
// unchanged.  Those templates call av()/vv()/a_adag() on host vectors, so each Lanczos step crosses
// PCIe/C2C; GpuLanczos.h keeps the recurrences and continued fractions of GreensFunction / ChiLoc on the
// device, and edgpu_greens_function / edgpu_chiloc (see edgpu.h) batch all of them.
//
// Requirements: the reference headers (EDLib::Storage::Storage, the models, alps::params /
// alps::hdf5) are included before this header; the model parameters are read from INPUT_FILE with the
// same dataset paths the reference models use (HubbardModel.h:55-67, SingleImpurityAndersonModel.h:199-222).
#ifndef EDLIB_GPU_GPUSTORAGE_H
#define EDLIB_GPU_GPUSTORAGE_H

#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../edgpu.h"

namespace EDLib {
namespace Storage {

template <class ModelType, int Kind>
class GpuStorage : public Storage<typename ModelType::precision> {
  static_assert(std::is_same<typename ModelType::precision, double>::value,
                "GpuStorage exchanges FP64 host vectors (the device precision is chosen separately)");

 public:
  typedef ModelType Model;
  typedef typename Model::precision prec;
  using Storage<prec>::n;
  using Storage<prec>::ntot;

  GpuStorage(alps::params &p, Model &m)
      : Storage<prec>(p), _model(m), _nev(p["arpack.NEV"]), _eval_only(p["storage.EIGENVALUES_ONLY"]) {
    _ncv = p.exists("arpack.NCV") ? int(p["arpack.NCV"]) : 2 * _nev + 3;
    _prec = (p.exists("gpu.PRECISION") && std::string(p["gpu.PRECISION"].template as<std::string>()) == "fp32")
                ? EDGPU_FP32 : EDGPU_FP64;
    check(edgpu_ctx_create(&_ctx, 0, 0), "edgpu_ctx_create");
    const int ns = p["NSITES"];
    std::string input = p["INPUT_FILE"];
    alps::hdf5::archive ar(input.c_str(), "r");
    int rc;
    if (std::is_base_of<::EDLib::Model::HubbardModel<prec>, Model>::value) {
      std::vector<std::vector<double>> t, J(ns, std::vector<double>(ns, 0.0));
      std::vector<double> U, mu, h(ns, 0.0);
      ar >> alps::make_pvp("hopping/values", t);
      ar >> alps::make_pvp("interaction/values", U);
      ar >> alps::make_pvp("chemical_potential/values", mu);
      if (ar.is_data("magnetic_field/values")) ar >> alps::make_pvp("magnetic_field/values", h);
      bool hasJ = ar.is_data("exchange/values");
      if (hasJ) ar >> alps::make_pvp("exchange/values", J);
      std::vector<double> tf, Jf;
      for (auto &r : t) tf.insert(tf.end(), r.begin(), r.end());
      for (auto &r : J) Jf.insert(Jf.end(), r.begin(), r.end());
      rc = edgpu_model_hubbard(_ctx, ns, tf.data(), U.data(), mu.data(), h.data(), hasJ ? Jf.data() : nullptr, &_m);
    } else {
      const int ml = p["siam.NORBITALS"];
      std::vector<std::vector<double>> epsk;
      std::vector<double> ef, vf, hf;
      ar >> alps::make_pvp("Bath/Epsk/values", epsk);
      for (auto &r : epsk) ef.insert(ef.end(), r.begin(), r.end());
      for (int im = 0; im < ml; ++im) {
        std::vector<std::vector<double>> vk, h0;
        ar >> alps::make_pvp("Bath/Vk_" + std::to_string(im) + "/values", vk);
        ar >> alps::make_pvp("H0_" + std::to_string(im) + "/values", h0);
        for (auto &r : vk) vf.insert(vf.end(), r.begin(), r.end());
        for (auto &r : h0) hf.insert(hf.end(), r.begin(), r.end());
      }
      double mu;
      ar >> alps::make_pvp("mu", mu);
      alps::numerics::tensor<double, 6> Ut;
      ar >> alps::make_pvp("interaction/values", Ut);
      std::vector<double> uf(Ut.data(), Ut.data() + Ut.size());
      rc = edgpu_model_siam(_ctx, ns, ml, ef.data(), vf.data(), hf.data(), mu, uf.data(), &_m);
    }
    ar.close();
    check(rc, "model upload");
    edgpu_model_set_limits(_m, Kind == EDGPU_SRS ? 0 : size_t(p["storage.MAX_DIM"]),
                           Kind == EDGPU_SRS ? 0 : size_t(p["storage.MAX_SIZE"]));
  }

  ~GpuStorage() {
    if (_m) edgpu_model_destroy(_m);
    if (_ctx) edgpu_ctx_destroy(_ctx);
  }

  // Storage::fill / reset / init (e.g. SpinResolvedStorage.h:120-250)
  void fill() {
    reset();
    long long dim = 0;
    const auto &s = _model.symmetry().sector();
    check(edgpu_fill(_m, Kind, s.nup(), s.ndown(), &dim), "fill");
    _zero = 0;
    if (dim == 1) {
      std::vector<double> e(1), one(1, 1.0);
      av(one.data(), e.data(), 1, true);
      _zero = e[0];
    }
  }
  void reset() {
    _model.symmetry().init();
    ntot() = int(_model.symmetry().sector().size());
    n() = ntot();
  }
  void init() { _model.symmetry().init(); }

  // Storage::diag (Storage.h:43-146) on the device; eigen-pairs copied into the base's containers
  int diag() {
    if (n() == 0) return 0;
    if (ntot() == 1) {
      zero_eigenapair();
      return 0;
    }
    const auto &s = _model.symmetry().sector();
    edgpu_diag_params dp{};
    dp.storage = Kind;
    dp.precision = _prec;
    dp.nev = _nev;
    dp.ncv = _ncv;
    dp.eigenvalues_only = _eval_only;
    std::vector<double> ev(_nev + 1), vecs;
    if (!_eval_only) vecs.assign(size_t(_nev + 1) * n(), 0.0);
    int nconv = 0;
    int rc = edgpu_diag_sector(_m, &dp, s.nup(), s.ndown(), ev.data(), &nconv, _eval_only ? nullptr : vecs.data(), n());
    if (rc < 0) return rc;
    this->eigenvalues().assign(ev.begin(), ev.begin() + nconv);
    if (_eval_only) {
      this->eigenvectors().assign(nconv, std::vector<prec>(1, prec(0.0)));
    } else {
      this->eigenvectors().assign(nconv, std::vector<prec>());
      for (int q = 0; q < nconv; ++q)
        this->eigenvectors()[q].assign(vecs.begin() + size_t(q) * n(), vecs.begin() + size_t(q + 1) * n());
    }
    return 0;
  }

  virtual void zero_eigenapair() {
    this->eigenvalues().assign(1, _zero);
    this->eigenvectors().assign(1, std::vector<prec>(1, prec(1.0)));
  }

  // Storage::av (w = H v, or w += H v with clear == false) on host vectors
  virtual void av(prec *v, prec *w, int nn, bool clear = true) { check(edgpu_av(_m, v, w, nn, clear ? 1 : 0, _prec), "av"); }

  prec vv(const std::vector<prec> &v, const std::vector<prec> &w) {
    double r = 0;
    check(edgpu_vv(_m, v.data(), w.data(), (long long)v.size(), &r), "vv");
    return r;
  }

  void a_adag(int i, const std::vector<prec> &invec, std::vector<prec> &outvec, const typename Model::Sector &next,
              bool a) {
    const auto &s = _model.symmetry().sector();
    check(edgpu_a_adag(_m, i, s.nup(), s.ndown(), next.nup(), next.ndown(), invec.data(), outvec.data(), a ? 1 : 0),
          "a_adag");
  }

  size_t vector_size(typename Model::Sector sector) { return sector.size(); }

  // the library handles behind this storage (for GpuLanczos.h and callers of the C ABI)
  edgpu_model *handle() const { return _m; }
  edgpu_ctx *context() const { return _ctx; }
  int device_precision() const { return _prec; }
  void constant_shift(prec) { throw std::logic_error("constant_shift is not supported on the GPU storage"); }

 private:
  void check(int rc, const char *what) {
    if (rc < 0) {
      std::ostringstream o;
      o << what << ": " << edgpu_last_error(_ctx);
      if (rc == EDGPU_ERR_CAPACITY) throw std::runtime_error(o.str());
      if (rc == EDGPU_ERR_COLLISION) throw std::logic_error(o.str());
      throw std::runtime_error(o.str());
    }
  }
  Model &_model;
  edgpu_ctx *_ctx = nullptr;
  edgpu_model *_m = nullptr;
  int _nev, _ncv, _eval_only, _prec;
  double _zero = 0;
};

template <class M>
using GpuSpinResolvedStorage = GpuStorage<M, EDGPU_SRS>;
template <class M>
using GpuCRSStorage = GpuStorage<M, EDGPU_CRS>;
template <class M>
using GpuSOCRSStorage = GpuStorage<M, EDGPU_SOCRS>;

}  // namespace Storage
}  // namespace EDLib

#endif  // EDLIB_GPU_GPUSTORAGE_H
