// Device-resident Lanczos for the reference's GreensFunction and ChiLoc on the GPU storage.
//
// The reference's EDLib::gf::Lanczos<Hamiltonian, MeshFactory, Args...> (include/edlib/Lanczos.h:16-231 of the
// reference) runs its recurrence on host vectors through Storage::av / Storage::vv: on the GPU storage that is
// two bus crossings per Lanczos step.  This partial specialisation for
// EDLib::Hamiltonian<EDLib::Storage::GpuStorage<Model, Kind>> keeps the protected interface GreensFunction and
// ChiLoc use -- lanczos(v), compute_continued_fraction, compute_sym_continued_fraction, hamiltonian(), beta(),
// freq_point(), suffix(), zero_freq(), update_static(), omega() -- with the same meaning, but
//   * lanczos(v) uploads the start vector once and runs the whole recurrence of Lanczos.h:36-77 on the device
//     (edgpu_lanczos: alpha/beta with the same indexing and the same beta < 1e-10 stop), and
//   * the continued fractions of every frequency point are evaluated on the device in one call
//     (edgpu_frac_points: get_frac_point's determinant recurrence and FLT_MAX rescaling, Lanczos.h:201-224).
// GreensFunction.h and ChiLoc.h compile unchanged against it.  Include it after the reference's Lanczos.h (the
// reference headers first, as for GpuStorage.h) and before the GreensFunction / ChiLoc of a GPU Hamiltonian
// are instantiated.
#ifndef EDLIB_GPU_GPULANCZOS_H
#define EDLIB_GPU_GPULANCZOS_H

#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "GpuStorage.h"

namespace EDLib {
namespace gf {

template <class ModelT, int Kind, class MeshFactory, typename... Args>
class Lanczos<EDLib::Hamiltonian<EDLib::Storage::GpuStorage<ModelT, Kind>>, MeshFactory, Args...> {
 protected:
  typedef EDLib::Hamiltonian<EDLib::Storage::GpuStorage<ModelT, Kind>> Ham;
  using precision = typename ModelT::precision;
  using Mesh = typename MeshFactory::MeshType;
  using mesh_index = typename Mesh::index_type;

 public:
  static constexpr bool device_resident = true;  // lets a caller check that this specialisation is in use

  Lanczos(alps::params &p, Ham &h, Args... args)
      : _ham(h), _omega(MeshFactory::createMesh(p, args...)), _nl(p["lanc.NLANC"]), _alpha(_nl, 0.0),
        _betal(_nl + 1, 0.0), _beta(p["lanc.BETA"].template as<precision>()) {}

  const Mesh &omega() const { return _omega; }

 protected:
  // Lanczos.h:36-77 on the device: fill the current sector, then the recurrence from v (host, FP64); returns the
  // number of steps.  v is left as it was (the reference leaves its last Lanczos vector there; neither
  // GreensFunction nor ChiLoc reads it afterwards).
  int lanczos(std::vector<precision> &v) {
    _ham.fill();
    std::fill(_alpha.begin(), _alpha.end(), 0.0);
    std::fill(_betal.begin(), _betal.end(), 0.0);
    if (v.empty()) return 0;
    const auto &s = _ham.model().symmetry().sector();
    int nl = 0;
    const int rc = edgpu_lanczos(_ham.storage().handle(), Kind, s.nup(), s.ndown(), v.data(), 1, _nl,
                                 _ham.storage().device_precision(), _alpha.data(), _betal.data(), &nl);
    if (rc < 0) throw std::runtime_error(std::string("edgpu_lanczos: ") + edgpu_last_error(_ham.storage().context()));
    return nl;
  }

  // Lanczos.h:83-100
  template <typename GF_TYPE>
  void compute_continued_fraction(double expectation_value, double excited_state, double groundstate, int nlanc, int isign,
                                  GF_TYPE &gf, const alps::gf::index_mesh::index_type &site,
                                  const alps::gf::index_mesh::index_type &spin) {
    const double expb = boltzmann(excited_state, groundstate);
    const int nw = _omega.extent();
    std::vector<double> ener(2 * nw), out(2 * nw);
    for (int w = 0; w < nw; ++w) {
      const std::complex<double> e = freq_point(w) + excited_state * isign;
      ener[2 * w] = e.real();
      ener[2 * w + 1] = e.imag();
    }
    frac(nlanc, isign, expectation_value, expb, ener, out);
    for (int w = 0; w < nw; ++w) gf(mesh_index(w), site, spin) += std::complex<double>(out[2 * w], out[2 * w + 1]);
  }

  // Lanczos.h:106-124
  template <typename GF_TYPE>
  void compute_sym_continued_fraction(double expectation_value, double excited_state, double groundstate, int nlanc,
                                      int isign, GF_TYPE &gf, const alps::gf::index_mesh::index_type &site) {
    const double expb = boltzmann(excited_state, groundstate);
    update_static(gf, site, expectation_value, expb);
    const int w0 = zero_freq(), nw = _omega.extent(), np = nw - w0;
    if (np <= 0) return;
    std::vector<double> ener(4 * np), out(4 * np);
    for (int q = 0; q < np; ++q) {
      const std::complex<double> e1 = freq_point(w0 + q) + excited_state * isign;
      const std::complex<double> e2 = -freq_point(w0 + q) + excited_state * isign;
      ener[2 * q] = e1.real();
      ener[2 * q + 1] = e1.imag();
      ener[2 * (np + q)] = e2.real();
      ener[2 * (np + q) + 1] = e2.imag();
    }
    frac(nlanc, isign, expectation_value, expb, ener, out);
    for (int q = 0; q < np; ++q)
      gf(mesh_index(w0 + q), site) += std::complex<double>(out[2 * q], out[2 * q + 1]) +
                                      std::complex<double>(out[2 * (np + q)], out[2 * (np + q) + 1]);
  }

  const Ham &hamiltonian() const { return _ham; }
  Ham &hamiltonian() { return _ham; }
  precision beta() const { return _beta; }

  // Lanczos.h:146-148: i w_n on a Matsubara mesh, w + i pi / beta on a real-frequency mesh
  std::complex<double> freq_point(int index) {
    return std::is_base_of<alps::gf::real_frequency_mesh, Mesh>::value
               ? std::complex<double>(_omega.points()[index], M_PI / _beta)
               : std::complex<double>(0.0, _omega.points()[index]);
  }
  std::string suffix() { return std::is_base_of<alps::gf::real_frequency_mesh, Mesh>::value ? "_r" : ""; }
  int zero_freq() { return std::is_base_of<alps::gf::matsubara_positive_mesh, Mesh>::value ? 1 : 0; }
  template <typename GF_TYPE>
  void update_static(GF_TYPE &gf, const alps::gf::index_mesh::index_type &site, double expectation_value, double expb) {
    if (std::is_base_of<alps::gf::matsubara_positive_mesh, Mesh>::value)
      gf(mesh_index(0), site) -= expectation_value * _beta * expb;
  }

 private:
  // the Boltzmann factor of Lanczos.h:87-90
  double boltzmann(double excited_state, double groundstate) const {
    return _beta * (excited_state - groundstate) > 25 ? 0.0 : std::exp(-_beta * (excited_state - groundstate));
  }
  void frac(int nlanc, int isign, double expectation_value, double expb, const std::vector<double> &ener,
            std::vector<double> &out) {
    const int rc = edgpu_frac_points(_ham.storage().context(), _alpha.data(), _betal.data(), nlanc, isign,
                                     expectation_value, expb, ener.data(), (int)(ener.size() / 2), out.data());
    if (rc < 0) throw std::runtime_error(std::string("edgpu_frac_points: ") + edgpu_last_error(_ham.storage().context()));
  }

  Ham &_ham;
  Mesh _omega;
  int _nl;
  std::vector<double> _alpha, _betal;
  precision _beta;
};

}  // namespace gf
}  // namespace EDLib

#endif  // EDLIB_GPU_GPULANCZOS_H
