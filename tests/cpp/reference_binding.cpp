// The GPU storage plugged into the reference's own Hamiltonian / GreensFunction / ChiLoc templates, with the
// device-resident Lanczos specialisation.
// Compiled against the reference headers and the oracle's stand-in headers (alps, Eigen).
#include "edlib/EDParams.h"
#include "edlib/Hamiltonian.h"
#include "edlib/GreensFunction.h"
#include "edlib/ChiLoc.h"
#include "edlib/MeshFactory.h"
#include "edlib_gpu/GpuStorage.h"
#include "edlib_gpu/GpuLanczos.h"  // GreensFunction / ChiLoc recurrences and fractions on the device

typedef EDLib::Hamiltonian<EDLib::Storage::GpuSpinResolvedStorage<EDLib::Model::HubbardModel<double>>> HamType;
typedef EDLib::Hamiltonian<EDLib::Storage::GpuCRSStorage<EDLib::Model::SingleImpurityAndersonModel<double>>> SiamType;

// the reference's GreensFunction / ChiLoc of a GPU Hamiltonian derive from the device-resident Lanczos
static_assert(EDLib::gf::Lanczos<HamType, EDLib::MatsubaraMeshFactory,
                                 alps::gf::statistics::statistics_type>::device_resident,
              "GpuLanczos.h specialisation not selected");

int main(int argc, char **argv) {
  alps::params p;
  EDLib::define_parameters(p);
  p["INPUT_FILE"] = argc > 1 ? argv[1] : "input.txt";
  try {
    HamType ham(p);
    ham.diag();
    EDLib::gf::GreensFunction<HamType, EDLib::MatsubaraMeshFactory, alps::gf::statistics::statistics_type> gf(
        p, ham, alps::gf::statistics::statistics_type::FERMIONIC);
    gf.compute();
    EDLib::gf::ChiLoc<HamType, EDLib::MatsubaraMeshFactory, alps::gf::statistics::statistics_type> chi(
        p, ham, alps::gf::statistics::statistics_type::BOSONIC);
    chi.compute();
    SiamType siam(p);
    std::cout << ham.eigenpairs().begin()->eigenvalue() << std::endl;
  } catch (std::exception &e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
