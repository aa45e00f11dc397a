// Oracle harness: drives the UNMODIFIED reference EDLib headers (compiled from the read-only
// reference tree against the stand-in headers in this directory) and prints eigenpairs,
// G(i w_n), chi(i w_n) and raw Hamiltonian-times-vector products as text.  It is test
// infrastructure: the fixtures under tests/golden/ are generated with it, and the
// restatement in oracle/edoracle.cpp is checked against it.
//
// usage: edlib_ref <input.txt> <mode>
//   input.txt : "param KEY VALUE" lines (EDLib parameter names, plus harness.MODEL =
//               HUBBARD|SIAM, harness.STORAGE = CRS|SRS|SOCRS, harness.NUP/NDN for mode av)
//               and "data <path> ..." datasets (read through the archive stand-in).
//   mode      : eigen | gf | chi | real | av | sigma
// Flow of mode chi follows test/Lanczos_Test.cpp:29-119 of the reference; mode sigma follows
// GreensFunction::compute_selfenergy (GreensFunction.h:202-222) without its file output: the model's
// bare_greens_function on the mesh of G_ij, then (Hubbard only) solve_dyson.  The Anderson model's
// solve_dyson builds NSITES x NSITES matrices of which it fills only the impurity block, so it is not run.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>

#include "edlib/EDParams.h"
#include "edlib/Hamiltonian.h"
#include "edlib/GreensFunction.h"
#include "edlib/ChiLoc.h"
#include "edlib/StaticObservables.h"
#include "edlib/MeshFactory.h"

static void load_params(const std::string &file, alps::params &p) {
  std::ifstream in(file.c_str());
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string tok;
    if (!(ls >> tok) || tok != "param") continue;
    std::string k, v;
    ls >> k >> v;
    p[k] = v;
  }
  p["INPUT_FILE"] = file;
}

template <class Ham>
static void print_eigen(Ham &ham, std::ostream &out) {
  out << std::setprecision(17);
  for (const auto &pr : ham.eigenpairs())
    out << "E " << pr.eigenvalue() << " " << pr.sector().nup() << " " << pr.sector().ndown() << "\n";
}

template <class GF>
static void print_gf3(const std::string &tag, const GF &g, std::ostream &out) {
  for (int w = 0; w < g.mesh1().extent(); ++w)
    for (int i = 0; i < g.mesh2().extent(); ++i)
      for (int s = 0; s < g.mesh3().extent(); ++s) {
        auto v = g(typename std::decay<decltype(g.mesh1())>::type::index_type(w), alps::gf::index_mesh::index_type(i),
                   alps::gf::index_mesh::index_type(s));
        out << tag << " " << w << " " << i << " " << s << " " << v.real() << " " << v.imag() << "\n";
      }
}

template <class GF>
static void print_gf2(const std::string &tag, const GF &g, std::ostream &out) {
  for (int w = 0; w < g.mesh1().extent(); ++w)
    for (int i = 0; i < g.mesh2().extent(); ++i) {
      auto v = g(typename std::decay<decltype(g.mesh1())>::type::index_type(w), alps::gf::index_mesh::index_type(i));
      out << tag << " " << w << " " << i << " " << v.real() << " " << v.imag() << "\n";
    }
}

template <class Ham>
static int run(alps::params &p, const std::string &mode) {
  std::ostream &out = std::cout;
  std::streambuf *orig = std::cout.rdbuf();
  // the reference prints progress on std::cout; keep results on stdout and progress on stderr
  std::ostringstream results;
  std::cout.rdbuf(std::cerr.rdbuf());
  Ham ham(p);
  if (mode == "av") {
    typedef typename Ham::ModelType::Sector Sector;
    int nup = p["harness.NUP"], ndn = p["harness.NDN"];
    int ns = p["NSITES"];
    EDLib::Combination comb(ns);
    Sector s(nup, ndn, size_t(comb.c_n_k(ns, nup)) * comb.c_n_k(ns, ndn));
    ham.model().symmetry().set_sector(s);
    ham.storage().fill();
    size_t n = s.size();
    std::vector<double> v(n), w(n, 0.0);
    for (size_t i = 0; i < n; ++i) v[i] = std::sin(0.37 * double(i) + 0.1);
    ham.storage().av(v.data(), w.data(), int(n), true);
    results << std::setprecision(17);
    for (size_t i = 0; i < n; ++i) results << "W " << i << " " << w[i] << "\n";
  } else {
    ham.diag();
    results << std::setprecision(17);
    print_eigen(ham, results);
    if (mode == "gf" || mode == "chi") {
      EDLib::gf::GreensFunction<Ham, EDLib::MatsubaraMeshFactory, alps::gf::statistics::statistics_type> gf(
          p, ham, alps::gf::statistics::statistics_type::FERMIONIC);
      gf.compute();
      print_gf3("G", gf.G(), results);
      print_gf3("GIJ", gf.G_ij(), results);
    }
    if (mode == "chi") {
      EDLib::StaticObservables<Ham> so(p);
      auto obs = so.calculate_static_observables(ham);
      for (auto &kv : obs) {
        results << "OBS " << kv.first.size() << " ";
        for (char c : kv.first) results << (c == ' ' ? '_' : c);
        for (double x : kv.second) results << " " << x;
        results << "\n";
      }
      EDLib::gf::ChiLoc<Ham, EDLib::MatsubaraMeshFactory, alps::gf::statistics::statistics_type> susc(
          p, ham, alps::gf::statistics::statistics_type::BOSONIC);
      double avg = 0.0;
      for (auto x : obs[so._M_]) avg += x / (2.0 * obs[so._M_].size());
      susc.template compute<EDLib::gf::SzOperator<double>>(&avg);
      print_gf2("CHISZ", susc.G(), results);
      print_gf2("CHISZIJ", susc.G_ij(), results);
      avg = 0.0;
      for (auto x : obs[so._N_]) avg += x / double(obs[so._N_].size());
      susc.template compute<EDLib::gf::NOperator<double>>(&avg);
      print_gf2("CHIN", susc.G(), results);
      print_gf2("CHINIJ", susc.G_ij(), results);
    }
    if (mode == "sigma") {
      EDLib::gf::GreensFunction<Ham, EDLib::MatsubaraMeshFactory, alps::gf::statistics::statistics_type> gf(
          p, ham, alps::gf::statistics::statistics_type::FERMIONIC);
      gf.compute();
      print_gf3("GIJ", gf.G_ij(), results);
      typedef typename std::decay<decltype(gf.G_ij())>::type GF;
      GF bare(gf.G_ij().mesh1(), gf.G_ij().mesh2(), gf.G_ij().mesh3());
      GF sigma(gf.G_ij().mesh1(), gf.G_ij().mesh2(), gf.G_ij().mesh3());
      ham.model().bare_greens_function(bare, p["lanc.BETA"].template as<double>());
      print_gf3("G0", bare, results);
      std::string model = p.exists("harness.MODEL") ? p["harness.MODEL"].template as<std::string>() : "HUBBARD";
      if (model == "HUBBARD") {
        ham.model().solve_dyson(bare, gf.G_ij(), sigma);
        print_gf3("SIGMA", sigma, results);
      }
    }
    if (mode == "real") {  // the same on the real-frequency mesh (RealFreqMeshFactory)
      EDLib::gf::GreensFunction<Ham, EDLib::RealFreqMeshFactory> gf(p, ham);
      gf.compute();
      print_gf3("G", gf.G(), results);
      print_gf3("GIJ", gf.G_ij(), results);
      EDLib::StaticObservables<Ham> so(p);
      auto obs = so.calculate_static_observables(ham);
      EDLib::gf::ChiLoc<Ham, EDLib::RealFreqMeshFactory> susc(p, ham);
      double avg = 0.0;
      for (auto x : obs[so._M_]) avg += x / (2.0 * obs[so._M_].size());
      susc.template compute<EDLib::gf::SzOperator<double>>(&avg);
      print_gf2("CHISZ", susc.G(), results);
      avg = 0.0;
      for (auto x : obs[so._N_]) avg += x / double(obs[so._N_].size());
      susc.template compute<EDLib::gf::NOperator<double>>(&avg);
      print_gf2("CHIN", susc.G(), results);
    }
  }
  std::cout.rdbuf(orig);
  out << results.str();
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    std::cerr << "usage: edlib_ref <input.txt> <eigen|gf|chi|real|av|sigma>\n";
    return 2;
  }
  alps::params p;
  EDLib::define_parameters(p);
  load_params(argv[1], p);
  std::string model = p.exists("harness.MODEL") ? p["harness.MODEL"].as<std::string>() : "HUBBARD";
  std::string storage = p.exists("harness.STORAGE") ? p["harness.STORAGE"].as<std::string>() : "CRS";
  std::string mode = argv[2];
  try {
    if (model == "HUBBARD") {
      typedef EDLib::Model::HubbardModel<double> M;
      if (storage == "CRS") return run<EDLib::Hamiltonian<EDLib::Storage::CRSStorage<M>>>(p, mode);
      if (storage == "SRS") return run<EDLib::Hamiltonian<EDLib::Storage::SpinResolvedStorage<M>>>(p, mode);
      if (storage == "SOCRS") return run<EDLib::Hamiltonian<EDLib::Storage::SOCRSStorage<M>>>(p, mode);
    } else if (model == "SIAM") {
      typedef EDLib::Model::SingleImpurityAndersonModel<double> M;
      if (storage == "CRS") return run<EDLib::Hamiltonian<EDLib::Storage::CRSStorage<M>>>(p, mode);
      if (storage == "SRS") return run<EDLib::Hamiltonian<EDLib::Storage::SpinResolvedStorage<M>>>(p, mode);
      if (storage == "SOCRS") return run<EDLib::Hamiltonian<EDLib::Storage::SOCRSStorage<M>>>(p, mode);
    }
  } catch (std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  std::cerr << "unknown model/storage\n";
  return 2;
}
