// Host-side objects behind the C ABI handles (private to the library).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/edgpu.h"
#include "edgpu_kernels.h"

struct edgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  edgpu::DeviceAllocator alloc;
  std::string err;
};

namespace edgpu {
namespace host {

struct ApiError : std::runtime_error {
  int code;
  ApiError(int c, const std::string &s) : std::runtime_error(s), code(c) {}
};

inline void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw ApiError(EDGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(x) ::edgpu::host::ck((x), #x)

template <typename F>
int guard(edgpu_ctx *ctx, F &&f) {
  try {
    return f();
  } catch (ApiError &e) {
    if (ctx) ctx->err = e.what();
    return e.code;
  } catch (std::bad_alloc &) {
    if (ctx) ctx->err = "host allocation failed";
    return EDGPU_ERR_CAPACITY;
  } catch (std::exception &e) {
    if (ctx) ctx->err = e.what();
    return EDGPU_ERR_ARG;
  }
}

// device buffer owned through the context's caching allocator
struct DBuf {
  DeviceAllocator *a = nullptr;
  void *p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(DeviceAllocator &al, size_t b) : a(&al), bytes(b) { p = al.alloc(b ? b : 16); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : a(o.a), p(o.p), bytes(o.bytes) { o.p = nullptr; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      reset();
      a = o.a;
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
    }
    return *this;
  }
  ~DBuf() { reset(); }
  void reset() {
    if (p && a) a->free(p);
    p = nullptr;
  }
  void adopt(DeviceAllocator &al, void *q) {
    reset();
    a = &al;
    p = q;
  }
  template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

struct SpinCsr {
  int rows = 0;
  long long nnz = 0;
  DBuf rp, col, v64, v32;
  int kmax = 0, ld = 0;           // longest row; rows rounded up to 4
  DBuf len, ell_col, ell_v64, ell_v32;  // k-major copy (SectorOp::dn_ell_*)
  DBuf vff, ell_vff;                     // float-float values (built on first use, ensure_ff)
  std::vector<int> hrp;            // host copy of the row pointers
};

struct Sector {
  int storage = 0, nup = 0, ndn = 0;
  long long dim = 0;
  int up_rows = 0, dn_rows = 0;
  DBuf diag64, diag32, crs_rp, crs_col, crs_v64, crs_v32;
  long long crs_nnz = 0;
  SectorOp<double> op64{};
  SectorOp<float> op32{};
  DBuf dop64, dop32;
  DBuf diagff;             // float-float tables of an SRS sector, built on first use (ensure_ff)
  SectorOp<ffloat> opff{};
  DBuf dopff;
  int srs_rows = 1, nitems = 1;
  int up_hops_item = 0;  // SRS: most up-spin hop entries of one work item (rows staged per item)
  template <typename T> const SectorOp<T> &op() const;
  template <typename T> const SectorOp<T> *dop() const;
};
template <> inline const SectorOp<double> &Sector::op<double>() const { return op64; }
template <> inline const SectorOp<float> &Sector::op<float>() const { return op32; }
template <> inline const SectorOp<double> *Sector::dop<double>() const { return dop64.as<SectorOp<double>>(); }
template <> inline const SectorOp<float> *Sector::dop<float>() const { return dop32.as<SectorOp<float>>(); }
template <> inline const SectorOp<ffloat> &Sector::op<ffloat>() const { return opff; }
template <> inline const SectorOp<ffloat> *Sector::dop<ffloat>() const { return dopff.as<SectorOp<ffloat>>(); }

// One eigen-pair; its vector is column `offset / n` of a shared block of Ritz vectors.
struct Pair {
  double E;
  int nup, ndn, id;
  int prec;
  long long n;
  std::shared_ptr<DBuf> block;
  long long offset;
  bool no_refine = false;  // its sector's FP64 continuation did not converge: not tried again
  template <typename T> T *vec() const { return block ? block->as<T>() + offset : nullptr; }
};

}  // namespace host
}  // namespace edgpu

struct edgpu_model {
  edgpu_ctx *ctx = nullptr;
  int kind = 0, ns = 0, ml = 0, ip = 0;
  std::vector<edgpu::Transition> T, V;
  std::vector<double> t, U, xmu, hmag, J, epsk, vk, h0, Ut;
  double mu = 0;
  size_t max_dim = 0, max_size = 0;
  edgpu::host::DBuf dTvff, dVvff;  // float-float transition values (ensure_ff)
  edgpu::host::DBuf dT, dV, dTv64, dTv32, dVv64, dVv32, dU, dxmu, dhmag, dJ, depsk, dh0, dUt, dbinom, dbasis, dninv;
  std::vector<long long> basis_off;
  edgpu::DevModel dm{};
  std::map<std::pair<int, int>, std::unique_ptr<edgpu::host::SpinCsr>> spin;
  std::map<std::tuple<int, int, int>, std::unique_ptr<edgpu::host::Sector>> sectors;
  edgpu::host::Sector *cur = nullptr;
  std::vector<edgpu::host::Pair> pairs;
  bool have_pairs = false, evals_only = false;
  int diag_storage = 1;
  int diag_ncv = 0, diag_maxitr = 1000;  // arpack.NCV (0: 2 nev + 3) and restart cycles of the last diag
  edgpu::OpTuning op_tune[2];  // operator variant per precision (0 FP64, 1 FP32), chosen on the first eigen batch
  long long st_spmv = 0, st_steps = 0, st_restarts = 0;
  double st_work = 0;
  int interacting() const { return kind == 0 ? ns : ml; }
};

namespace edgpu {
namespace host {

template <typename T>
DBuf upload(edgpu_ctx *c, const std::vector<T> &v) {
  DBuf b(c->alloc, sizeof(T) * std::max<size_t>(v.size(), 1));
  if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream));
  return b;
}

inline void sync(edgpu_ctx *c) {
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaGetLastError());
}

// The eigen-pairs a Boltzmann average keeps (GreensFunction.h:125-140): Z over every pair, a pair kept unless
// its weight exp(-beta (E - E0)) is below the cut-off (with the reference's epsilon guard).
struct Kept {
  const Pair *pair;
  double bf;
};

inline void boltzmann(const edgpu_model *m, double beta, double cutoff, double &E0, double &Z, std::vector<Kept> &keep) {
  E0 = m->pairs.front().E;
  Z = 0.0;
  for (auto &p : m->pairs) Z += std::exp(-(p.E - E0) * beta);
  for (auto &p : m->pairs) {
    double bf = std::exp(-(p.E - E0) * beta);
    if (std::fabs(cutoff - bf) > std::numeric_limits<double>::epsilon() && bf < cutoff) continue;
    keep.push_back({&p, bf});
  }
}

// FP64 continuation of the FP32 eigen-solve for the sectors holding kept pairs (driver.cu); returns the
// worst status (EDGPU_NOT_CONVERGED when a sector's continuation did not converge: its pairs stay FP32)
int refine_kept(edgpu_model *const *ms, int count, double beta, double cutoff);

void finish_model(edgpu_model *m);
Sector *get_sector(edgpu_model *m, int storage, int nup, int ndn);
// Builds (once) the float-float tables and SectorOp of a spin-resolved sector from its FP64 ones.
void ensure_ff(edgpu_model *m, Sector *s);
template <typename T> MvShape mv_shape(const Sector &s);
void merge_shape(MvShape &a, const MvShape &b);
template <typename T> void apply_h(edgpu_model *m, Sector *s, const T *x, T *y, const T *z, double cz);
int diag_dispatch(edgpu_model *m, const edgpu_diag_params *p, int *npairs);
int diag_many_dispatch(edgpu_model *const *ms, int count, const edgpu_diag_params *p, int *npairs);
int diag_sector_dispatch(edgpu_model *m, const edgpu_diag_params *p, int nup, int ndn, double *evals, int *nconv,
                         double *evecs, long long ldv);
int sector_order(const edgpu_model *m, const int *list, int n_in, int *out);

// Green's functions (gf.cu)
int gf_dispatch(edgpu_model *m, const edgpu_gf_params *p, double *G, double *Gij, double *Z);
int chi_dispatch(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chiij, double *Z);
int gf_many_dispatch(edgpu_model *const *ms, int count, const edgpu_gf_params *p, int chi, int op, const double *avg,
                     double *const *G, double *const *Gij, double *Z);
int gf_weighted_dispatch(edgpu_model *m, const edgpu_gf_params *p, const double *weights, int nrows, double *G,
                         double *Z);
// self-energy from the Dyson equation (dyson.cu)
int self_energy_dispatch(edgpu_model *m, const edgpu_gf_params *p, const double *Gij, double *G0, double *Sigma);
// continuous-batching request loop (driver.cu)
edgpu_server *server_create(edgpu_ctx *c, int prec, size_t budget);
long long server_submit(edgpu_server *s, edgpu_model *m, const edgpu_diag_params *dp, const edgpu_gf_params *gp,
                        double *G, double *Gij, double *Z);
void server_step(edgpu_server *s, int *running, int *queued);
int server_poll(edgpu_server *s, long long ticket, int *npairs);
void server_destroy(edgpu_server *s);
edgpu_ctx *server_ctx(edgpu_server *s);
int static_obs(edgpu_model *m, double beta, double cutoff, double *n, double *n_up, double *n_dn, double *mag,
               double *d_occ, double *mimj, double *n_eff, double *energy);
template <typename T>
void lanczos_batch(edgpu_model *m, const std::vector<Sector *> &secs, const std::vector<T *> &starts, int nlanc,
                   std::vector<DBuf> &alpha, std::vector<DBuf> &beta, std::vector<DBuf> &state);

}  // namespace host
}  // namespace edgpu
