// Host side of the library behind the C ABI in include/edgpu.h: model upload, sector construction and
// the batched restarted-Lanczos eigen-solver that replaces the ARPACK loop.  All vector work runs in the
// kernels of tables.cu, spmv.cu and krylov.cu on the context's stream; the host orders launches, reads
// the few scalars that steer restarts (once per restart cycle) and copies results out.
#include <climits>
#include <cstdio>

#include "model_internal.h"

#include <atomic>
#include <deque>
#include <cstdlib>

namespace edgpu {
using host::ApiError;

static std::atomic<long long> g_launches{0};
long long launch_count() { return g_launches.load(); }

int occupancy_grid(const void *fn, int block, size_t smem, int nitems) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void *, int, size_t>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  int g = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, fn, block, smem);
    auto it = cache.find(key);
    if (it != cache.end()) {
      g = it->second;
    } else {
      int nsm = 0, per = 0;
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, smem);
      g = std::max(1, nsm) * std::max(1, per);
      cache[key] = g;
    }
  }
  return nitems < g ? std::max(1, nitems) : g;
}
void note_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ============================================================================ allocator
void *DeviceAllocator::alloc(size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  auto it = free_.find(bytes);
  if (it != free_.end()) {
    void *p = it->second;
    free_.erase(it);
    live_[p] = bytes;
    in_use_ += bytes;
    return p;
  }
  if (budget && held_ + bytes > budget) {
    // give back cached blocks first
    for (auto &kv : free_) {
      cudaFree(kv.second);
      held_ -= kv.first;
    }
    free_.clear();
    if (held_ + bytes > budget)
      throw ApiError(EDGPU_ERR_CAPACITY, "device memory budget exceeded: need " + std::to_string(bytes) + " bytes, budget " +
                                             std::to_string(budget) + ", held " + std::to_string(held_));
  }
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (auto &kv : free_) {
      cudaFree(kv.second);
      held_ -= kv.first;
    }
    free_.clear();
    e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw ApiError(EDGPU_ERR_CAPACITY, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
  }
  held_ += bytes;
  in_use_ += bytes;
  live_[p] = bytes;
  return p;
}

void DeviceAllocator::free(void *p) {
  auto it = live_.find(p);
  if (it == live_.end()) return;
  in_use_ -= it->second;
  free_.insert({it->second, p});
  live_.erase(it);
}

void DeviceAllocator::release_all() {
  for (auto &kv : free_) cudaFree(kv.second);
  for (auto &kv : live_) cudaFree(kv.first);
  free_.clear();
  live_.clear();
  held_ = in_use_ = 0;
}

}  // namespace edgpu

namespace edgpu {
namespace host {

int err_flag(edgpu_ctx *c, const DBuf &e) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, e.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  return h;
}

// ============================================================================ model upload
void finish_model(edgpu_model *m) {
  edgpu_ctx *c = m->ctx;
  if (m->ns < 1 || m->ns > kMaxNs) throw ApiError(EDGPU_ERR_ARG, "NSITES must be in [1, 20]");
  m->ip = 2 * m->ns;
  std::vector<double> tv64, vv64;
  std::vector<float> tv32, vv32;
  for (auto &t : m->T) { tv64.push_back(t.value); tv32.push_back((float)t.value); }
  for (auto &t : m->V) { vv64.push_back(t.value); vv32.push_back((float)t.value); }
  m->dT = upload(c, m->T);
  m->dV = upload(c, m->V);
  m->dTv64 = upload(c, tv64);
  m->dTv32 = upload(c, tv32);
  m->dVv64 = upload(c, vv64);
  m->dVv32 = upload(c, vv32);
  std::vector<long long> binom((kMaxNs + 2) * (kMaxNs + 2), 0);
  for (int n = 0; n <= kMaxNs + 1; ++n)
    for (int k = 0; k <= n; ++k) binom[n * (kMaxNs + 2) + k] = binom_at_host(n, k);
  m->dbinom = upload(c, binom);
  m->basis_off.assign(m->ns + 2, 0);
  for (int k = 0; k <= m->ns; ++k) m->basis_off[k + 1] = m->basis_off[k] + binom_at_host(m->ns, k);
  m->dbasis = DBuf(c->alloc, sizeof(int) * (size_t)m->basis_off[m->ns + 1]);
  m->dninv = DBuf(c->alloc, sizeof(int) * (size_t)(m->ns + 1) * ((size_t)1 << m->ns));
  DevModel &d = m->dm;
  d.kind = m->kind;
  d.ns = m->ns;
  d.ip = m->ip;
  d.ml = m->ml;
  d.nT = (int)m->T.size();
  d.nV = (int)m->V.size();
  d.T = m->dT.as<Transition>();
  d.V = m->dV.as<Transition>();
  d.binom = m->dbinom.as<long long>();
  d.basis = m->dbasis.as<int>();
  d.ninv = m->dninv.as<int>();
  if (m->kind == 0) {
    std::vector<double> xmu2 = m->xmu;
    while (xmu2.size() < 2) xmu2.push_back(0.0);
    m->dU = upload(c, m->U);
    m->dxmu = upload(c, xmu2);
    m->dhmag = upload(c, m->hmag);
    d.U = m->dU.as<double>();
    d.xmu = m->dxmu.as<double>();
    d.hmag = m->dhmag.as<double>();
    d.J = nullptr;
    if (!m->J.empty()) {
      m->dJ = upload(c, m->J);
      d.J = m->dJ.as<double>();
    }
  } else {
    m->depsk = upload(c, m->epsk);
    m->dh0 = upload(c, m->h0);
    m->dUt = upload(c, m->Ut);
    d.epsk = m->depsk.as<double>();
    d.h0 = m->dh0.as<double>();
    d.Ut = m->dUt.as<double>();
    d.mu = m->mu;
  }
  build_tables(d, m->basis_off.data(), m->dbasis.as<int>(), m->dninv.as<int>(), c->stream);
  sync(c);
}

// ============================================================================ sectors
SpinCsr *get_spin(edgpu_model *m, int spin, int k) {
  auto key = std::make_pair(spin, k);
  auto it = m->spin.find(key);
  if (it != m->spin.end()) return it->second.get();
  edgpu_ctx *c = m->ctx;
  std::unique_ptr<SpinCsr> s(new SpinCsr());
  long long rows = binom_at_host(m->ns, k);
  s->rows = (int)rows;
  DBuf count(c->alloc, sizeof(long long) * rows), rp(c->alloc, sizeof(long long) * (rows + 1)),
      tmp(c->alloc, sizeof(long long) * scan_tmp_size(rows)), err(c->alloc, sizeof(int));
  s->rp = DBuf(c->alloc, sizeof(int) * (rows + 1));
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), c->stream));
  int *col = nullptr;
  double *v64 = nullptr;
  float *v32 = nullptr;
  launch_spin_csr(m->dm, spin, k, rows, m->dbasis.as<int>() + m->basis_off[k], count.as<long long>(),
                  rp.as<long long>(), tmp.as<long long>(), s->rp.as<int>(), &col, &v64, &v32, &s->nnz, err.as<int>(),
                  c->alloc, c->stream);
  s->col.adopt(c->alloc, col);
  s->v64.adopt(c->alloc, v64);
  s->v32.adopt(c->alloc, v32);
  if (err_flag(c, err)) throw ApiError(EDGPU_ERR_CAPACITY, "per-spin hopping row longer than the row buffer");
  {
    // k-major copy for the operator kernels' column tiles
    std::vector<int> &hrp = s->hrp;
    hrp.assign(rows + 1, 0);
    CK(cudaMemcpyAsync(hrp.data(), s->rp.p, sizeof(int) * (rows + 1), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (long long d = 0; d < rows; ++d) s->kmax = std::max(s->kmax, hrp[d + 1] - hrp[d]);
    s->ld = (int)((rows + 3) & ~3LL);
    const size_t cells = (size_t)std::max(1, s->kmax) * s->ld;
    s->len = DBuf(c->alloc, sizeof(int) * s->ld);
    s->ell_col = DBuf(c->alloc, sizeof(int) * cells);
    s->ell_v64 = DBuf(c->alloc, sizeof(double) * cells);
    s->ell_v32 = DBuf(c->alloc, sizeof(float) * cells);
    CK(cudaMemsetAsync(s->len.p, 0, s->len.bytes, c->stream));
    CK(cudaMemsetAsync(s->ell_col.p, 0, s->ell_col.bytes, c->stream));
    CK(cudaMemsetAsync(s->ell_v64.p, 0, s->ell_v64.bytes, c->stream));
    CK(cudaMemsetAsync(s->ell_v32.p, 0, s->ell_v32.bytes, c->stream));
    launch_spin_ell(s->rp.as<int>(), s->col.as<int>(), s->v64.as<double>(), s->v32.as<float>(), (int)rows, s->ld,
                    s->len.as<int>(), s->ell_col.as<int>(), s->ell_v64.as<double>(), s->ell_v32.as<float>(), c->stream);
  }
  SpinCsr *raw = s.get();
  m->spin[key] = std::move(s);
  return raw;
}

template <typename T>
void fill_common(edgpu_model *m, const Sector &s, SectorOp<T> &op, const T *diag, const T *tval, const T *vval) {
  op.storage = s.storage;
  op.ns = m->ns;
  op.ip = m->ip;
  op.nup = s.nup;
  op.ndn = s.ndn;
  op.dim = s.dim;
  op.up_rows = s.up_rows;
  op.dn_rows = s.dn_rows;
  op.diag = diag;
  op.up_basis = m->dbasis.as<int>() + m->basis_off[s.nup];
  op.dn_basis = m->dbasis.as<int>() + m->basis_off[s.ndn];
  op.ninv_up = m->dninv.as<int>() + ((size_t)s.nup << m->ns);
  op.ninv_dn = m->dninv.as<int>() + ((size_t)s.ndn << m->ns);
  op.nT = (int)m->T.size();
  op.nV = (int)m->V.size();
  op.T_ = m->dT.as<Transition>();
  op.V_ = m->dV.as<Transition>();
  op.T_val = tval;
  op.V_val = vval;
}

void ensure_ff(edgpu_model *m, Sector *s) {
  if (s->dopff.p) return;
  if (s->storage != kSRS) throw ApiError(EDGPU_ERR_ARG, "float-float recurrences need spin-resolved storage");
  edgpu_ctx *c = m->ctx;
  auto conv = [&](DBuf &dst, const DBuf &src, long long n) {  // n FP64 values -> float-float
    dst = DBuf(c->alloc, sizeof(ffloat) * (size_t)std::max<long long>(n, 1));
    launch_convert<ffloat>(src.as<double>(), dst.as<ffloat>(), n, c->stream);
  };
  if (!m->dTvff.p) {
    conv(m->dTvff, m->dTv64, (long long)m->T.size());
    conv(m->dVvff, m->dVv64, (long long)m->V.size());
  }
  SpinCsr *up = get_spin(m, 0, s->nup), *dn = get_spin(m, 1, s->ndn);
  for (SpinCsr *sp : {up, dn}) {
    if (!sp->vff.p) conv(sp->vff, sp->v64, sp->nnz);  // the CSR values are adopted buffers: counts, not bytes
    if (!sp->ell_vff.p) conv(sp->ell_vff, sp->ell_v64, (long long)std::max(1, sp->kmax) * sp->ld);
  }
  conv(s->diagff, s->diag64, s->dim);
  const SectorOp<double> &d = s->op64;
  SectorOp<ffloat> &o = s->opff;
  o.storage = d.storage;
  o.ns = d.ns;
  o.ip = d.ip;
  o.nup = d.nup;
  o.ndn = d.ndn;
  o.dim = d.dim;
  o.up_rows = d.up_rows;
  o.dn_rows = d.dn_rows;
  o.diag = s->diagff.as<ffloat>();
  o.up_rp = d.up_rp;
  o.up_col = d.up_col;
  o.up_val = up->vff.as<ffloat>();
  o.dn_rp = d.dn_rp;
  o.dn_col = d.dn_col;
  o.dn_val = dn->vff.as<ffloat>();
  o.dn_nnz = d.dn_nnz;
  o.dn_len = d.dn_len;
  o.dn_ell_col = d.dn_ell_col;
  o.dn_ell_val = dn->ell_vff.as<ffloat>();
  o.dn_ld = d.dn_ld;
  o.crs_rp = nullptr;
  o.crs_col = nullptr;
  o.crs_val = nullptr;
  o.up_basis = d.up_basis;
  o.dn_basis = d.dn_basis;
  o.ninv_up = d.ninv_up;
  o.ninv_dn = d.ninv_dn;
  o.nT = d.nT;
  o.nV = d.nV;
  o.T_ = d.T_;
  o.V_ = d.V_;
  o.T_val = m->dTvff.as<ffloat>();
  o.V_val = m->dVvff.as<ffloat>();
  s->dopff = DBuf(c->alloc, sizeof(SectorOp<ffloat>));
  CK(cudaMemcpyAsync(s->dopff.p, &s->opff, sizeof(SectorOp<ffloat>), cudaMemcpyHostToDevice, c->stream));
  sync(c);
}

Sector *get_sector(edgpu_model *m, int storage, int nup, int ndn) {
  if (storage < 0 || storage > 2) throw ApiError(EDGPU_ERR_ARG, "unknown storage");
  if (nup < 0 || ndn < 0 || nup > m->ns || ndn > m->ns) throw ApiError(EDGPU_ERR_ARG, "sector out of range");
  auto key = std::make_tuple(storage, nup, ndn);
  auto it = m->sectors.find(key);
  if (it != m->sectors.end()) return it->second.get();
  edgpu_ctx *c = m->ctx;
  std::unique_ptr<Sector> s(new Sector());
  s->storage = storage;
  s->nup = nup;
  s->ndn = ndn;
  s->up_rows = (int)binom_at_host(m->ns, nup);
  s->dn_rows = (int)binom_at_host(m->ns, ndn);
  s->dim = (long long)s->up_rows * s->dn_rows;
  const size_t nTV = m->T.size() + m->V.size();
  if (storage != kSRS && m->max_dim && (size_t)s->dim > m->max_dim)
    throw ApiError(EDGPU_ERR_CAPACITY, "Current sector request more memory than allocated. Increase MAX_DIM parameter. Requested " +
                                           std::to_string(s->dim) + ", allocated " + std::to_string(m->max_dim) + ".");
  if (storage == kSOCRS && m->max_size && (size_t)s->dim * nTV > m->max_size)
    throw ApiError(EDGPU_ERR_CAPACITY, "New sector request more memory than allocated. Increase MAX_SIZE parameter. Requested " +
                                           std::to_string((size_t)s->dim * nTV) + ", allocated " + std::to_string(m->max_size) + ".");
  s->diag64 = DBuf(c->alloc, sizeof(double) * s->dim);
  s->diag32 = DBuf(c->alloc, sizeof(float) * s->dim);
  fill_common<double>(m, *s, s->op64, s->diag64.as<double>(), m->dTv64.as<double>(), m->dVv64.as<double>());
  fill_common<float>(m, *s, s->op32, s->diag32.as<float>(), m->dTv32.as<float>(), m->dVv32.as<float>());
  launch_diag(m->dm, s->op64, s->diag64.as<double>(), s->diag32.as<float>(), c->stream);
  if (storage == kSRS) {
    SpinCsr *up = get_spin(m, 0, nup), *dn = get_spin(m, 1, ndn);
    s->op64.up_rp = s->op32.up_rp = up->rp.as<int>();
    s->op64.up_col = s->op32.up_col = up->col.as<int>();
    s->op64.up_val = up->v64.as<double>();
    s->op32.up_val = up->v32.as<float>();
    s->op64.dn_rp = s->op32.dn_rp = dn->rp.as<int>();
    s->op64.dn_col = s->op32.dn_col = dn->col.as<int>();
    s->op64.dn_val = dn->v64.as<double>();
    s->op32.dn_val = dn->v32.as<float>();
    s->op64.dn_nnz = s->op32.dn_nnz = (int)dn->nnz;
    s->op64.dn_len = s->op32.dn_len = dn->len.as<int>();
    s->op64.dn_ell_col = s->op32.dn_ell_col = dn->ell_col.as<int>();
    s->op64.dn_ell_val = dn->ell_v64.as<double>();
    s->op32.dn_ell_val = dn->ell_v32.as<float>();
    s->op64.dn_ld = s->op32.dn_ld = dn->ld;
    if (s->dim > (long long)INT_MAX)
      throw ApiError(EDGPU_ERR_CAPACITY, "spin-resolved sector above 2^31 - 1 states");
    s->srs_rows = srs_item_rows(s->up_rows, s->dn_rows);
    s->nitems = (s->up_rows + s->srs_rows - 1) / s->srs_rows;
    for (int it = 0; it < s->nitems; ++it) {
      const int u0 = it * s->srs_rows, u1 = std::min(s->up_rows, u0 + s->srs_rows);
      s->up_hops_item = std::max(s->up_hops_item, up->hrp[u1] - up->hrp[u0]);
    }
  } else {
    s->nitems = (int)((s->dim + kItemElems - 1) / kItemElems);
  }
  if (storage == kCRS) {
    DBuf count(c->alloc, sizeof(long long) * s->dim), tmp(c->alloc, sizeof(long long) * scan_tmp_size(s->dim)),
        err(c->alloc, sizeof(int));
    s->crs_rp = DBuf(c->alloc, sizeof(long long) * (s->dim + 1));
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), c->stream));
    int *col = nullptr;
    double *v64 = nullptr;
    float *v32 = nullptr;
    launch_crs(m->dm, s->op64, count.as<long long>(), s->crs_rp.as<long long>(), tmp.as<long long>(), &col, &v64, &v32,
               &s->crs_nnz, err.as<int>(), c->alloc, c->stream);
    s->crs_col.adopt(c->alloc, col);
    s->crs_v64.adopt(c->alloc, v64);
    s->crs_v32.adopt(c->alloc, v32);
    if (err_flag(c, err)) throw ApiError(EDGPU_ERR_CAPACITY, "sector row longer than the row buffer");
    if (m->max_size && (size_t)s->crs_nnz > m->max_size)
      throw ApiError(EDGPU_ERR_CAPACITY, "Current sector request more memory than allocated. Increase MAX_SIZE parameter. Requested " +
                                             std::to_string(s->crs_nnz) + ", allocated " + std::to_string(m->max_size) + ".");
    s->op64.crs_rp = s->op32.crs_rp = s->crs_rp.as<long long>();
    s->op64.crs_col = s->op32.crs_col = s->crs_col.as<int>();
    s->op64.crs_val = s->crs_v64.as<double>();
    s->op32.crs_val = s->crs_v32.as<float>();
  }
  if (storage == kSOCRS) {
    DBuf err(c->alloc, sizeof(int));
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), c->stream));
    launch_socrs_check(m->dm, s->op64, err.as<int>(), c->stream);
    int e = err_flag(c, err);
    if (e == 2) throw ApiError(EDGPU_ERR_COLLISION, "Attempt to use addElement() to add diagonal element. Use addDiagonal() instead!");
    if (e == 3) throw ApiError(EDGPU_ERR_COLLISION, "Collision. Check a, adag, numState, ninv_value!");
  }
  s->dop64 = DBuf(c->alloc, sizeof(SectorOp<double>));
  s->dop32 = DBuf(c->alloc, sizeof(SectorOp<float>));
  CK(cudaMemcpyAsync(s->dop64.p, &s->op64, sizeof(SectorOp<double>), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(s->dop32.p, &s->op32, sizeof(SectorOp<float>), cudaMemcpyHostToDevice, c->stream));
  // no synchronisation: every later use of the tables is ordered on the context's stream, and the copies of
  // the host-side SectorOps are staged before cudaMemcpyAsync returns (pageable source)
  CK(cudaGetLastError());
  Sector *raw = s.get();
  m->sectors[key] = std::move(s);
  return raw;
}

// shared memory an operator launch over this sector needs (see spmv.cu)
template <typename T>
MvShape mv_shape(const Sector &s) {
  MvShape sh{s.storage, 0};
  if (s.storage == kSRS) {
    long long e = (long long)s.srs_rows * s.dn_rows;
    long long cap = (long long)(120 * 1024) / (long long)sizeof(T);
    sh.xs_elems = (int)std::min(e, cap);
    sh.xs_staged = sh.xs_elems;
    // long rows: the item's up-spin source rows can be staged beside its own rows when both fit in 112 KB
    // (two blocks per SM); whether they are is the operator tuner's choice, or EDGPU_SRS_STAGE_KB's (the
    // environment variable, else the build's default) when the tuner is off or the variable is set
    const long long es = e + (long long)s.up_hops_item * s.dn_rows;
    if (s.dn_rows >= kSrsLongRow && es * (long long)sizeof(T) <= 112 * 1024LL) sh.xs_staged = (int)es;
    const char *v = getenv("EDGPU_SRS_STAGE_KB");
    const long long stage_kb = std::min(112LL, std::max(0LL, v ? atoll(v) : (long long)EDGPU_SRS_STAGE_KB));
    sh.staged = sh.xs_staged > sh.xs_elems && (long long)sh.xs_staged * (long long)sizeof(T) <= stage_kb * 1024LL;
  }
  return sh;
}

void merge_shape(MvShape &a, const MvShape &b) {
  a.storage = b.storage;
  a.xs_elems = std::max(a.xs_elems, b.xs_elems);
  a.xs_staged = std::max(a.xs_staged, b.xs_staged);
  a.staged = a.staged || b.staged;
}

// ============================================================================ one-off operator application
template <typename T>
void apply_h(edgpu_model *m, Sector *s, const T *x, T *y, const T *z, double cz) {
  edgpu_ctx *c = m->ctx;
  MvTask<T> t{};
  t.op = s->dop<T>();
  t.srs_rows = s->srs_rows;
  t.item_begin = 0;
  t.x = x;
  t.y = y;
  t.z = z;
  t.c = cz;
  t.dot_partial = nullptr;
  std::vector<int> map(s->nitems, 0);
  DBuf dt = upload(c, std::vector<MvTask<T>>{t});
  DBuf dm = upload(c, map);
  MvShape sh = mv_shape<T>(*s);
  sh.plain = z == nullptr;
  launch_mv<T>(dt.as<MvTask<T>>(), dm.as<int>(), s->nitems, sh, c->stream);
  CK(cudaGetLastError());
  sync(c);
  m->st_spmv += 1;
  m->st_work += (double)s->dim;
}

// ============================================================================ eigen-solver
struct EigSectorJob {
  edgpu_model *owner = nullptr;
  Sector *s;
  int nev, m;
  double tol = 1e-12;
  int maxitr = 1000;
  bool eval_only = false;
  std::vector<double> evals;
  std::vector<std::shared_ptr<DBuf>> evecs;
  int info = 0;
  int cycles = 0;
  // multiplicity check: after the nev wanted pairs converge (phase 1), the basis restarts from the
  // converged Ritz vectors plus a fresh random vector and runs until nev + 1 pairs converge (phase 2);
  // a copy of a degenerate eigenvalue missed by the single-vector Krylov space enters below the old
  // nev-th value, and the check repeats until none does.
  bool check = true;
  int check_cycles = 0;  // 0: run the check to convergence; > 0: give it this many restart cycles
  int phase = 1, checks = 0, phase_cycles = 0;
  double last = 0.0;
  std::shared_ptr<DBuf> start;  // first basis vector in the batch's precision (nullptr: a seeded random vector)
  int prec = -1;                // precision of the solve (EDGPU_FP32 / EDGPU_FP64); -1: the call's
  int want = 0;                 // > 0: only the `want` lowest of the nev Ritz pairs must meet tol (all nev kept)
};

// Column stride of an eigen-solver basis: n rounded up to whole 16-byte groups (aligned vector loads).
template <typename T>
long long padded_ld(long long n) {
  const long long v = 16 / (long long)sizeof(T);
  return (n + v - 1) / v * v;
}

// One step of a batch captured once as a CUDA graph and replayed: one launch per step instead of one per
// kernel.  The captured kernels read their tasks from device memory, so the graph stays valid while the
// host rewrites the task array between replays.
struct StepGraph {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  template <class F>
  void capture(cudaStream_t st, F &&fn) {
    const long long before = launch_count();
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    fn();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    kernels = launch_count() - before;
    note_launch(-kernels);  // counted when replayed
    CK(e);
    const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0ull);
    cudaGraphDestroy(g);
    CK(ei);
  }
  void launch(cudaStream_t st) {
    CK(cudaGraphLaunch(exec, st));
    note_launch(kernels);
  }
  ~StepGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// Lock-step thick-restart Lanczos over a changing set of sectors (of one or many models).  Sectors join
// between restart cycles (add) and leave when they finish (cycle reports them); the device state of the
// sectors admitted together lives in one arena group, released when the last of them finishes.  Every
// kernel walks all current sectors; a sector's arithmetic does not depend on which others share the
// launches (fixed-order per-chunk reductions), so a result is the same alone and in any mix.
template <typename T>
class EigBatch {
 public:
  EigBatch(edgpu_model *m, int ld, edgpu_ctx *c = nullptr) : m_(m), c_(c ? c : m->ctx), ld_(ld) {
    if (ld_ > kMaxLd || ld_ > 65) throw ApiError(EDGPU_ERR_ARG, "ncv above 64 is not supported");
    const char *ke = getenv("EDGPU_KEEP_EXTRA");
    keep_extra_ = ke ? atoi(ke) : -1;
    trace_ = getenv("EDGPU_TRACE_BATCH") != nullptr;  // one stderr line per finished sector
    gram_explicit_ = getenv("EDGPU_GRAM_EXPLICIT") != nullptr && atoi(getenv("EDGPU_GRAM_EXPLICIT")) != 0;
    const char *kc = getenv("EDGPU_KEEP_CAP");            // percent of the rest of the basis (default 66)
    if (kc && atoi(kc) > 0 && atoi(kc) < 100) keep_cap_ = atoi(kc);
  }

  size_t active() const { return slots_.size(); }

  // Admit sectors: their bases start from a seeded random vector at the next cycle.
  void add(const std::vector<EigSectorJob *> &jobs) {
    if (jobs.empty()) return;
    for (auto *j : jobs)
      if (j->m + 1 > ld_) throw ApiError(EDGPU_ERR_ARG, "ncv above 64 is not supported");
    std::unique_ptr<Group> g(new Group());
    auto al = [](size_t x) { return (x + 31) & ~size_t(31); };  // 256-byte alignment in units of 8 bytes
    size_t nvec = 0, nsmall = 0;
    for (auto *j : jobs) {
      const long long n = j->s->dim, ldv = padded_ld<T>(n);
      const size_t nch = (size_t)((n + kCgsChunk - 1) / kCgsChunk);
      const size_t gp = (size_t)(j->m + 1) * (j->m + 2) / 2;
      nvec += 2 * al((sizeof(T) * (size_t)(j->m + 1) * ldv + 7) / 8) + al((sizeof(T) * (size_t)ldv + 7) / 8);
      const size_t nsup = (size_t)cgs_nsup((int)nch);
      nsmall += 2 * al((size_t)ld_ * ld_) + 2 * al(nch * ld_) + al(3 * nch) + al(4) + al(nch * gp) +
                al(nsup * (2 * ld_ + 2)) + al(ld_) + al(ld_ / 2 + 1) + al(nsup / 2 + 1);
    }
    g->vec = DBuf(c_->alloc, 8 * nvec);
    g->small = DBuf(c_->alloc, 8 * nsmall);
    g->st = DBuf(c_->alloc, sizeof(int) * 8 * jobs.size());
    g->hst.assign(8 * jobs.size(), 0);
    CK(cudaMemsetAsync(g->small.p, 0, 8 * nsmall, c_->stream));
    for (size_t i = 0; i < jobs.size(); ++i) {
      g->hst[8 * i + 0] = -1;  // no basis vector yet
      g->hst[8 * i + 1] = 1;   // orthogonalise a random vector first
    }
    CK(cudaMemcpyAsync(g->st.p, g->hst.data(), sizeof(int) * g->hst.size(), cudaMemcpyHostToDevice, c_->stream));
    double *pv = g->vec.template as<double>(), *ps = g->small.template as<double>();
    const int gid = (int)groups_.size();
    for (size_t i = 0; i < jobs.size(); ++i) {
      EigSectorJob *j = jobs[i];
      const long long n = j->s->dim, ldv = padded_ld<T>(n);
      const size_t nch = (size_t)((n + kCgsChunk - 1) / kCgsChunk);
      const size_t gp = (size_t)(j->m + 1) * (j->m + 2) / 2;
      const size_t vb = al((sizeof(T) * (size_t)(j->m + 1) * ldv + 7) / 8);
      Slot sl;
      sl.job = j;
      sl.group = gid;
      sl.index = (int)i;
      sl.V = reinterpret_cast<T *>(pv);
      sl.V2 = reinterpret_cast<T *>(pv + vb);
      sl.w = reinterpret_cast<T *>(pv + 2 * vb);
      pv += 2 * vb + al((sizeof(T) * (size_t)ldv + 7) / 8);
      sl.Tm = ps;
      ps += al((size_t)ld_ * ld_);
      sl.E = ps;
      ps += al((size_t)ld_ * ld_);
      sl.hpart = ps;
      ps += al(nch * ld_);
      sl.hpart2 = ps;
      ps += al(nch * ld_);
      sl.npart = ps;
      ps += al(3 * nch);
      sl.nsc = ps;
      ps += al(4);
      sl.gpart = ps;
      sl.gstride = (int)gp;
      ps += al(nch * gp);
      const size_t nsup = (size_t)cgs_nsup((int)nch);
      sl.spart = ps;
      ps += al(nsup * (2 * ld_ + 2));
      sl.hv = ps;
      ps += al(ld_);
      sl.ord = reinterpret_cast<int *>(ps);
      ps += al(ld_ / 2 + 1);
      sl.cnt = reinterpret_cast<int *>(ps);  // zeroed with the arena; every launch leaves it zero
      ps += al(nsup / 2 + 1);
      sl.st = g->st.template as<int>() + 8 * i;
      slots_.push_back(sl);
    }
    g->live = (int)jobs.size();
    groups_.push_back(std::move(g));
    fresh_ = true;
    dirty_ = true;
  }

  // One restart cycle of every current sector: grow each basis to its restart size, Rayleigh-Ritz on
  // the projected matrices, then per sector finish, restart thick, or start the multiplicity check.
  void cycle(std::vector<EigSectorJob *> &finished) {
    if (slots_.empty()) return;
    if (dirty_) rebuild();
    const int nt = (int)slots_.size();
    if (fresh_) {  // random start vectors of the sectors admitted since the last cycle
      launch_eig_random<T>(dtasks_.template as<EigTask<T>>(), cmap_.template as<int>(), nchunks_, c_->stream);
      fresh_ = false;
    }
    for (int guard_steps = 0; guard_steps < 4 * ld_ + 256;) {
      int need = 0;
      for (auto &sl : slots_)
        if (!sl.done) need = std::max(need, sl.job->m - sl.jhost);
      if (need <= 0) break;
      for (int q = 0; q < need; ++q) step_->launch(c_->stream);
      guard_steps += need;
      if (m_) m_->st_steps += need;
      for (auto &sl : slots_)
        if (!sl.done) {
          edgpu_model *ow = sl.job->owner ? sl.job->owner : m_;
          const int k = std::min(need, sl.job->m - sl.jhost);
          if (ow) {
            ow->st_work += (double)k * (double)sl.job->s->dim;
            ow->st_spmv += k;
            if (ow != m_) ow->st_steps += k;
          }
        }
      CK(cudaGetLastError());
      pull_status();
      bool all_full = true;
      for (auto &sl : slots_) {
        if (sl.done) continue;
        const int *st = status_of(sl);
        sl.jhost = st[2] ? sl.job->m : std::min(st[0], sl.job->m - 1);
        if (!st[2]) all_full = false;
      }
      if (all_full) break;
    }
    launch_eig_jacobi<T>(dtasks_.template as<EigTask<T>>(), nt, theta_.template as<double>(), Y_.template as<double>(),
                         resid_.template as<double>(), ld_, work_.template as<double>(), status_.template as<int>(),
                         c_->stream);
    h_theta_.resize((size_t)nt * ld_);
    h_resid_.resize((size_t)nt * ld_);
    CK(cudaMemcpyAsync(h_theta_.data(), theta_.p, sizeof(double) * h_theta_.size(), cudaMemcpyDeviceToHost, c_->stream));
    CK(cudaMemcpyAsync(h_resid_.data(), resid_.p, sizeof(double) * h_resid_.size(), cudaMemcpyDeviceToHost, c_->stream));
    pull_status();
    std::vector<int> restart_k(nt, 0), h_keep(nt, 0);
    std::vector<T *> h_out(nt, nullptr);
    bool any_restart = false, any_done = false;
    for (int i = 0; i < nt; ++i) {
      Slot &sl = slots_[i];
      if (sl.done) continue;
      EigSectorJob &J = *sl.job;
      const double tol = J.tol;
      const int nb = status_of(sl)[0];
      const int nev = std::min(J.nev, nb);
      const int want = J.phase == 2 ? std::min(J.nev + 1, nb) : (J.want > 0 ? std::min(J.want, nev) : nev);
      const double *th_i = &h_theta_[(size_t)i * ld_];
      const double *rs_i = &h_resid_[(size_t)i * ld_];
      double anorm = 0;
      for (int q = 0; q < nb; ++q) anorm = std::max(anorm, std::fabs(th_i[q]));
      auto ok = [&](int q) { return rs_i[q] <= tol * std::max(std::fabs(th_i[q]), 1e-3 * std::max(anorm, 1e-300)); };
      bool conv = true;
      for (int q = 0; q < want; ++q)
        if (!ok(q)) conv = false;
      const bool whole = nb >= J.s->dim;
      if (whole) conv = true;
      const bool give_up = J.cycles >= J.maxitr;
      J.cycles += 1;
      bool check_restart = false;
      if (J.check && J.phase == 2 && J.check_cycles > 0 && !conv && !give_up) {
        // quick check: after `check_cycles` restart cycles of the deflated space, stop unless a new
        // Ritz value has already dropped below the nev-th converged one
        if (++J.phase_cycles >= J.check_cycles && !(th_i[nev - 1] < J.last - 10.0 * tol * std::max(1.0, std::fabs(J.last))))
          conv = true;
      }
      if (conv && !whole && J.check && nev == J.nev && J.m < J.s->dim) {
        if (J.phase == 1) {
          J.phase = 2;
          J.phase_cycles = 0;
          J.last = th_i[nev - 1];
          check_restart = true;
        } else if (th_i[nev - 1] < J.last - 10.0 * tol * std::max(1.0, std::fabs(J.last)) && J.checks < 8) {
          J.checks += 1;
          J.phase_cycles = 0;
          J.last = th_i[nev - 1];
          check_restart = true;
        }
      }
      if (check_restart && !give_up) {
        // restart from the nev converged Ritz vectors and a fresh random vector (mode 1, coupling 0)
        restart_k[i] = -nev;
        h_keep[i] = nev;
        h_out[i] = sl.V2;
        any_restart = true;
      } else if (conv || give_up || nev < J.nev) {
        J.info = conv ? 0 : EDGPU_NOT_CONVERGED;
        int nconv = 0;
        for (int q = 0; q < nev; ++q) {
          if (conv || ok(q)) nconv = q + 1;
          else break;
        }
        J.evals.assign(th_i, th_i + nconv);
        if ((!J.eval_only || sizeof(T) == 4) && nconv > 0) {
          auto ev = std::make_shared<DBuf>(c_->alloc, sizeof(T) * (size_t)nconv * J.s->dim);
          J.evecs.push_back(ev);
          h_keep[i] = -nconv;
          h_out[i] = ev->template as<T>();
        }
        sl.done = true;
        any_done = true;
        restart_k[i] = kEigDone;  // every later kernel skips this sector
        if (trace_)
          fprintf(stderr, "batch<%s>: sector (%d,%d) dim %lld done: cycles %d phase %d checks %d, batch steps %lld\n",
                  sizeof(T) == 4 ? "fp32" : "fp64", J.s->nup, J.s->ndn, J.s->dim, J.cycles, J.phase, J.checks,
                  m_ ? m_->st_steps : -1ll);
      } else {
        // thick restart: keep the wanted Ritz vectors plus one more per wanted pair that has converged (at least
        // one, at most two thirds of the rest of the basis), as ARPACK's dsaup2 grows its kept set; the rest of
        // the basis is rebuilt by new Lanczos steps.  On Anderson-12 this took 18 % fewer element-steps than a
        // fixed (ncv - nev) / 4 (caps of one half: 4 % more; 75-95 %: the same as two thirds).  EDGPU_KEEP_EXTRA = n
        // keeps a fixed n instead, EDGPU_KEEP_CAP = p caps at p % of the rest.
        const int base = J.phase == 2 ? J.nev + 1 : J.nev;
        int extra;
        if (keep_extra_ >= 0) {
          extra = keep_extra_;
        } else {
          int nc = 0;
          for (int q = 0; q < want; ++q)
            if (ok(q)) ++nc;
          extra = std::max(1, std::min(nc, keep_cap_ * (nb - base) / 100));
        }
        int k = std::min(nb - 1, base + extra);
        k = std::max(k, std::min(base, nb - 1));
        restart_k[i] = k;
        h_keep[i] = k;
        h_out[i] = sl.V2;
        any_restart = true;
      }
    }
    CK(cudaMemcpyAsync(keep_.p, h_keep.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, c_->stream));
    CK(cudaMemcpyAsync(outv_.p, h_out.data(), sizeof(T *) * nt, cudaMemcpyHostToDevice, c_->stream));
    launch_eig_restart<T>(dtasks_.template as<EigTask<T>>(), cmap_.template as<int>(), nchunks_, keep_.template as<int>(),
                          Y_.template as<double>(), ld_, outv_.template as<T *>(), c_->stream);
    CK(cudaGetLastError());
    if (any_restart) {
      if (m_) m_->st_restarts += 1;
      bool draw = false;
      for (int i = 0; i < nt; ++i) {
        if (!restart_k[i] || restart_k[i] == kEigDone) continue;
        const bool fresh = restart_k[i] < 0;  // multiplicity check: random vector instead of the residual
        const int k = fresh ? -restart_k[i] : restart_k[i];
        std::swap(slots_[i].V, slots_[i].V2);
        tasks_[i].V = slots_[i].V;
        if (fresh) draw = true;
        slots_[i].jhost = fresh ? k - 1 : k;
      }
      // the kept vectors' Gram block for the one-pass orthogonalisation, from the old block and Y (before the
      // reset changes the basis sizes); EDGPU_GRAM_EXPLICIT=1 measures it over the new vectors instead
      CK(cudaMemcpyAsync(rkbuf_.p, restart_k.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, c_->stream));
      if (!gram_explicit_)
        launch_eig_gram_proj<T>(dtasks_.template as<EigTask<T>>(), nt, rkbuf_.template as<int>(),
                                Y_.template as<double>(), ld_, c_->stream);
      // projected matrices, basis sizes and modes reset on the device in one launch
      CK(cudaMemcpyAsync(dtasks_.p, tasks_.data(), sizeof(EigTask<T>) * nt, cudaMemcpyHostToDevice, c_->stream));
      launch_eig_reset<T>(dtasks_.template as<EigTask<T>>(), nt, rkbuf_.template as<int>(), theta_.template as<double>(),
                          ld_, c_->stream);
      if (gram_explicit_)
        launch_eig_gram<T>(dtasks_.template as<EigTask<T>>(), cmap_.template as<int>(), nchunks_, nt,
                           rkbuf_.template as<int>(), c_->stream);
      // a fresh w (from the task's own seed and draw count) for every task now in mode 1
      if (draw) launch_eig_random<T>(dtasks_.template as<EigTask<T>>(), cmap_.template as<int>(), nchunks_, c_->stream);
    }
    sync(c_);
    if (take_mv_stall() || take_cgs_stall())
      throw ApiError(EDGPU_ERR_CUDA, "a bulk copy into shared memory did not complete");
    if (any_done) retire(finished);  // finished sectors leave before any further launch
  }

 private:
  struct Group {
    DBuf vec, small, st;
    std::vector<int> hst;  // host copy of the status words
    int live = 0;
  };
  struct Slot {
    EigSectorJob *job = nullptr;
    int group = 0, index = 0;
    T *V = nullptr, *V2 = nullptr, *w = nullptr;
    double *Tm = nullptr, *E = nullptr, *hpart = nullptr, *hpart2 = nullptr, *npart = nullptr, *nsc = nullptr,
           *gpart = nullptr, *spart = nullptr, *hv = nullptr;
    int *cnt = nullptr, *ord = nullptr;
    int gstride = 0;
    int *st = nullptr;
    int jhost = -1;
    bool done = false;
  };

  const int *status_of(const Slot &sl) const { return &groups_[sl.group]->hst[8 * (size_t)sl.index]; }

  void pull_status() {
    for (auto &g : groups_)
      if (g && g->live > 0)
        CK(cudaMemcpyAsync(g->hst.data(), g->st.p, sizeof(int) * g->hst.size(), cudaMemcpyDeviceToHost, c_->stream));
    sync(c_);
  }

  // Finished sectors leave the batch; an arena group is released with its last sector.
  void retire(std::vector<EigSectorJob *> &finished) {
    std::vector<Slot> keep;
    for (auto &sl : slots_) {
      if (!sl.done) {
        keep.push_back(sl);
        continue;
      }
      finished.push_back(sl.job);
      if (--groups_[sl.group]->live == 0) groups_[sl.group].reset();
    }
    slots_.swap(keep);
    dirty_ = true;
  }

  // Device task array, item / chunk maps, per-launch work arrays and the step graph of the current set.
  void rebuild() {
    const int nt = (int)slots_.size();
    tasks_.assign(nt, EigTask<T>{});
    std::vector<int> item_task, chunk_task, leaders;
    shape_ = MvShape{slots_[0].job->s->storage, 0};
    for (int i = 0; i < nt; ++i) {
      const Slot &sl = slots_[i];
      const Sector &s = *sl.job->s;
      const long long n = s.dim;
      const int nch = (int)((n + kCgsChunk - 1) / kCgsChunk);
      EigTask<T> &t = tasks_[i];
      t.op = s.dop<T>();
      t.srs_rows = s.srs_rows;
      t.item_begin = (int)item_task.size();
      t.nitems = s.nitems;
      t.chunk_begin = (int)chunk_task.size();
      t.nchunks = nch;
      t.n = n;
      t.ldv = padded_ld<T>(n);
      t.m = sl.job->m;
      t.ld = ld_;
      t.V = sl.V;
      t.w = sl.w;
      t.Tm = sl.Tm;
      t.hpart = sl.hpart;
      t.hpart2 = sl.hpart2;
      t.spart = sl.spart;
      t.hv = sl.hv;
      t.ord = sl.ord;
      t.cnt = sl.cnt;
      t.npart = sl.npart;
      t.nsc = sl.nsc;
      t.E = sl.E;
      t.gpart = sl.gpart;
      t.gstride = sl.gstride;
      t.st = sl.st;
      t.seed = 0x5eed0000ull ^ ((unsigned long long)s.nup << 32) ^ ((unsigned long long)s.ndn << 8) ^
               (unsigned long long)s.storage;
      t.start = sl.job->start ? sl.job->start->template as<T>() : nullptr;
      for (int q = 0; q < s.nitems; ++q) item_task.push_back(i);
      for (int q = 0; q < nch; ++q) {
        if (q % kCgsSup == 0) leaders.push_back((int)chunk_task.size());
        chunk_task.push_back(i);
      }
      merge_shape(shape_, mv_shape<T>(s));
    }
    dtasks_ = upload(c_, tasks_);
    dmap_ = upload(c_, item_task);
    cmap_ = upload(c_, chunk_task);
    lmap_ = upload(c_, leaders);
    nleaders_ = (int)leaders.size();
    nitems_ = (int)item_task.size();
    nchunks_ = (int)chunk_task.size();
    theta_ = DBuf(c_->alloc, sizeof(double) * (size_t)nt * ld_);
    Y_ = DBuf(c_->alloc, sizeof(double) * (size_t)nt * ld_ * ld_);
    resid_ = DBuf(c_->alloc, sizeof(double) * (size_t)nt * ld_);
    work_ = DBuf(c_->alloc, sizeof(double) * (size_t)nt * 4 * ld_ * ld_);  // the projected eigen-solve's workspace
    status_ = DBuf(c_->alloc, sizeof(int) * nt);
    keep_ = DBuf(c_->alloc, sizeof(int) * nt);
    outv_ = DBuf(c_->alloc, sizeof(T *) * nt);
    rkbuf_ = DBuf(c_->alloc, sizeof(int) * nt);
    // The operator tuner: on the batch's first build every variant of the eigen-step operator (blocks per
    // SM x source-row staging; all compute the same sums in the same order) is timed on the batch's own
    // tasks and the fastest kept for the batch's life and recorded in the model of its first sector.
    // EDGPU_OP_TUNE=0 turns it off; a set EDGPU_SRS_STAGE_KB fixes the staging choice.
    if (!tuned_) {
      tuned_ = true;
      const char *off = getenv("EDGPU_OP_TUNE");
      if (!(off && atoi(off) == 0) && shape_.storage == kSRS) {
        long long maxld = 1;
        for (auto &sl : slots_) maxld = std::max(maxld, padded_ld<T>(sl.job->s->dim));
        DBuf scratch(c_->alloc, sizeof(T) * (size_t)maxld);
        tune_ = tune_eig_mv<T>(dtasks_.template as<EigTask<T>>(), dmap_.template as<int>(), nitems_, shape_,
                               scratch.template as<T>(), c_->stream);
        sync(c_);
        edgpu_model *owner = slots_[0].job->owner ? slots_[0].job->owner : m_;
        owner->op_tune[sizeof(T) == 4 ? 1 : 0] = tune_;
      }
    }
    if (tune_.done && tune_.ms > 0) {
      shape_.mb = tune_.mb;
      if (!getenv("EDGPU_SRS_STAGE_KB")) shape_.staged = tune_.staged;
    }
    prepare_eig_step<T>(shape_);
    step_.reset(new StepGraph());
    EigTask<T> *dt = dtasks_.template as<EigTask<T>>();
    const int *dm = dmap_.template as<int>(), *cm = cmap_.template as<int>(), *lm = lmap_.template as<int>();
    const int ni = nitems_, nc = nchunks_, nl = nleaders_;
    const MvShape sh = shape_;
    step_->capture(c_->stream, [&]() { launch_eig_step<T>(dt, dm, ni, cm, nc, lm, nl, nt, sh, c_->stream); });
    dirty_ = false;
  }

  edgpu_model *m_;
  edgpu_ctx *c_;
  int ld_;
  int keep_extra_ = -1;
  bool trace_ = false;
  bool gram_explicit_ = false;
  int keep_cap_ = 66;
  bool tuned_ = false;
  OpTuning tune_;
  bool dirty_ = true, fresh_ = false;
  std::vector<std::unique_ptr<Group>> groups_;
  std::vector<Slot> slots_;
  std::vector<EigTask<T>> tasks_;
  DBuf dtasks_, dmap_, cmap_, lmap_, theta_, Y_, resid_, work_, status_, keep_, outv_, rkbuf_;
  int nitems_ = 0, nchunks_ = 0, nleaders_ = 0;
  MvShape shape_{};
  std::unique_ptr<StepGraph> step_;
  std::vector<double> h_theta_, h_resid_;
};

template <typename T>
void solve_batch(edgpu_model *m, std::vector<EigSectorJob *> &jobs) {
  if (jobs.empty()) return;
  int mmax = 0;
  for (auto *j : jobs) mmax = std::max(mmax, j->m);
  EigBatch<T> b(m, mmax + 1);
  b.add(jobs);
  std::vector<EigSectorJob *> finished;
  while (b.active()) b.cycle(finished);
}

// FP64 Rayleigh-Ritz refinement of the FP32 Ritz vectors of a group of solved sectors: W = H X with the
// FP64 operator, then the projected generalised problem (X^T W, X^T X) in FP64 (krylov.cu, k_rr_*).
// Eigenvalues then carry the square of the FP32 vectors' error.
void refine_fp32(edgpu_model *m, std::vector<EigSectorJob *> &jobs) {
  edgpu_ctx *c = m->ctx;
  std::vector<RrTask> rr;
  std::vector<int> rr_items, mv_items;
  std::vector<MvTask<double>> mv;
  std::vector<EigSectorJob *> owner;
  std::vector<DBuf> keep;
  MvShape shape{jobs.empty() ? 1 : jobs[0]->s->storage, 0};
  int nref = 0;
  for (auto *J : jobs) {
    const int k = (int)J->evals.size();
    if (k >= 1 && k <= 32 && !J->evecs.empty()) ++nref;
  }
  if (!nref) return;
  // Ritz values / rotations and statuses of every refined sector in one buffer each (one copy back)
  DBuf thy(c->alloc, sizeof(double) * (size_t)nref * (32 + 32 * 32)), stat(c->alloc, sizeof(int) * (size_t)nref * 4);
  for (auto *J : jobs) {
    const int k = (int)J->evals.size();
    if (k < 1 || k > 32 || J->evecs.empty()) continue;
    const long long n = J->s->dim;
    keep.emplace_back(c->alloc, sizeof(double) * (size_t)k * n);
    double *X = keep.back().as<double>();
    keep.emplace_back(c->alloc, sizeof(double) * (size_t)k * n);
    double *W = keep.back().as<double>();
    const int nit = (int)((n + kItemElems - 1) / kItemElems);
    keep.emplace_back(c->alloc, sizeof(double) * (size_t)nit * 2 * k * k);
    double *part = keep.back().as<double>();
    double *theta = thy.as<double>() + rr.size() * (32 + 32 * 32);
    int *status = stat.as<int>() + rr.size() * 4;
    launch_to_double<float>(J->evecs[0]->as<float>(), X, (long long)k * n, c->stream);
    for (int q = 0; q < k; ++q) {
      MvTask<double> t{};
      t.op = J->s->dop<double>();
      t.srs_rows = J->s->srs_rows;
      t.item_begin = (int)mv_items.size();
      t.x = X + (size_t)q * n;
      t.y = W + (size_t)q * n;
      mv.push_back(t);
      for (int it = 0; it < J->s->nitems; ++it) mv_items.push_back((int)mv.size() - 1);
    }
    merge_shape(shape, mv_shape<double>(*J->s));
    RrTask r{};
    r.n = n;
    r.k = k;
    r.item_begin = (int)rr_items.size();
    r.nitems = nit;
    r.X = X;
    r.W = W;
    r.part = part;
    r.theta = theta;
    r.Y = theta + 32;
    r.out = J->evecs[0]->as<float>();
    r.status = status;
    rr.push_back(r);
    for (int it = 0; it < nit; ++it) rr_items.push_back((int)rr.size() - 1);
    owner.push_back(J);
    m->st_spmv += k;
    m->st_work += (double)k * (double)n;
  }
  if (rr.empty()) return;
  DBuf dmv = upload(c, mv), dmvi = upload(c, mv_items), drr = upload(c, rr), drri = upload(c, rr_items);
  DBuf work(c->alloc, sizeof(double) * rr.size() * 4 * 64 * 64);
  shape.plain = 1;  // W = H X: no z term, no dots
  launch_mv<double>(dmv.as<MvTask<double>>(), dmvi.as<int>(), (int)mv_items.size(), shape, c->stream);
  launch_rr(drr.as<RrTask>(), drri.as<int>(), (int)rr_items.size(), (int)rr.size(), work.as<double>(), c->stream);
  CK(cudaGetLastError());
  std::vector<double> th(rr.size() * (32 + 32 * 32));
  std::vector<int> stt(rr.size() * 4);
  CK(cudaMemcpyAsync(th.data(), thy.p, sizeof(double) * th.size(), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(stt.data(), stat.p, sizeof(int) * stt.size(), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  for (size_t q = 0; q < rr.size(); ++q) {
    const double *tq = th.data() + q * (32 + 32 * 32);
    if (stt[q * 4] == 0) owner[q]->evals.assign(tq, tq + rr[q].k);
  }
}

// Sectors of one model for Hamiltonian::diag, in the reference order: dim-1 sectors are solved on the spot
// (eigen-pair (H_00, [1]), Storage.h:53-60), the others become eigen-solver jobs.
struct DiagSlot {
  int kind;  // 1: one-state sector, 2: eigen-solver job
  double zero_e;
  Sector *s;
  EigSectorJob *job;
};

template <typename T>
void diag_prepare(edgpu_model *m, const edgpu_diag_params *p, std::vector<DiagSlot> &slots,
                  std::vector<std::unique_ptr<EigSectorJob>> &jobs) {
  edgpu_ctx *c = m->ctx;
  if (p->nev < 1) throw ApiError(EDGPU_ERR_ARG, "arpack.NEV must be positive");
  const int ncv_p = p->ncv > 0 ? p->ncv : 2 * p->nev + 3;
  const double tol = p->tol > 0 ? p->tol : (sizeof(T) == 8 ? 1e-12 : 2e-6);
  const int maxitr = p->maxitr > 0 ? p->maxitr : 1000;
  const bool evals_only = p->eigenvalues_only != 0;
  std::vector<int> order(2 * ((m->ns + 1) * (m->ns + 1) + std::max(0, p->n_sectors)));
  const int nsec = sector_order(m, p->sectors, p->sectors ? p->n_sectors : 0, order.data());
  m->pairs.clear();
  m->have_pairs = false;
  m->evals_only = evals_only;
  m->diag_storage = p->storage;
  m->diag_ncv = p->ncv;
  m->diag_maxitr = maxitr;
  m->st_spmv = m->st_steps = m->st_restarts = 0;
  m->st_work = 0;
  for (int q = 0; q < nsec; ++q) {
    int nup = order[2 * q], ndn = order[2 * q + 1];
    Sector *s = get_sector(m, p->storage, nup, ndn);
    if (s->dim == 0) continue;
    if (s->dim == 1) {
      double e = 0;
      CK(cudaMemcpyAsync(&e, s->diag64.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      sync(c);
      slots.push_back({1, e, s, nullptr});
      continue;
    }
    const int ncv = (int)std::min<long long>(ncv_p, s->dim);
    std::unique_ptr<EigSectorJob> J(new EigSectorJob());
    J->owner = m;
    J->s = s;
    J->nev = std::min(p->nev, ncv - 1);
    J->m = ncv;
    J->tol = tol;
    J->maxitr = maxitr;
    J->eval_only = evals_only;
    J->check = p->multiplicity_check != 1;
    J->check_cycles = p->multiplicity_check >= 2 ? p->multiplicity_check - 1 : 0;
    slots.push_back({2, 0.0, s, J.get()});
    jobs.push_back(std::move(J));
  }
}

// Eigen-pairs of a model once all its jobs have finished: insertion ids in the reference's sector order,
// stable sort by energy (the std::set<EigenPair> order).  Returns the worst job status.
template <typename T>
int diag_finish(edgpu_model *m, std::vector<DiagSlot> &slots, int *npairs) {
  edgpu_ctx *c = m->ctx;
  const int prec = sizeof(T) == 8 ? EDGPU_FP64 : EDGPU_FP32;
  int worst = 0, id = 0;
  for (auto &sl : slots) {
    if (sl.kind == 1) {
      auto ev = std::make_shared<DBuf>(c->alloc, sizeof(T));
      T one = (T)1;
      CK(cudaMemcpyAsync(ev->p, &one, sizeof(T), cudaMemcpyHostToDevice, c->stream));
      m->pairs.push_back(Pair{sl.zero_e, sl.s->nup, sl.s->ndn, id++, prec, 1, ev, 0});
    } else {
      EigSectorJob &J = *sl.job;
      if (m->evals_only) J.evecs.clear();
      if (J.info) worst = J.info;
      const long long n = J.s->dim;
      std::shared_ptr<DBuf> blk = J.evecs.empty() ? nullptr : J.evecs[0];
      const int jp = J.prec >= 0 ? J.prec : prec;
      for (size_t q = 0; q < J.evals.size(); ++q)
        m->pairs.push_back(Pair{J.evals[q], J.s->nup, J.s->ndn, id++, jp, n, blk, (long long)q * n});
    }
  }
  std::stable_sort(m->pairs.begin(), m->pairs.end(), [](const Pair &a, const Pair &b) { return a.E < b.E; });
  m->have_pairs = true;
  if (npairs) *npairs = (int)m->pairs.size();
  sync(c);
  return worst;
}

// Hamiltonian::diag for `count` models at once: every sector of every model goes into the same batched
// eigen-solve (one launch per phase covers all of them), then each model gets its eigen-pairs in its own
// reference order.  A single model is the count == 1 case.
template <typename T>
int diag_many_impl(edgpu_model *const *ms, int count, const edgpu_diag_params *p, int *npairs) {
  if (count < 1) throw ApiError(EDGPU_ERR_ARG, "no models");
  edgpu_ctx *c = ms[0]->ctx;
  for (int q = 0; q < count; ++q)
    if (!ms[q] || ms[q]->ctx != c) throw ApiError(EDGPU_ERR_ARG, "models of one batch must share a context");
  std::vector<std::vector<DiagSlot>> slots(count);
  std::vector<std::unique_ptr<EigSectorJob>> jobs;
  for (int mi = 0; mi < count; ++mi) diag_prepare<T>(ms[mi], p, slots[mi], jobs);
  // batches bounded by memory and max_batch over every sector of every model
  std::vector<EigSectorJob *> group;
  size_t gbytes = 0;
  const size_t gcap = (size_t)24 << 30;
  const size_t gmax = p->max_batch > 0 ? (size_t)std::min(p->max_batch, 2048) : 2048;
  auto flush = [&]() {
    if (group.empty()) return;
    solve_batch<T>(ms[0], group);
    if (sizeof(T) == 4) refine_fp32(ms[0], group);
    group.clear();
    gbytes = 0;
  };
  for (auto &J : jobs) {
    size_t bytes = sizeof(T) * (size_t)(2 * J->m + 3) * J->s->dim;
    if (!group.empty() && (group.size() >= gmax || gbytes + bytes > gcap)) flush();
    group.push_back(J.get());
    gbytes += bytes;
  }
  flush();
  int worst = 0;
  for (int mi = 0; mi < count; ++mi) {
    const int w = diag_finish<T>(ms[mi], slots[mi], npairs ? npairs + mi : nullptr);
    if (w) worst = w;
  }
  return worst;
}

// FP64 continuation of an FP32 eigen-solve for the pairs a Boltzmann average keeps.  An FP32 Ritz vector
// carries an error of order 1e-6 after its FP64 Rayleigh-Ritz refinement, which the Green's functions and
// susceptibilities inherit at first order; the FP64 eigenvalues do not need it (their error is the square).
// Per sector holding kept FP32 pairs (they are the sector's k lowest): the sector's thick-restart Lanczos runs
// again in FP64 for its d distinct eigenvalues among those k, from a start vector that combines the k FP32
// Ritz vectors with fixed pseudo-random weights, so the unwanted directions start at the FP32 level and only
// the remaining digits are iterated for.  A single start vector spans one direction of a degenerate
// eigenvalue, so a sector whose kept eigenvalues repeat (within 1e-9 relative) runs as many continuations as
// the largest multiplicity, with independent weights, and each degenerate eigenspace is assembled from their
// Ritz vectors by Gram-Schmidt in FP64.  The kept pairs then hold FP64 vectors; their eigenvalues (already
// FP64 from the Rayleigh-Ritz step) are left as they are, so neither the pair order nor the Boltzmann weights
// change.  Every sector of every model of the call shares the batched eigen-solver launches.
int refine_kept(edgpu_model *const *ms, int count, double beta, double cutoff) {
  if (count < 1) return EDGPU_OK;
  edgpu_ctx *c = ms[0]->ctx;
  struct Plan {
    edgpu_model *m;
    Sector *s;
    std::vector<int> idx;   // indices into m->pairs of every pair of the sector, ascending
    std::vector<int> cl;    // cluster (distinct eigenvalue) of each
    int kept = 0;           // idx[0, kept): the pairs to refine (up to the sector's highest kept FP32 one)
    int ncl = 0, ncl_kept = 0, njobs = 0, first_job = 0;
    std::vector<double> ecl;  // eigenvalue of each cluster
  };
  std::vector<Plan> plans;
  std::vector<std::unique_ptr<EigSectorJob>> jobs;
  for (int mi = 0; mi < count; ++mi) {
    edgpu_model *m = ms[mi];
    if (!m->have_pairs || m->pairs.empty() || m->evals_only) continue;
    double E0, Z;
    std::vector<Kept> keep;
    boltzmann(m, beta, cutoff, E0, Z, keep);
    std::vector<std::pair<int, int>> secs;
    for (auto &kp : keep)
      if (kp.pair->prec == EDGPU_FP32 && kp.pair->n > 1) {
        std::pair<int, int> sk(kp.pair->nup, kp.pair->ndn);
        if (std::find(secs.begin(), secs.end(), sk) == secs.end()) secs.push_back(sk);
      }
    for (auto &sk : secs) {
      Plan P;
      P.m = m;
      P.s = get_sector(m, m->diag_storage, sk.first, sk.second);
      // the sector's pairs in ascending order up to its highest kept FP32 one (pairs refined by an earlier call
      // at a lower temperature are part of the seed and are refined again with the rest)
      std::vector<int> all;
      int last_kept = -1;
      for (size_t q = 0; q < m->pairs.size(); ++q) {
        const Pair &pr = m->pairs[q];
        if (pr.nup != sk.first || pr.ndn != sk.second) continue;
        all.push_back((int)q);
        const double bf = std::exp(-(pr.E - E0) * beta);
        if (pr.prec == EDGPU_FP32 &&
            (bf >= cutoff || std::fabs(cutoff - bf) <= std::numeric_limits<double>::epsilon()))
          last_kept = (int)all.size() - 1;
      }
      if (last_kept < 0) continue;
      if (m->pairs[all[last_kept]].no_refine) continue;  // a continuation of this sector failed before
      P.idx = all;
      P.kept = last_kept + 1;
      int run = 0;
      for (size_t q = 0; q < P.idx.size(); ++q) {
        const double e = m->pairs[P.idx[q]].E;
        if (q == 0 || std::fabs(e - P.ecl.back()) > 1e-9 * std::max(1.0, std::fabs(e))) {
          P.ecl.push_back(e);
          run = 0;
        }
        ++run;
        P.cl.push_back((int)P.ecl.size() - 1);
        if ((int)q < P.kept) P.njobs = std::max(P.njobs, run);
      }
      P.ncl = (int)P.ecl.size();
      P.ncl_kept = P.cl[P.kept - 1] + 1;
      const long long n = P.s->dim;
      const int ncv_p = m->diag_ncv > 0 ? m->diag_ncv : 0;
      const int k = (int)P.idx.size();
      // the basis of the original solve (arpack.NCV, or 2 NEV + 3 with NEV at least the sector's pair count)
      int ncv = ncv_p > 0 ? ncv_p : 2 * (int)all.size() + 3;
      ncv = (int)std::min<long long>(std::max(ncv, P.ncl + 2), n);
      if (ncv > 64) ncv = 64;
      // the seeds: pair q of the sector weighs w(job, q), a fixed pseudo-random value in +-[0.5, 1.5)
      std::vector<const void *> vptr(k);
      std::vector<int> is64(k);
      for (int q = 0; q < k; ++q) {
        const Pair &pr = m->pairs[P.idx[q]];
        is64[q] = pr.prec == EDGPU_FP64;
        vptr[q] = is64[q] ? (const void *)pr.vec<double>() : (const void *)pr.vec<float>();
      }
      DBuf dptrs = upload(c, vptr), d64 = upload(c, is64);
      P.first_job = (int)jobs.size();
      for (int r = 0; r < P.njobs; ++r) {
        std::vector<double> w(k);
        for (int q = 0; q < k; ++q) {
          unsigned long long h = 0x9e3779b97f4a7c15ull * (unsigned long long)(r * 131 + q + 1);
          h ^= h >> 29;
          h *= 0xbf58476d1ce4e5b9ull;
          h ^= h >> 32;
          const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
          w[q] = (u < 0.5 ? -1.0 : 1.0) * (0.5 + 2.0 * std::fabs(u - 0.5));
        }
        DBuf dw = upload(c, w);
        std::unique_ptr<EigSectorJob> J(new EigSectorJob());
        J->owner = m;
        J->s = P.s;
        // every distinct eigenvalue the FP32 solve found in the sector is in the seed and kept through the
        // restarts, so a kept pair's error only has to be damped against the sector's spectrum beyond them (the
        // gap to its nearest neighbour in the sector no longer sets the rate); only the kept ones must converge
        J->nev = P.ncl;
        J->want = P.ncl_kept;
        J->m = ncv;
        // residuals to 1e-13 |E|: the static observables and the chi_N zero-frequency term (which multiplies
        // the error of <N> by 2 beta <N>) inherit the vectors' error at first order
        J->tol = 1e-13;
        J->maxitr = std::min(m->diag_maxitr, 300);
        J->eval_only = false;
        J->check = false;
        J->start = std::make_shared<DBuf>(c->alloc, sizeof(double) * (size_t)n);
        launch_seed_combine(dptrs.as<const void *>(), d64.as<int>(), dw.as<double>(), k, n, J->start->as<double>(),
                            c->stream);
        sync(c);  // the weights' buffers are released on return
        jobs.push_back(std::move(J));
      }
      plans.push_back(std::move(P));
    }
  }
  if (jobs.empty()) return EDGPU_OK;
  const bool trace = getenv("EDGPU_TRACE_REFINE") != nullptr;
  if (trace)
    for (auto &P : plans)
      fprintf(stderr, "refine: sector (%d,%d) dim %lld pairs %zu clusters %d continuations %d E[0] %.15g\n", P.s->nup,
              P.s->ndn, P.s->dim, P.idx.size(), P.ncl, P.njobs, P.ecl[0]);
  // batches bounded by device memory, as in Hamiltonian::diag
  {
    std::vector<EigSectorJob *> group;
    size_t gbytes = 0;
    const size_t gcap = (size_t)24 << 30;
    for (auto &J : jobs) {
      const size_t bytes = sizeof(double) * (size_t)(2 * J->m + 4) * J->s->dim;
      if (!group.empty() && gbytes + bytes > gcap) {
        solve_batch<double>(ms[0], group);
        group.clear();
        gbytes = 0;
      }
      group.push_back(J.get());
      gbytes += bytes;
    }
    solve_batch<double>(ms[0], group);
  }
  int worst = EDGPU_OK;
  DBuf parts(c->alloc, sizeof(double) * 64), dot(c->alloc, sizeof(double));
  for (auto &P : plans) {
    const long long n = P.s->dim;
    if (trace)
      for (int r = 0; r < P.njobs; ++r) {
        const EigSectorJob &J = *jobs[P.first_job + r];
        fprintf(stderr, "refine: sector (%d,%d) continuation %d: cycles %d info %d converged %zu E %.15g (%.3g from FP32)\n",
                P.s->nup, P.s->ndn, r, J.cycles, J.info, J.evals.size(), J.evals.empty() ? 0.0 : J.evals[0],
                J.evals.empty() ? 0.0 : J.evals[0] - P.ecl[0]);
      }
    bool ok = true;
    for (int r = 0; r < P.njobs && ok; ++r) {
      const EigSectorJob &J = *jobs[P.first_job + r];
      if (J.info || (int)J.evals.size() < P.ncl_kept || J.evecs.empty()) ok = false;
      for (int g = 0; ok && g < P.ncl_kept; ++g)
        if (std::fabs(J.evals[g] - P.ecl[g]) > 1e-8 * std::max(1.0, std::fabs(P.ecl[g]))) ok = false;
    }
    if (!ok) {  // the continuation did not reach the FP32 solve's eigenvalues: the pairs keep their FP32 vectors
      worst = EDGPU_NOT_CONVERGED;
      for (int q = 0; q < P.kept; ++q) P.m->pairs[P.idx[q]].no_refine = true;
      continue;
    }
    const int k = P.kept;
    auto out = std::make_shared<DBuf>(c->alloc, sizeof(double) * (size_t)k * n);
    double *B = out->as<double>();
    for (int q = 0, q0 = 0; q < k; ++q) {
      const int g = P.cl[q];
      if (q > 0 && P.cl[q - 1] != g) q0 = q;
      const int r = q - q0;  // the r-th member of cluster g comes from continuation r
      const EigSectorJob &J = *jobs[P.first_job + r];
      double *dst = B + (size_t)q * n;
      CK(cudaMemcpyAsync(dst, J.evecs[0]->as<double>() + (size_t)g * n, sizeof(double) * (size_t)n,
                         cudaMemcpyDeviceToDevice, c->stream));
      if (r > 0) {  // Gram-Schmidt against the cluster's earlier members, then normalise
        for (int pq = q0; pq < q; ++pq) {
          launch_dot_partials<double>(B + (size_t)pq * n, dst, n, parts.as<double>(), 64, c->stream);
          launch_reduce(parts.as<double>(), 64, dot.as<double>(), c->stream);
          launch_axpy_dev(dst, B + (size_t)pq * n, dot.as<double>(), n, c->stream);
        }
        launch_dot_partials<double>(dst, dst, n, parts.as<double>(), 64, c->stream);
        launch_reduce(parts.as<double>(), 64, dot.as<double>(), c->stream);
        launch_scale<double>(dst, n, dot.as<double>(), 1, c->stream);
      }
    }
    CK(cudaGetLastError());
    for (int q = 0; q < k; ++q) {
      Pair &pr = P.m->pairs[P.idx[q]];
      pr.block = out;
      pr.offset = (long long)q * n;
      pr.prec = EDGPU_FP64;
    }
  }
  sync(c);
  return worst;
}

template <typename T>
int diag_impl(edgpu_model *m, const edgpu_diag_params *p, int *npairs) {
  return diag_many_impl<T>(&m, 1, p, npairs);
}

// Hamiltonian::diag in EDGPU_MIXED precision: every sector with FP32 vectors and the FP64 Rayleigh-Ritz step
// (eigenvalues to FP64 accuracy), except sectors asking for more than 32 pairs (beyond that step) and sectors
// whose basis spans the whole sector (at most ncv states: one restart cycle; the FP32 basis of a whole space
// with degenerate multiplets does not give the lowest nev of them), which are solved in FP64.  The FP32 pairs
// are continued in FP64 later, by the FP64 Green's-function calls or edgpu_refine_eigenpairs, where a
// Boltzmann average keeps them.  (Solving every sector up to 16384 states in FP64 instead puts them in a second
// lock-step batch whose latency-bound steps are not hidden behind the large sectors': on the 12-orbital
// Anderson model it cost 0.29 s per solve.)
inline bool mixed_in_fp64(const EigSectorJob &J) { return J.nev > 32 || (long long)J.m >= J.s->dim; }

int diag_many_mixed(edgpu_model *const *ms, int count, const edgpu_diag_params *p, int *npairs) {
  if (count < 1) throw ApiError(EDGPU_ERR_ARG, "no models");
  edgpu_ctx *c = ms[0]->ctx;
  for (int q = 0; q < count; ++q)
    if (!ms[q] || ms[q]->ctx != c) throw ApiError(EDGPU_ERR_ARG, "models of one batch must share a context");
  std::vector<std::vector<DiagSlot>> slots(count);
  std::vector<std::unique_ptr<EigSectorJob>> jobs;
  for (int mi = 0; mi < count; ++mi) diag_prepare<double>(ms[mi], p, slots[mi], jobs);
  std::vector<EigSectorJob *> j64, j32;
  for (auto &J : jobs) {
    if (mixed_in_fp64(*J)) {
      J->prec = EDGPU_FP64;
      j64.push_back(J.get());
    } else {
      J->prec = EDGPU_FP32;
      J->tol = p->tol > 0 ? p->tol : 2e-6;
      j32.push_back(J.get());
    }
  }
  const size_t gcap = (size_t)24 << 30;
  const size_t gmax = p->max_batch > 0 ? (size_t)std::min(p->max_batch, 2048) : 2048;
  auto run = [&](std::vector<EigSectorJob *> &list, auto tag) {
    using T = decltype(tag);
    std::vector<EigSectorJob *> group;
    size_t gbytes = 0;
    auto flush = [&]() {
      if (group.empty()) return;
      solve_batch<T>(ms[0], group);
      if (sizeof(T) == 4) refine_fp32(ms[0], group);
      group.clear();
      gbytes = 0;
    };
    for (auto *J : list) {
      const size_t bytes = sizeof(T) * (size_t)(2 * J->m + 3) * J->s->dim;
      if (!group.empty() && (group.size() >= gmax || gbytes + bytes > gcap)) flush();
      group.push_back(J);
      gbytes += bytes;
    }
    flush();
  };
  run(j64, double());
  run(j32, float());
  int worst = 0;
  for (int mi = 0; mi < count; ++mi) {
    const int w = diag_finish<double>(ms[mi], slots[mi], npairs ? npairs + mi : nullptr);
    if (w) worst = w;
  }
  return worst;
}

// Storage::diag for one sector (Storage.h:43-146): eigenvalues ascending, Ritz vectors to the host.
template <typename T>
int diag_sector_impl(edgpu_model *m, const edgpu_diag_params *p, int nup, int ndn, double *evals, int *nconv,
                     double *evecs, long long ldv) {
  edgpu_ctx *c = m->ctx;
  Sector *s = get_sector(m, p->storage, nup, ndn);
  *nconv = 0;
  if (s->dim == 0) return EDGPU_OK;
  if (s->dim == 1) {
    CK(cudaMemcpyAsync(evals, s->diag64.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    if (evecs) evecs[0] = 1.0;
    *nconv = 1;
    return EDGPU_OK;
  }
  const int ncv_p = p->ncv > 0 ? p->ncv : 2 * p->nev + 3;
  const int ncv = (int)std::min<long long>(ncv_p, s->dim);
  EigSectorJob J;
  J.s = s;
  J.nev = std::min(p->nev, ncv - 1);
  J.m = ncv;
  J.check = p->multiplicity_check != 1;
  J.check_cycles = p->multiplicity_check >= 2 ? p->multiplicity_check - 1 : 0;
  std::vector<EigSectorJob *> one{&J};
  const double tol = p->tol > 0 ? p->tol : (sizeof(T) == 8 ? 1e-12 : 2e-6);
  J.tol = tol;
  J.maxitr = p->maxitr > 0 ? p->maxitr : 1000;
  J.eval_only = evecs == nullptr;
  solve_batch<T>(m, one);
  if (sizeof(T) == 4) refine_fp32(m, one);
  *nconv = (int)J.evals.size();
  for (int q = 0; q < *nconv; ++q) evals[q] = J.evals[q];
  if (evecs && !J.evecs.empty()) {
    DBuf d(c->alloc, sizeof(double) * s->dim);
    for (int q = 0; q < *nconv; ++q) {
      const T *src = J.evecs[0]->as<T>() + (size_t)q * s->dim;
      if (sizeof(T) == 8) {
        CK(cudaMemcpyAsync(evecs + (size_t)q * ldv, src, sizeof(double) * s->dim, cudaMemcpyDeviceToHost, c->stream));
      } else {
        launch_to_double<float>((const float *)src, d.as<double>(), s->dim, c->stream);
        CK(cudaMemcpyAsync(evecs + (size_t)q * ldv, d.p, sizeof(double) * s->dim, cudaMemcpyDeviceToHost, c->stream));
      }
      sync(c);
    }
  }
  return J.info;
}

int diag_sector_dispatch(edgpu_model *m, const edgpu_diag_params *p, int nup, int ndn, double *evals, int *nconv,
                         double *evecs, long long ldv) {
  if (p->nev < 1) throw ApiError(EDGPU_ERR_ARG, "arpack.NEV must be positive");
  if (p->precision == EDGPU_FP32) return diag_sector_impl<float>(m, p, nup, ndn, evals, nconv, evecs, ldv);
  return diag_sector_impl<double>(m, p, nup, ndn, evals, nconv, evecs, ldv);
}

// SzSymmetry's sector order (SzSymmetry.h:51-54, 72-98): the same comparator through std::sort.
int sector_order(const edgpu_model *m, const int *list, int n_in, int *out) {
  struct Sec {
    int up, dn;
    size_t size;
  };
  std::vector<Sec> v;
  const int ns = m->ns;
  if (list) {
    for (int i = 0; i < n_in; ++i) {
      int a = list[2 * i], b = list[2 * i + 1];
      if (a < 0 || b < 0 || a > ns || b > ns) throw ApiError(EDGPU_ERR_ARG, "sector out of range");
      v.push_back({a, b, (size_t)(binom_at_host(ns, a) * binom_at_host(ns, b))});
    }
  } else {
    for (int i = 0; i <= ns; ++i)
      for (int j = 0; j <= ns; ++j) v.push_back({i, j, (size_t)(binom_at_host(ns, i) * binom_at_host(ns, j))});
  }
  std::sort(v.begin(), v.end(), [](const Sec &a, const Sec &b) {
    return a.size < b.size || (a.size == b.size && a.up < b.up && a.dn < b.dn) ||
           (a.size == b.size && a.up == b.up && a.dn < b.dn);
  });
  for (size_t i = 0; i < v.size(); ++i) {
    out[2 * i] = v[i].up;
    out[2 * i + 1] = v[i].dn;
  }
  return (int)v.size();
}

int diag_dispatch(edgpu_model *m, const edgpu_diag_params *p, int *npairs) {
  if (p->precision == EDGPU_MIXED) return diag_many_mixed(&m, 1, p, npairs);
  if (p->precision == EDGPU_FP32) return diag_impl<float>(m, p, npairs);
  return diag_impl<double>(m, p, npairs);
}

int diag_many_dispatch(edgpu_model *const *ms, int count, const edgpu_diag_params *p, int *npairs) {
  if (p->precision == EDGPU_MIXED) return diag_many_mixed(ms, count, p, npairs);
  if (p->precision == EDGPU_FP32) return diag_many_impl<float>(ms, count, p, npairs);
  return diag_many_impl<double>(ms, count, p, npairs);
}

template MvShape mv_shape<float>(const Sector &);
template MvShape mv_shape<double>(const Sector &);

template void apply_h<float>(edgpu_model *, Sector *, const float *, float *, const float *, double);
template void apply_h<double>(edgpu_model *, Sector *, const double *, double *, const double *, double);

}  // namespace host
}  // namespace edgpu

// ============================================================================ serving
// A request loop with continuous batching: every admitted request's sectors join one running lock-step
// eigen-solver batch between restart cycles (EigBatch::add), leave it when they converge, and a request's
// Green's function runs as soon as its spectrum is complete.  Admission is FIFO by device-memory footprint.
namespace edgpu {
namespace host {

struct ServerRequest {
  long long ticket = 0;
  edgpu_model *m = nullptr;
  edgpu_diag_params dp{};
  std::vector<int> sectors;
  bool gf = false;
  edgpu_gf_params gp{};
  std::vector<int> orbs;
  double *G = nullptr, *Gij = nullptr, *Z = nullptr;
  std::vector<DiagSlot> slots;
  std::vector<std::unique_ptr<EigSectorJob>> jobs;
  int pending = 0;
  int state = 0;  // 0 queued, 1 running, 2 done, < 0 failed (edgpu status)
  int npairs = 0;
  size_t bytes = 0;
};

}  // namespace host
}  // namespace edgpu

struct edgpu_server {
  edgpu_ctx *ctx = nullptr;
  int prec = EDGPU_FP32;
  size_t budget = 0, in_use = 0;
  long long next = 0;
  std::deque<edgpu::host::ServerRequest *> queue;
  std::map<long long, std::unique_ptr<edgpu::host::ServerRequest>> reqs;
  std::map<const edgpu::host::EigSectorJob *, edgpu::host::ServerRequest *> job_req;
  std::unique_ptr<edgpu::host::EigBatch<float>> b32;
  std::unique_ptr<edgpu::host::EigBatch<double>> b64;
  int running = 0;
};

namespace edgpu {
namespace host {

static const int kServerLd = 65;  // projected-matrix dimension of the served batch (ncv <= 64)

edgpu_server *server_create(edgpu_ctx *c, int prec, size_t budget) {
  std::unique_ptr<edgpu_server> s(new edgpu_server());
  s->ctx = c;
  s->prec = prec == EDGPU_FP64 || prec == EDGPU_MIXED ? prec : EDGPU_FP32;
  if (!budget) {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    budget = fr / 10 * 8;
  }
  s->budget = budget;
  if (s->prec != EDGPU_FP64) s->b32.reset(new EigBatch<float>(nullptr, kServerLd, c));
  if (s->prec != EDGPU_FP32) s->b64.reset(new EigBatch<double>(nullptr, kServerLd, c));
  return s.release();
}

// eigen-solver footprint of a request (bases, restart copies, residuals), from the sector dimensions
static size_t request_bytes(const edgpu_model *m, const edgpu_diag_params *p, int prec) {
  const size_t el = prec == EDGPU_FP64 ? 8 : 4;
  const int ncv_p = p->ncv > 0 ? p->ncv : 2 * p->nev + 3;
  auto one = [&](int nup, int ndn) -> size_t {
    const long long d = binom_at_host(m->ns, nup) * binom_at_host(m->ns, ndn);
    if (d <= 1) return 0;
    const long long ncv = std::min<long long>(ncv_p, d);
    return el * (size_t)(2 * (ncv + 1) + 1) * (size_t)d;
  };
  size_t b = 0;
  if (p->sectors && p->n_sectors > 0) {
    for (int q = 0; q < p->n_sectors; ++q) b += one(p->sectors[2 * q], p->sectors[2 * q + 1]);
  } else {
    for (int nup = 0; nup <= m->ns; ++nup)
      for (int ndn = 0; ndn <= m->ns; ++ndn) b += one(nup, ndn);
  }
  return b;
}

long long server_submit(edgpu_server *s, edgpu_model *m, const edgpu_diag_params *dp, const edgpu_gf_params *gp,
                        double *G, double *Gij, double *Z) {
  if (m->ctx != s->ctx) throw ApiError(EDGPU_ERR_ARG, "the model belongs to another context");
  if (dp->nev < 1) throw ApiError(EDGPU_ERR_ARG, "arpack.NEV must be positive");
  const int ncv = dp->ncv > 0 ? dp->ncv : 2 * dp->nev + 3;
  if (ncv > kServerLd - 1) throw ApiError(EDGPU_ERR_ARG, "ncv above 64 is not supported");
  std::unique_ptr<ServerRequest> r(new ServerRequest());
  r->ticket = s->next++;
  r->m = m;
  r->dp = *dp;
  r->dp.precision = s->prec;
  if (dp->sectors && dp->n_sectors > 0) {
    r->sectors.assign(dp->sectors, dp->sectors + 2 * dp->n_sectors);
    r->dp.sectors = r->sectors.data();
  } else {
    r->dp.sectors = nullptr;
    r->dp.n_sectors = 0;
  }
  if (gp) {
    r->gf = true;
    r->gp = *gp;
    r->gp.precision = s->prec;
    if (gp->orbitals && gp->n_orbitals > 0) {
      r->orbs.assign(gp->orbitals, gp->orbitals + 2 * gp->n_orbitals);
      r->gp.orbitals = r->orbs.data();
    } else {
      r->gp.orbitals = nullptr;
      r->gp.n_orbitals = 0;
    }
  }
  r->G = G;
  r->Gij = Gij;
  r->Z = Z;
  r->bytes = request_bytes(m, &r->dp, s->prec);
  const long long t = r->ticket;
  s->queue.push_back(r.get());
  s->reqs[t] = std::move(r);
  return t;
}

static bool same_gf(const edgpu_gf_params &a, const std::vector<int> &oa, const edgpu_gf_params &b,
                    const std::vector<int> &ob) {
  return a.beta == b.beta && a.nomega == b.nomega && a.nlanc == b.nlanc && a.cutoff == b.cutoff && oa == ob;
}

// One scheduling round of the request loop.  EDGPU_FP32 / EDGPU_FP64 servers run one lock-step batch of that
// precision; an EDGPU_MIXED server routes each sector as Hamiltonian::diag does in that precision (sectors
// asking for more than 32 pairs to its FP64 batch, the rest to its FP32 batch with the FP64 Rayleigh-Ritz
// step), so a request's eigen-pairs are the same as the solve alone in that precision.
static void server_step_any(edgpu_server *s) {
  std::vector<ServerRequest *> ready;
  // admission: FIFO while the footprint fits (always at least one request when nothing runs)
  while (!s->queue.empty()) {
    ServerRequest *r = s->queue.front();
    if (s->running > 0 && s->in_use + r->bytes > s->budget) break;
    s->queue.pop_front();
    try {
      if (s->prec == EDGPU_FP32) diag_prepare<float>(r->m, &r->dp, r->slots, r->jobs);
      else diag_prepare<double>(r->m, &r->dp, r->slots, r->jobs);
    } catch (ApiError &e) {
      r->state = e.code;
      continue;
    }
    r->state = 1;
    s->running += 1;
    s->in_use += r->bytes;
    std::vector<EigSectorJob *> j32, j64;
    for (auto &J : r->jobs) {
      s->job_req[J.get()] = r;
      if (s->prec == EDGPU_FP32) {
        j32.push_back(J.get());
      } else if (s->prec == EDGPU_FP64 || mixed_in_fp64(*J)) {
        if (s->prec == EDGPU_MIXED) J->prec = EDGPU_FP64;
        j64.push_back(J.get());
      } else {
        J->prec = EDGPU_FP32;
        J->tol = r->dp.tol > 0 ? r->dp.tol : 2e-6;
        j32.push_back(J.get());
      }
    }
    r->pending = (int)(j32.size() + j64.size());
    if (!j32.empty()) s->b32->add(j32);
    if (!j64.empty()) s->b64->add(j64);
    if (r->pending == 0) ready.push_back(r);
  }
  // one restart cycle of every admitted sector
  std::vector<EigSectorJob *> finished, f32;
  if (s->b32 && s->b32->active()) s->b32->cycle(f32);
  if (s->b64 && s->b64->active()) s->b64->cycle(finished);
  if (!f32.empty()) refine_fp32(f32[0]->owner, f32);
  finished.insert(finished.end(), f32.begin(), f32.end());
  for (auto *J : finished) {
    auto it = s->job_req.find(J);
    if (it == s->job_req.end()) continue;
    ServerRequest *r = it->second;
    s->job_req.erase(it);
    if (--r->pending == 0) ready.push_back(r);
  }
  // spectra complete: eigen-pairs, then the Green's functions of requests sharing parameters together
  std::vector<ServerRequest *> gfq;
  for (auto *r : ready) {
    const int w = s->prec == EDGPU_FP32 ? diag_finish<float>(r->m, r->slots, &r->npairs)
                                        : diag_finish<double>(r->m, r->slots, &r->npairs);
    (void)w;
    if (r->gf) gfq.push_back(r);
    else r->state = 2;
  }
  while (!gfq.empty()) {
    std::vector<ServerRequest *> grp, rest;
    for (auto *r : gfq) {
      if (grp.empty() || same_gf(grp[0]->gp, grp[0]->orbs, r->gp, r->orbs)) grp.push_back(r);
      else rest.push_back(r);
    }
    std::vector<edgpu_model *> ms;
    std::vector<double *> G, Gij;
    std::vector<double> Z(grp.size(), 0.0);
    for (auto *r : grp) {
      ms.push_back(r->m);
      G.push_back(r->G);
      Gij.push_back(r->Gij);
    }
    int rc = gf_many_dispatch(ms.data(), (int)ms.size(), &grp[0]->gp, 0, 0, nullptr, G.data(), Gij.data(), Z.data());
    for (size_t q = 0; q < grp.size(); ++q) {
      if (grp[q]->Z) *grp[q]->Z = Z[q];
      grp[q]->state = rc < 0 ? rc : 2;
    }
    gfq.swap(rest);
  }
  for (auto *r : ready) {
    s->running -= 1;
    s->in_use -= std::min(s->in_use, r->bytes);
    r->jobs.clear();
    r->slots.clear();
  }
}

void server_step(edgpu_server *s, int *running, int *queued) {
  server_step_any(s);
  if (running) *running = s->running;
  if (queued) *queued = (int)s->queue.size();
}

int server_poll(edgpu_server *s, long long ticket, int *npairs) {
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) throw ApiError(EDGPU_ERR_ARG, "unknown ticket");
  if (npairs) *npairs = it->second->npairs;
  return it->second->state;
}

void server_destroy(edgpu_server *s) { delete s; }

}  // namespace host
}  // namespace edgpu

namespace edgpu {
namespace host {
edgpu_ctx *server_ctx(edgpu_server *s) { return s->ctx; }
}  // namespace host
}  // namespace edgpu
