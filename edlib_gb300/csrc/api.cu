// The extern "C" entry points of include/edgpu.h.  Each one validates its arguments, runs inside the
// context's error guard (no exception crosses the ABI) and forwards to the host driver.
#include "model_internal.h"

using namespace edgpu;
using namespace edgpu::host;

namespace {

Transition hop(int a, int b, double v, int sf, int spin) {
  Transition t{};
  t.quad = 0;
  t.a = a;
  t.b = b;
  t.value = v;
  t.sign_factor = sf;
  t.spin = spin;
  return t;
}

template <typename T>
void download(edgpu_ctx *c, T *dst, const void *src, size_t n) {
  CK(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToHost, c->stream));
  sync(c);
}

template <typename T>
int av_impl(edgpu_model *m, const double *v, double *w, long long n, int clear) {
  edgpu_ctx *c = m->ctx;
  Sector *s = m->cur;
  if (!s) throw ApiError(EDGPU_ERR_STATE, "fill() has not been called");
  if (n != s->dim) throw ApiError(EDGPU_ERR_ARG, "vector length does not match the filled sector");
  DBuf dv(c->alloc, sizeof(double) * n), dw(c->alloc, sizeof(double) * n);
  CK(cudaMemcpyAsync(dv.p, v, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  if (!clear) CK(cudaMemcpyAsync(dw.p, w, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  if (sizeof(T) == 8) {
    DBuf y(c->alloc, sizeof(double) * n);
    apply_h<double>(m, s, dv.as<double>(), y.as<double>(), clear ? nullptr : dw.as<double>(), 1.0);
    download(c, w, y.p, n);
  } else {
    DBuf x32(c->alloc, sizeof(float) * n), z32(c->alloc, sizeof(float) * n), y32(c->alloc, sizeof(float) * n),
        y64(c->alloc, sizeof(double) * n);
    launch_convert<float>(dv.as<double>(), x32.as<float>(), n, c->stream);
    if (!clear) launch_convert<float>(dw.as<double>(), z32.as<float>(), n, c->stream);
    apply_h<float>(m, s, x32.as<float>(), y32.as<float>(), clear ? nullptr : z32.as<float>(), 1.0);
    launch_to_double<float>(y32.as<float>(), y64.as<double>(), n, c->stream);
    download(c, w, y64.p, n);
  }
  return EDGPU_OK;
}

}  // namespace

extern "C" {

int edgpu_ctx_create(edgpu_ctx **out, int device, size_t hbm_budget) {
  if (!out) return EDGPU_ERR_ARG;
  *out = nullptr;
  edgpu_ctx *c = new (std::nothrow) edgpu_ctx();
  if (!c) return EDGPU_ERR_CAPACITY;
  int rc = guard(c, [&]() {
    CK(cudaSetDevice(device));
    c->device = device;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->alloc.budget = hbm_budget;
    return EDGPU_OK;
  });
  if (rc) {
    delete c;
    return rc;
  }
  *out = c;
  return EDGPU_OK;
}

int edgpu_ctx_destroy(edgpu_ctx *c) {
  if (!c) return EDGPU_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->alloc.release_all();
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return EDGPU_OK;
}

const char *edgpu_last_error(const edgpu_ctx *c) { return c ? c->err.c_str() : "null context"; }

size_t edgpu_ctx_device_bytes(const edgpu_ctx *c) { return c ? c->alloc.held() : 0; }

void *edgpu_ctx_stream(const edgpu_ctx *c) { return c ? (void *)c->stream : nullptr; }

int edgpu_model_hubbard(edgpu_ctx *c, int ns, const double *t, const double *U, const double *xmu, const double *hmag,
                        const double *J, edgpu_model **out) {
  if (!c || !out || !t || !U || !xmu) return EDGPU_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<edgpu_model> m(new edgpu_model());
  int rc = guard(c, [&]() {
    if (ns < 1 || ns > kMaxNs) throw ApiError(EDGPU_ERR_ARG, "NSITES must be in [1, 20]");
    m->ctx = c;
    m->kind = 0;
    m->ns = ns;
    m->U.assign(U, U + ns);
    m->xmu.assign(xmu, xmu + ns);
    m->hmag.assign(ns, 0.0);
    if (hmag) m->hmag.assign(hmag, hmag + ns);
    if (J) m->J.assign(J, J + (size_t)ns * ns);
    for (int k = 0; k < ns * ns; ++k)
      if (!std::isfinite(t[k])) throw ApiError(EDGPU_ERR_ARG, "non-finite hopping");
    m->t.assign(t, t + (size_t)ns * ns);
    for (int ii = 0; ii < ns; ++ii)
      for (int jj = 0; jj < ns; ++jj) {
        double v = t[(size_t)ii * ns + jj];
        if (std::fabs(v) > 1e-10)
          for (int is = 0; is < 2; ++is) m->T.push_back(hop(ii + is * ns, jj + is * ns, v, -1, is));
      }
    finish_model(m.get());
    return EDGPU_OK;
  });
  if (rc) return rc;
  *out = m.release();
  return EDGPU_OK;
}

int edgpu_model_siam(edgpu_ctx *c, int ns, int ml, const double *epsk, const double *vk, const double *h0, double mu,
                     const double *U, edgpu_model **out) {
  if (!c || !out || !epsk || !vk || !h0 || !U) return EDGPU_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<edgpu_model> m(new edgpu_model());
  int rc = guard(c, [&]() {
    if (ml > ns) throw ApiError(EDGPU_ERR_ARG, "Incorrect values for the total number of sites and the number of orbitals. Please check input file.");
    if (ns < 1 || ns > kMaxNs || ml < 1) throw ApiError(EDGPU_ERR_ARG, "NSITES must be in [1, 20], NORBITALS >= 1");
    m->ctx = c;
    m->kind = 1;
    m->ns = ns;
    m->ml = ml;
    m->mu = mu;
    const int nk = ns - ml;
    m->epsk.assign(epsk, epsk + (size_t)nk * 2);
    m->vk.assign(vk, vk + (size_t)ml * nk * 2);
    m->h0.assign(h0, h0 + (size_t)ml * ml * 2);
    const size_t m4 = (size_t)ml * ml * ml * ml;
    m->Ut.assign(U, U + 4 * m4);
    // SingleImpurityAndersonModel.h:232-254
    for (int im = 0; im < ml; ++im)
      for (int jm = 0; jm < im; ++jm)
        for (int is = 0; is < 2; ++is) {
          double h = m->h0[((size_t)im * ml + jm) * 2 + is];
          if (std::fabs(h) > 1e-10) {
            m->T.push_back(hop(im + is * ns, jm + is * ns, h, 1, is));
            m->T.push_back(hop(jm + is * ns, im + is * ns, h, 1, is));
          }
        }
    for (int im = 0; im < ml; ++im)
      for (int ik = 0; ik < nk; ++ik)
        for (int is = 0; is < 2; ++is) {
          double v = m->vk[((size_t)im * nk + ik) * 2 + is];
          if (std::fabs(v) > 1e-10) {
            m->T.push_back(hop(im + is * ns, ik + ml + is * ns, v, 1, is));
            m->T.push_back(hop(ik + ml + is * ns, im + is * ns, v, 1, is));
          }
        }
    // SingleImpurityAndersonModel.h:256-274
    auto Ut = [&](int s1, int s2, int i, int j, int k, int l) {
      return m->Ut[((((size_t)(s1 * 2 + s2) * ml + i) * ml + j) * ml + k) * ml + l];
    };
    for (int s1 = 0; s1 < 2; ++s1)
      for (int s2 = 0; s2 < 2; ++s2)
        for (int i = 0; i < ml; ++i)
          for (int j = 0; j < ml; ++j)
            for (int k = 0; k < ml; ++k)
              for (int l = 0; l < ml; ++l) {
                if (((i == l) && (j == k) && (s1 == s2)) || ((i == k) && (j == l))) continue;
                double u = Ut(s1, s2, i, j, k, l);
                if (std::fabs(u) != 0.0) {
                  Transition t{};
                  t.quad = 1;
                  t.k = k + s1 * ns;
                  t.l = l + s2 * ns;
                  t.j = j + s2 * ns;
                  t.i = i + s1 * ns;
                  t.value = 0.5 * u;
                  t.sign_factor = 1;
                  t.spin = -1;
                  m->V.push_back(t);
                }
              }
    finish_model(m.get());
    return EDGPU_OK;
  });
  if (rc) return rc;
  *out = m.release();
  return EDGPU_OK;
}

int edgpu_model_destroy(edgpu_model *m) {
  if (!m) return EDGPU_ERR_ARG;
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
  return EDGPU_OK;
}

int edgpu_model_transitions(const edgpu_model *m, int which) {
  if (!m) return EDGPU_ERR_ARG;
  return which == 0 ? (int)m->T.size() : (int)m->V.size();
}

int edgpu_model_set_limits(edgpu_model *m, size_t max_dim, size_t max_size) {
  if (!m) return EDGPU_ERR_ARG;
  m->max_dim = max_dim;
  m->max_size = max_size;
  return EDGPU_OK;
}

long long edgpu_binom(const edgpu_model *m, int n, int k) { return m ? binom_at_host(n, k) : -1; }

int edgpu_basis(edgpu_model *m, int k, int *out) {
  if (!m || !out || k < 0 || k > m->ns) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    download<int>(m->ctx, out, m->dbasis.as<int>() + m->basis_off[k], (size_t)binom_at_host(m->ns, k));
    return EDGPU_OK;
  });
}

int edgpu_ninv(edgpu_model *m, int k, int *out) {
  if (!m || !out || k < 0 || k > m->ns) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    download<int>(m->ctx, out, m->dninv.as<int>() + ((size_t)k << m->ns), (size_t)1 << m->ns);
    return EDGPU_OK;
  });
}

int edgpu_sector_order(const edgpu_model *m, const int *list, int n_in, int *out, int *n_out) {
  if (!m || !out) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    int n = sector_order(m, list, n_in, out);
    if (n_out) *n_out = n;
    return EDGPU_OK;
  });
}

int edgpu_fill(edgpu_model *m, int storage, int nup, int ndn, long long *dim) {
  if (!m) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    m->cur = get_sector(m, storage, nup, ndn);
    if (dim) *dim = m->cur->dim;
    return EDGPU_OK;
  });
}

int edgpu_av(edgpu_model *m, const double *v, double *w, long long n, int clear, int prec) {
  if (!m || !v || !w) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    return prec == EDGPU_FP32 ? av_impl<float>(m, v, w, n, clear) : av_impl<double>(m, v, w, n, clear);
  });
}

int edgpu_spmv(edgpu_model *m, int storage, int nup, int ndn, const void *x, void *y, int nvec, long long ldx, int prec,
               int accumulate, void *stream) {
  if (!m || !x || !y || nvec < 1) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    Sector *s = get_sector(m, storage, nup, ndn);  // builds the sector's tables on the context's stream, synchronised
    if (ldx < s->dim) throw ApiError(EDGPU_ERR_ARG, "ldx is below the sector dimension");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto run = [&](auto tag) {
      using T = decltype(tag);
      if (((uintptr_t)x | (uintptr_t)y) % sizeof(T)) throw ApiError(EDGPU_ERR_ARG, "vectors are not aligned to their type");
      std::vector<MvTask<T>> tasks(nvec);
      std::vector<int> map;
      for (int q = 0; q < nvec; ++q) {
        MvTask<T> &t = tasks[q];
        t.op = s->dop<T>();
        t.srs_rows = s->srs_rows;
        t.item_begin = (int)map.size();
        t.x = static_cast<const T *>(x) + (size_t)q * ldx;
        t.y = static_cast<T *>(y) + (size_t)q * ldx;
        t.z = accumulate ? t.y : nullptr;  // w += H v: every element reads its own y before it writes it
        t.c = accumulate ? 1.0 : 0.0;
        t.dot_partial = nullptr;
        for (int it = 0; it < s->nitems; ++it) map.push_back(q);
      }
      // the task list lives in stream-ordered memory, released on the caller's stream after the launch
      const size_t tb = sizeof(MvTask<T>) * tasks.size(), mb = sizeof(int) * map.size();
      void *buf = nullptr;
      CK(cudaMallocAsync(&buf, tb + mb + 16, st));
      char *dt = static_cast<char *>(buf), *dm = dt + ((tb + 15) & ~size_t(15));
      CK(cudaMemcpyAsync(dt, tasks.data(), tb, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(dm, map.data(), mb, cudaMemcpyHostToDevice, st));
      MvShape sh = mv_shape<T>(*s);
      sh.plain = accumulate ? 0 : 1;
      const OpTuning &tu = m->op_tune[sizeof(T) == 4 ? 1 : 0];
      if (tu.done && tu.ms > 0 && !getenv("EDGPU_SRS_STAGE_KB")) sh.staged = tu.staged;
      launch_mv<T>(reinterpret_cast<const MvTask<T> *>(dt), reinterpret_cast<const int *>(dm), (int)map.size(), sh, st);
      CK(cudaGetLastError());
      CK(cudaFreeAsync(buf, st));
    };
    if (prec == EDGPU_FP32) run(float());
    else run(double());
    return EDGPU_OK;
  });
}

int edgpu_a_adag(edgpu_model *m, int spin_orbital, int nup, int ndn, int tnup, int tndn, const double *in, double *out,
                 int annihilate) {
  if (!m || !in || !out) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    if (spin_orbital < 0 || spin_orbital >= 2 * m->ns) throw ApiError(EDGPU_ERR_ARG, "spin-orbital out of range");
    Sector *s = get_sector(m, m->cur ? m->cur->storage : kCRS, nup, ndn);
    Sector *t = get_sector(m, s->storage, tnup, tndn);
    DBuf din(c->alloc, sizeof(double) * s->dim), dout(c->alloc, sizeof(double) * t->dim);
    CK(cudaMemcpyAsync(din.p, in, sizeof(double) * s->dim, cudaMemcpyHostToDevice, c->stream));
    launch_a_adag<double>(s->op64, t->op64, spin_orbital, annihilate, din.as<double>(), dout.as<double>(), 0, c->stream);
    download(c, out, dout.p, (size_t)t->dim);
    return EDGPU_OK;
  });
}

int edgpu_vv(edgpu_model *m, const double *v, const double *w, long long n, double *out) {
  if (!m || !v || !w || !out || n < 0) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    DBuf dv(c->alloc, sizeof(double) * (n + 1)), dw(c->alloc, sizeof(double) * (n + 1)), part(c->alloc, sizeof(double) * 64),
        r(c->alloc, sizeof(double));
    CK(cudaMemcpyAsync(dv.p, v, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dw.p, w, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    launch_dot_partials<double>(dv.as<double>(), dw.as<double>(), n, part.as<double>(), 64, c->stream);
    launch_reduce(part.as<double>(), 64, r.as<double>(), c->stream);
    download(c, out, r.p, 1);
    return EDGPU_OK;
  });
}

int edgpu_diag(edgpu_model *m, const edgpu_diag_params *p, int *npairs) {
  if (!m || !p) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return diag_dispatch(m, p, npairs); });
}

int edgpu_diag_many(edgpu_model *const *models, int count, const edgpu_diag_params *p, int *npairs) {
  if (!models || count < 1 || !models[0] || !p) return EDGPU_ERR_ARG;
  return guard(models[0]->ctx, [&]() { return diag_many_dispatch(models, count, p, npairs); });
}

int edgpu_greens_function_many(edgpu_model *const *models, int count, const edgpu_gf_params *p, double *const *G,
                               double *const *G_ij, double *Z) {
  if (!models || count < 1 || !models[0] || !p) return EDGPU_ERR_ARG;
  return guard(models[0]->ctx, [&]() { return gf_many_dispatch(models, count, p, 0, 0, nullptr, G, G_ij, Z); });
}

int edgpu_chiloc_many(edgpu_model *const *models, int count, const edgpu_gf_params *p, int op, const double *avg,
                      double *const *chi, double *const *chi_ij, double *Z) {
  if (!models || count < 1 || !models[0] || !p || !avg) return EDGPU_ERR_ARG;
  return guard(models[0]->ctx, [&]() { return gf_many_dispatch(models, count, p, 1, op, avg, chi, chi_ij, Z); });
}

int edgpu_diag_sector(edgpu_model *m, const edgpu_diag_params *p, int nup, int ndn, double *evals, int *nconv,
                      double *evecs, long long ldv) {
  if (!m || !p || !evals || !nconv) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return diag_sector_dispatch(m, p, nup, ndn, evals, nconv, evecs, ldv); });
}

int edgpu_eigenpairs(const edgpu_model *m, double *evals, int *sectors, int *ids, int max_pairs) {
  if (!m) return EDGPU_ERR_ARG;
  if (!m->have_pairs) return EDGPU_ERR_STATE;
  int n = std::min<int>(max_pairs, (int)m->pairs.size());
  for (int q = 0; q < n; ++q) {
    if (evals) evals[q] = m->pairs[q].E;
    if (sectors) { sectors[2 * q] = m->pairs[q].nup; sectors[2 * q + 1] = m->pairs[q].ndn; }
    if (ids) ids[q] = m->pairs[q].id;
  }
  return EDGPU_OK;
}

int edgpu_eigenvector(edgpu_model *m, int index, double *out, long long n) {
  if (!m || !out) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    if (!m->have_pairs || index < 0 || index >= (int)m->pairs.size()) throw ApiError(EDGPU_ERR_ARG, "no such eigen-pair");
    const Pair &p = m->pairs[index];
    if (m->evals_only || !p.block) throw ApiError(EDGPU_ERR_STATE, "eigenvectors were not kept (EIGENVALUES_ONLY)");
    if (n != p.n) throw ApiError(EDGPU_ERR_ARG, "wrong eigenvector length");
    edgpu_ctx *c = m->ctx;
    if (p.prec == EDGPU_FP64) {
      download(c, out, p.vec<double>(), (size_t)n);
    } else {
      DBuf d(c->alloc, sizeof(double) * n);
      launch_to_double<float>(p.vec<float>(), d.as<double>(), n, c->stream);
      download(c, out, d.p, (size_t)n);
    }
    return EDGPU_OK;
  });
}

int edgpu_greens_function(edgpu_model *m, const edgpu_gf_params *p, double *G, double *G_ij, double *Z) {
  if (!m || !p) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return gf_dispatch(m, p, G, G_ij, Z); });
}

int edgpu_greens_function_weighted(edgpu_model *m, const edgpu_gf_params *p, const double *weights, int nrows,
                                   double *G, double *Z) {
  if (!m || !p || !weights || nrows < 1) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return gf_weighted_dispatch(m, p, weights, nrows, G, Z); });
}

int edgpu_self_energy(edgpu_model *m, const edgpu_gf_params *p, const double *G_ij, double *G0, double *Sigma) {
  if (!m || !p || !G_ij) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return self_energy_dispatch(m, p, G_ij, G0, Sigma); });
}

int edgpu_operator_tuning(const edgpu_model *m, int prec, int *blocks_per_sm, int *staged, double *ms) {
  if (!m || (prec != EDGPU_FP32 && prec != EDGPU_FP64)) return EDGPU_ERR_ARG;
  const edgpu::OpTuning &tu = m->op_tune[prec == EDGPU_FP32 ? 1 : 0];
  if (blocks_per_sm) *blocks_per_sm = tu.mb;
  if (staged) *staged = tu.staged;
  if (ms) *ms = tu.done ? tu.ms : -1.0;
  return EDGPU_OK;
}

int edgpu_chiloc(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chi_ij, double *Z) {
  if (!m || !p) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return chi_dispatch(m, p, op, avg, chi, chi_ij, Z); });
}

int edgpu_refine_eigenpairs(edgpu_model *const *models, int count, double beta, double cutoff) {
  if (!models || count < 1 || !models[0] || !(beta > 0) || !(cutoff >= 0)) return EDGPU_ERR_ARG;
  for (int q = 0; q < count; ++q)
    if (!models[q] || models[q]->ctx != models[0]->ctx) return EDGPU_ERR_ARG;
  return guard(models[0]->ctx, [&]() { return refine_kept(models, count, beta, cutoff); });
}

int edgpu_static_observables(edgpu_model *m, double beta, double cutoff, double *n, double *n_up, double *n_dn,
                             double *mag, double *d_occ, double *mimj, double *n_eff, double *energy) {
  if (!m) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() { return static_obs(m, beta, cutoff, n, n_up, n_dn, mag, d_occ, mimj, n_eff, energy); });
}

int edgpu_lanczos(edgpu_model *m, int storage, int nup, int ndn, const double *starts, int count, int nlanc, int prec,
                  double *alpha, double *beta, int *nl) {
  if (!m || !starts || count < 0 || nlanc < 1) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    Sector *s = get_sector(m, storage, nup, ndn);
    const long long n = s->dim;
    DBuf d64(c->alloc, sizeof(double) * n * std::max(count, 1));
    CK(cudaMemcpyAsync(d64.p, starts, sizeof(double) * n * count, cudaMemcpyHostToDevice, c->stream));
    std::vector<DBuf> a, b, st;
    std::vector<Sector *> secs(count, s);
    if (prec == EDGPU_FP32) {
      DBuf d32(c->alloc, sizeof(float) * n * std::max(count, 1));
      launch_convert<float>(d64.as<double>(), d32.as<float>(), n * count, c->stream);
      std::vector<float *> ptr;
      for (int q = 0; q < count; ++q) ptr.push_back(d32.as<float>() + q * n);
      lanczos_batch<float>(m, secs, ptr, nlanc, a, b, st);
    } else {
      std::vector<double *> ptr;
      for (int q = 0; q < count; ++q) ptr.push_back(d64.as<double>() + q * n);
      lanczos_batch<double>(m, secs, ptr, nlanc, a, b, st);
    }
    for (int q = 0; q < count; ++q) {
      if (alpha) download(c, alpha + (size_t)q * nlanc, a[q].p, (size_t)nlanc);
      if (beta) download(c, beta + (size_t)q * (nlanc + 1), b[q].p, (size_t)(nlanc + 1));
      int sh[2];
      download(c, sh, st[q].p, 2);
      if (nl) nl[q] = sh[1];
    }
    return EDGPU_OK;
  });
}

__global__ void k_frac_explicit(const double *alpha, const double *beta, int nlanc, int isign, double scale,
                                const double *ener, int nz, double *out) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nz) return;
  double2 r = frac_point(alpha, beta, nlanc, isign, scale, make_double2(ener[2 * p], ener[2 * p + 1]));
  out[2 * p] = r.x;
  out[2 * p + 1] = r.y;
}

int edgpu_frac_points(edgpu_ctx *c, const double *alpha, const double *beta, int nlanc, int isign, double expectation,
                      double expb, const double *ener, int nz, double *out) {
  if (!c || !alpha || !beta || !ener || !out || nlanc < 1 || nz < 0) return EDGPU_ERR_ARG;
  return guard(c, [&]() {
    DBuf da(c->alloc, sizeof(double) * nlanc), db(c->alloc, sizeof(double) * (nlanc + 1)),
        de(c->alloc, sizeof(double) * 2 * std::max(nz, 1)), dout(c->alloc, sizeof(double) * 2 * std::max(nz, 1));
    CK(cudaMemcpyAsync(da.p, alpha, sizeof(double) * nlanc, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(db.p, beta, sizeof(double) * (nlanc + 1), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(de.p, ener, sizeof(double) * 2 * nz, cudaMemcpyHostToDevice, c->stream));
    if (nz) {
      k_frac_explicit<<<(nz + 127) / 128, 128, 0, c->stream>>>(da.as<double>(), db.as<double>(), nlanc, isign,
                                                                   expectation * expb, de.as<double>(), nz, dout.as<double>()); note_launch();
    }
    CK(cudaGetLastError());
    download(c, out, dout.p, (size_t)2 * nz);
    return EDGPU_OK;
  });
}

int edgpu_bench_spmv(edgpu_model *m, int storage, int nup, int ndn, int nvec, int prec, int reps, double *ms_per_launch,
                     double *bytes_per_launch) {
  if (!m || nvec < 1 || reps < 1) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    Sector *s = get_sector(m, storage, nup, ndn);
    auto run = [&](auto tag) {
      using T = decltype(tag);
      const long long n = s->dim;
      DBuf X(c->alloc, sizeof(T) * n * nvec), Y(c->alloc, sizeof(T) * n * nvec);
      CK(cudaMemsetAsync(X.p, 0, sizeof(T) * n * nvec, c->stream));
      std::vector<MvTask<T>> tasks(nvec);
      std::vector<int> map;
      for (int q = 0; q < nvec; ++q) {
        MvTask<T> &t = tasks[q];
        t.op = s->dop<T>();
        t.srs_rows = s->srs_rows;
        t.item_begin = (int)map.size();
        t.x = X.as<T>() + q * n;
        t.y = Y.as<T>() + q * n;
        t.z = nullptr;
        t.c = 0.0;
        t.dot_partial = nullptr;
        for (int it = 0; it < s->nitems; ++it) map.push_back(q);
      }
      DBuf dt = upload(c, tasks), dm = upload(c, map);
      MvShape smem = mv_shape<T>(*s);
      smem.plain = 1;
      const OpTuning &tu = m->op_tune[sizeof(T) == 4 ? 1 : 0];
      if (tu.done && tu.ms > 0 && !getenv("EDGPU_SRS_STAGE_KB")) smem.staged = tu.staged;
      for (int w = 0; w < 2; ++w) launch_mv<T>(dt.as<MvTask<T>>(), dm.as<int>(), (int)map.size(), smem, c->stream);
      cudaEvent_t e0, e1;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      CK(cudaEventRecord(e0, c->stream));
      for (int r = 0; r < reps; ++r) launch_mv<T>(dt.as<MvTask<T>>(), dm.as<int>(), (int)map.size(), smem, c->stream);
      CK(cudaEventRecord(e1, c->stream));
      sync(c);
      if (take_mv_stall() || take_cgs_stall())
        throw ApiError(EDGPU_ERR_CUDA, "a bulk copy into shared memory did not complete");
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (ms_per_launch) *ms_per_launch = (double)ms / reps;
      // x read and y written per vector; the diagonal once (every vector of the launch shares the sector)
      if (bytes_per_launch) *bytes_per_launch = (2.0 * nvec + 1.0) * (double)n * sizeof(T);
    };
    if (prec == EDGPU_FP32) run(float());
    else run(double());
    return EDGPU_OK;
  });
}

__global__ void k_bench_fill(float *f, double *d, long long n, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long h = (i + 1) * 0x9e3779b97f4a7c15ull ^ seed;
    h ^= h >> 31;
    h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 29;
    const double v = ((double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5) * 1e-3;
    if (f) f[i] = (float)v;
    if (d) d[i] = v;
  }
}

int edgpu_bench_spmv_batch(edgpu_model *const *models, int count, int storage, int prec, int reps, double *ms_per_launch,
                           double *bytes_per_launch, long long *states) {
  if (!models || count < 1 || !models[0] || reps < 1) return EDGPU_ERR_ARG;
  for (int q = 0; q < count; ++q)
    if (!models[q] || models[q]->ctx != models[0]->ctx) return EDGPU_ERR_ARG;
  edgpu_model *m0 = models[0];
  return guard(m0->ctx, [&]() {
    edgpu_ctx *c = m0->ctx;
    // every sector of every model with more than one state: one task each, as the eigen step's operator
    std::vector<Sector *> secs;
    for (int q = 0; q < count; ++q) {
      std::vector<int> order(2 * (models[q]->ns + 1) * (models[q]->ns + 1));
      const int nsec = sector_order(models[q], nullptr, 0, order.data());
      for (int k = 0; k < nsec; ++k) {
        Sector *s = get_sector(models[q], storage, order[2 * k], order[2 * k + 1]);
        if (s->dim > 1) secs.push_back(s);
      }
    }
    auto run = [&](auto tag) {
      using T = decltype(tag);
      std::vector<long long> off(secs.size() + 1, 0);
      const long long v = 16 / (long long)sizeof(T);
      for (size_t k = 0; k < secs.size(); ++k) off[k + 1] = off[k] + (secs[k]->dim + v - 1) / v * v;
      const long long tot = off.back();
      DBuf X(c->alloc, sizeof(T) * tot), Y(c->alloc, sizeof(T) * tot);
      k_bench_fill<<<1024, 256, 0, c->stream>>>(sizeof(T) == 4 ? X.as<float>() : nullptr,
                                                sizeof(T) == 8 ? X.as<double>() : nullptr, tot, 3);
      note_launch();
      std::vector<MvTask<T>> tasks(secs.size());
      std::vector<int> map;
      MvShape sh{storage, 0};
      double bytes = 0;
      long long nst = 0;
      for (size_t k = 0; k < secs.size(); ++k) {
        MvTask<T> &t = tasks[k];
        t.op = secs[k]->dop<T>();
        t.srs_rows = secs[k]->srs_rows;
        t.item_begin = (int)map.size();
        t.x = X.as<T>() + off[k];
        t.y = Y.as<T>() + off[k];
        t.z = nullptr;
        t.c = 0.0;
        t.dot_partial = nullptr;
        for (int it = 0; it < secs[k]->nitems; ++it) map.push_back((int)k);
        merge_shape(sh, mv_shape<T>(*secs[k]));
        bytes += 3.0 * (double)secs[k]->dim * sizeof(T);  // x read, y written, the sector's diagonal read
        nst += secs[k]->dim;
      }
      DBuf dt = upload(c, tasks), dm = upload(c, map);
      sh.plain = 1;
      const OpTuning &tu = m0->op_tune[sizeof(T) == 4 ? 1 : 0];  // the variant the eigen step runs
      if (tu.done && tu.ms > 0 && !getenv("EDGPU_SRS_STAGE_KB")) sh.staged = tu.staged;
      for (int w = 0; w < 2; ++w) launch_mv<T>(dt.as<MvTask<T>>(), dm.as<int>(), (int)map.size(), sh, c->stream);
      cudaEvent_t e0, e1;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      CK(cudaEventRecord(e0, c->stream));
      for (int r = 0; r < reps; ++r) launch_mv<T>(dt.as<MvTask<T>>(), dm.as<int>(), (int)map.size(), sh, c->stream);
      CK(cudaEventRecord(e1, c->stream));
      sync(c);
      if (take_mv_stall() || take_cgs_stall())
        throw ApiError(EDGPU_ERR_CUDA, "a bulk copy into shared memory did not complete");
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (ms_per_launch) *ms_per_launch = (double)ms / reps;
      if (bytes_per_launch) *bytes_per_launch = bytes;
      if (states) *states = nst;
    };
    if (prec == EDGPU_FP32) run(float());
    else run(double());
    return EDGPU_OK;
  });
}

int edgpu_bench_cgs(edgpu_model *m, int storage, int nup, int ndn, int nbasis, int ntasks, int prec, int reps,
                    double *ms_dot, double *ms_upd, double *bytes_dot, double *bytes_upd) {
  if (!m || nbasis < 1 || nbasis > 64 || ntasks < 1 || reps < 1) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    edgpu_ctx *c = m->ctx;
    Sector *s = get_sector(m, storage, nup, ndn);
    auto run = [&](auto tag) {
      using T = decltype(tag);
      const long long n = s->dim, ldv = (n + 16 / (long long)sizeof(T) - 1) / (16 / (long long)sizeof(T)) *
                                              (16 / (long long)sizeof(T));
      const int ld = nbasis + 1;
      const int nch = (int)((n + kCgsChunk - 1) / kCgsChunk);
      // ntasks independent bases of the sector: nbasis columns (+1 spare), w, a saved copy of w
      DBuf V(c->alloc, sizeof(T) * (size_t)ntasks * (nbasis + 1) * ldv), W(c->alloc, sizeof(T) * (size_t)ntasks * ldv),
          W0(c->alloc, sizeof(T) * (size_t)ntasks * ldv),
          small(c->alloc, sizeof(double) * (size_t)ntasks *
                              (2 * ld * ld + 2 * (size_t)nch * ld + 3 * nch + 4 + (size_t)cgs_nsup(nch) * (2 * ld + 2) +
                               ld + ld / 2 + 1 + cgs_nsup(nch) / 2 + 1)),
          st(c->alloc, sizeof(int) * 8 * ntasks);
      const long long nv = (long long)ntasks * (nbasis + 1) * ldv;
      k_bench_fill<<<1024, 256, 0, c->stream>>>(sizeof(T) == 4 ? V.as<float>() : nullptr,
                                                sizeof(T) == 8 ? V.as<double>() : nullptr, nv, 1);
      note_launch();
      k_bench_fill<<<1024, 256, 0, c->stream>>>(sizeof(T) == 4 ? W0.as<float>() : nullptr,
                                                sizeof(T) == 8 ? W0.as<double>() : nullptr, (long long)ntasks * ldv, 2);
      note_launch();
      CK(cudaMemsetAsync(small.p, 0, small.bytes, c->stream));
      std::vector<int> st0((size_t)8 * ntasks, 0);
      std::vector<EigTask<T>> tasks(ntasks);
      std::vector<int> cmap, lmap;
      double *ps = small.as<double>();
      for (int q = 0; q < ntasks; ++q) {
        st0[(size_t)8 * q] = nbasis - 1;
        EigTask<T> &t = tasks[q];
        t = EigTask<T>{};
        t.op = s->dop<T>();
        t.chunk_begin = (int)cmap.size();
        t.nchunks = nch;
        t.n = n;
        t.ldv = ldv;
        t.m = nbasis;
        t.ld = ld;
        t.V = V.as<T>() + (size_t)q * (nbasis + 1) * ldv;
        t.w = W.as<T>() + (size_t)q * ldv;
        t.Tm = ps;
        ps += (size_t)ld * ld;
        t.E = ps;
        ps += (size_t)ld * ld;
        t.hpart = ps;
        ps += (size_t)nch * ld;
        t.hpart2 = ps;
        ps += (size_t)nch * ld;
        t.npart = ps;
        ps += 3 * (size_t)nch;
        t.nsc = ps;
        ps += 4;
        t.spart = ps;
        ps += (size_t)cgs_nsup(nch) * (2 * ld + 2);
        t.hv = ps;
        ps += ld;
        t.ord = reinterpret_cast<int *>(ps);
        ps += ld / 2 + 1;
        t.cnt = reinterpret_cast<int *>(ps);  // zeroed with the buffer; every launch leaves it zero
        ps += cgs_nsup(nch) / 2 + 1;
        t.st = st.as<int>() + 8 * q;
        for (int k = 0; k < nch; ++k) {
          if (k % kCgsSup == 0) lmap.push_back((int)cmap.size());
          cmap.push_back(q);
        }
      }
      CK(cudaMemcpyAsync(st.p, st0.data(), sizeof(int) * st0.size(), cudaMemcpyHostToDevice, c->stream));
      DBuf dt = upload(c, tasks), dm = upload(c, cmap), dl = upload(c, lmap);
      cudaEvent_t e0, e1, e2;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      CK(cudaEventCreate(&e2));
      double tdot = 0, tupd = 0;
      prepare_cgs<T>();
      for (int r = -2; r < reps; ++r) {  // two untimed rounds
        CK(cudaMemcpyAsync(W.p, W0.p, W.bytes, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaEventRecord(e0, c->stream));
        launch_cgs_dot<T>(dt.as<EigTask<T>>(), dm.as<int>(), (int)cmap.size(), c->stream);
        launch_cgs_coef<T>(dt.as<EigTask<T>>(), dm.as<int>(), dl.as<int>(), (int)lmap.size(), c->stream);
        CK(cudaEventRecord(e1, c->stream));
        launch_cgs_upd<T>(dt.as<EigTask<T>>(), dm.as<int>(), (int)cmap.size(), c->stream);
        CK(cudaEventRecord(e2, c->stream));
        sync(c);
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, e0, e1));
        CK(cudaEventElapsedTime(&b, e1, e2));
        if (r >= 0) {
          tdot += a;
          tupd += b;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaEventDestroy(e2);
      if (take_cgs_stall()) throw ApiError(EDGPU_ERR_CUDA, "a bulk copy into shared memory did not complete");
      if (ms_dot) *ms_dot = tdot / reps;
      if (ms_upd) *ms_upd = tupd / reps;
      // per task: the nbasis columns (V[j] among them) and w read (dot pass); the columns read and w read and
      // written (update pass)
      if (bytes_dot) *bytes_dot = (double)ntasks * (nbasis + 1) * (double)n * sizeof(T);
      if (bytes_upd) *bytes_upd = (double)ntasks * (nbasis + 2) * (double)n * sizeof(T);
    };
    if (prec == EDGPU_FP32) run(float());
    else run(double());
    return EDGPU_OK;
  });
}

int edgpu_server_create(edgpu_ctx *c, int precision, size_t hbm_budget, edgpu_server **out) {
  if (!c || !out) return EDGPU_ERR_ARG;
  *out = nullptr;
  return guard(c, [&]() {
    *out = server_create(c, precision, hbm_budget);
    return EDGPU_OK;
  });
}

int edgpu_server_destroy(edgpu_server *s) {
  if (!s) return EDGPU_ERR_ARG;
  server_destroy(s);
  return EDGPU_OK;
}

int edgpu_server_submit(edgpu_server *s, edgpu_model *m, const edgpu_diag_params *dp, const edgpu_gf_params *gp,
                        double *G, double *G_ij, double *Z, long long *ticket) {
  if (!s || !m || !dp || !ticket) return EDGPU_ERR_ARG;
  return guard(m->ctx, [&]() {
    *ticket = server_submit(s, m, dp, gp, G, G_ij, Z);
    return EDGPU_OK;
  });
}

int edgpu_server_step(edgpu_server *s, int *running, int *queued) {
  if (!s) return EDGPU_ERR_ARG;
  return guard(server_ctx(s), [&]() {
    server_step(s, running, queued);
    return EDGPU_OK;
  });
}

int edgpu_server_poll(edgpu_server *s, long long ticket, int *state, int *npairs) {
  if (!s || !state) return EDGPU_ERR_ARG;
  return guard(server_ctx(s), [&]() {
    *state = server_poll(s, ticket, npairs);
    return EDGPU_OK;
  });
}

long long edgpu_launch_count(void) { return edgpu::launch_count(); }

int edgpu_selftest_bulk_wait(edgpu_ctx *ctx, int rounds, int *gave_up, int *flagged) {
  if (!ctx || rounds < 1 || rounds > (1 << 22) || !gave_up || !flagged) return EDGPU_ERR_ARG;
  return guard(ctx, [&]() {
    DBuf d(ctx->alloc, sizeof(int));
    CK(cudaMemsetAsync(d.p, 0, sizeof(int), ctx->stream));
    launch_wait_selftest(rounds, d.as<int>(), ctx->stream);
    CK(cudaMemcpyAsync(gave_up, d.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *flagged = take_mv_stall() ? 1 : 0;
    return EDGPU_OK;
  });
}

int edgpu_stats(const edgpu_model *m, long long *spmv_vectors, long long *lanczos_steps, long long *restarts,
                double *element_steps) {
  if (!m) return EDGPU_ERR_ARG;
  if (element_steps) *element_steps = m->st_work;
  if (spmv_vectors) *spmv_vectors = m->st_spmv;
  if (lanczos_steps) *lanczos_steps = m->st_steps;
  if (restarts) *restarts = m->st_restarts;
  return EDGPU_OK;
}

}  // extern "C"
