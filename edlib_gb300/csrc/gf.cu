// Green's-function and susceptibility drivers on the device.
//
// * GreensFunction::compute (include/edlib/GreensFunction.h:109-159): Z over all eigen-pairs, Boltzmann
//   cut-off, per kept pair and orbital/spin the start vectors c+|n> and c|n> (create_particles /
//   annihilate_particles, GreensFunction.h:389-462), then the Lanczos recurrence and the continued
//   fraction into G_g / G_l; pairs (c_i + c_j) for G_ij (GreensFunction.h:290-359).
// * ChiLoc::compute<Op> (include/edlib/ChiLoc.h:180-276): start vectors O|n> in the same sector,
//   symmetrised bosonic fraction, zero-frequency sum rule with the c2/w^2 + c4/w^4 tail.
// * StaticObservables (include/edlib/StaticObservables.h:106-158, 356-421): Boltzmann averages of
//   occupation observables over the kept eigen-pairs.
// All start vectors of a call are built first, their norms read back once, and every recurrence of
// the call advances together in one batched launch per phase.
#include "model_internal.h"

namespace edgpu {

__global__ void k_gf_finalize(double *Gg, double *Gl, double *Ggij, double *Glij, double *G, double *Gij, int nw,
                              int nint, double Z, const int *diag, int ndiag, const int *pairs, int npairs, int nspin) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const long long n1 = (long long)nint * nspin, n2 = (long long)nint * nint * nspin;
  double *gg = Gg + 2 * w * n1, *gl = Gl + 2 * w * n1, *ggij = Ggij + 2 * w * n2, *glij = Glij + 2 * w * n2;
  for (long long e = 0; e < 2 * n1; ++e) { gg[e] /= Z; gl[e] /= Z; }
  for (long long e = 0; e < 2 * n2; ++e) { ggij[e] /= Z; glij[e] /= Z; }
  // GreensFunction::non_local_gf (GreensFunction.h:336-359)
  for (int q = 0; q < npairs; ++q) {
    int i = pairs[2 * q], j = pairs[2 * q + 1];
    for (int s = 0; s < nspin; ++s) {
      long long x = ((long long)(nint * i + j) * nspin + s) * 2;
      for (int jj = 0; jj < 2; ++jj) {
        long long y = ((long long)(jj ? j : i) * nspin + s) * 2;
        ggij[x] -= gg[y]; ggij[x + 1] -= gg[y + 1];
        glij[x] -= gl[y]; glij[x + 1] -= gl[y + 1];
      }
      ggij[x] *= 0.5; ggij[x + 1] *= 0.5;
      glij[x] *= 0.5; glij[x + 1] *= 0.5;
    }
  }
  for (int q = 0; q < ndiag; ++q) {
    int o = diag[q];
    for (int s = 0; s < nspin; ++s) {
      long long x = ((long long)(nint * o + o) * nspin + s) * 2, y = ((long long)o * nspin + s) * 2;
      ggij[x] = gg[y]; ggij[x + 1] = gg[y + 1];
      glij[x] = gl[y]; glij[x + 1] = gl[y + 1];
    }
  }
  double *g = G + 2 * w * n1, *gij = Gij + 2 * w * n2;
  for (long long e = 0; e < 2 * n1; ++e) g[e] = gg[e] + gl[e];
  for (long long e = 0; e < 2 * n2; ++e) gij[e] = ggij[e] + glij[e];
}

__global__ void k_div(double *x, long long n, double Z) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] /= Z;
}

// ChiLoc::non_local_correction's combination step (ChiLoc.h:262-275)
__global__ void k_chi_combine(double *g, double *gij, int nw, int nint, const int *diag, int ndiag, const int *pairs,
                              int npairs) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  double *a = g + 2 * (long long)w * nint, *b = gij + 2 * (long long)w * nint * nint;
  for (int q = 0; q < npairs; ++q) {
    int i = pairs[2 * q], j = pairs[2 * q + 1];
    long long x = 2 * (long long)(nint * i + j);
    for (int jj = 0; jj < 2; ++jj) {
      int o = jj ? j : i;
      b[x] -= a[2 * o];
      b[x + 1] -= a[2 * o + 1];
    }
    b[x] *= 0.5;
    b[x + 1] *= 0.5;
  }
  for (int q = 0; q < ndiag; ++q) {
    int o = diag[q];
    b[2 * (long long)(nint * o + o)] = a[2 * o];
    b[2 * (long long)(nint * o + o) + 1] = a[2 * o + 1];
  }
}

// occupation statistics of one eigenvector: quantity q of group blockIdx.y
template <typename T>
__global__ void k_static(SectorOp<T> op, const T *v, int nint, int Q, double *partial) {
  __shared__ double red[8];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int q0 = blockIdx.y * 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < op.dim; i += (long long)gridDim.x * blockDim.x) {
    const double x = (double)v[i];
    const double wgt = x * x;
    const state_t s = sector_state(op, i);
    for (int qq = 0; qq < 8; ++qq) {
      const int q = q0 + qq;
      if (q >= Q) break;
      double f;
      if (q < nint) {
        f = occ(s, q, op.ip);
      } else if (q < 2 * nint) {
        f = occ(s, q - nint + op.ns, op.ip);
      } else if (q < 3 * nint) {
        int o = q - 2 * nint;
        f = occ(s, o, op.ip) * occ(s, o + op.ns, op.ip);
      } else if (q < 3 * nint + nint * nint) {
        int r = q - 3 * nint, o1 = r / nint, o2 = r % nint;
        // StaticObservables.h:383-385 reads the second down occupation at bit orb2 + interacting_orbitals()
        f = (double)(occ(s, o1, op.ip) - occ(s, o1 + op.ns, op.ip)) * (double)(occ(s, o2, op.ip) - occ(s, o2 + nint, op.ip));
      } else {
        f = wgt;
      }
      acc[qq] += wgt * f;
    }
  }
  for (int qq = 0; qq < 8; ++qq) {
    double s = block_sum<256>(acc[qq], red);
    if (threadIdx.x == 0 && q0 + qq < Q) partial[(long long)(q0 + qq) * gridDim.x + blockIdx.x] = s;
  }
}

namespace host {

template <typename T>
struct LzJob {
  Sector *s = nullptr;
  DBuf buf[3];
  DBuf alpha, beta, part_a, part_b, scal, state;
};

template <typename T>
void run_lanczos(edgpu_model *m, std::vector<LzJob<T> *> &jobs, int nlanc) {
  edgpu_ctx *c = m->ctx;
  if (jobs.empty() || nlanc <= 0) return;
  std::vector<LzTask<T>> tasks(jobs.size());
  std::vector<int> item_task;
  int smem = 0;
  for (size_t q = 0; q < jobs.size(); ++q) {
    LzJob<T> &J = *jobs[q];
    Sector &s = *J.s;
    J.alpha = DBuf(c->alloc, sizeof(double) * nlanc);
    J.beta = DBuf(c->alloc, sizeof(double) * (nlanc + 1));
    J.part_a = DBuf(c->alloc, sizeof(double) * s.nitems);
    J.part_b = DBuf(c->alloc, sizeof(double) * s.nitems);
    J.scal = DBuf(c->alloc, sizeof(double) * 2);
    J.state = DBuf(c->alloc, sizeof(int) * 2);
    CK(cudaMemsetAsync(J.alpha.p, 0, sizeof(double) * nlanc, c->stream));
    CK(cudaMemsetAsync(J.beta.p, 0, sizeof(double) * (nlanc + 1), c->stream));
    CK(cudaMemsetAsync(J.scal.p, 0, sizeof(double) * 2, c->stream));
    CK(cudaMemsetAsync(J.state.p, 0, sizeof(int) * 2, c->stream));
    LzTask<T> &t = tasks[q];
    t.op = s.dop<T>();
    t.srs_rows = s.srs_rows;
    t.item_begin = (int)item_task.size();
    t.nitems = s.nitems;
    for (int b = 0; b < 3; ++b) t.buf[b] = J.buf[b].template as<T>();
    t.alpha = J.alpha.template as<double>();
    t.beta = J.beta.template as<double>();
    t.part_a = J.part_a.template as<double>();
    t.part_b = J.part_b.template as<double>();
    t.scal = J.scal.template as<double>();
    t.state = J.state.template as<int>();
    t.nlanc_max = nlanc;
    for (int it = 0; it < s.nitems; ++it) item_task.push_back((int)q);
    smem = std::max(smem, smem_elems_for<T>(s));
  }
  DBuf dt = upload(c, tasks), dm = upload(c, item_task);
  for (int it = 0; it < nlanc; ++it)
    launch_lz_step<T>(dt.template as<LzTask<T>>(), dm.template as<int>(), (int)item_task.size(), (int)jobs.size(), it, smem, c->stream);
  CK(cudaGetLastError());
  sync(c);
  m->st_steps += nlanc;
  for (auto *J : jobs) {
    m->st_work += (double)nlanc * (double)J->s->dim;
    m->st_spmv += nlanc;
  }
}

static void orbital_lists(const edgpu_model *m, const edgpu_gf_params *p, std::vector<int> &diag, std::vector<int> &pairs) {
  const int nint = m->interacting();
  std::vector<std::pair<int, int>> lst;
  if (p->orbitals && p->n_orbitals > 0) {
    for (int q = 0; q < p->n_orbitals; ++q) lst.push_back({p->orbitals[2 * q], p->orbitals[2 * q + 1]});
  } else {
    for (int i = 0; i < nint; ++i) lst.push_back({i, i});
  }
  for (auto &pr : lst) {
    if (pr.first < 0 || pr.second < 0 || pr.first >= nint || pr.second >= nint)
      throw ApiError(EDGPU_ERR_ARG, "orbital index out of range");
    if (pr.first == pr.second) diag.push_back(pr.first);
    else { pairs.push_back(pr.first); pairs.push_back(pr.second); }
  }
  std::sort(diag.begin(), diag.end());
  diag.erase(std::unique(diag.begin(), diag.end()), diag.end());
  for (size_t q = 0; q < pairs.size(); ++q)
    if (std::find(diag.begin(), diag.end(), pairs[q]) == diag.end()) diag.push_back(pairs[q]);
}

struct Kept {
  const Pair *pair;
  double bf;
};

static void boltzmann(const edgpu_model *m, double beta, double cutoff, double &E0, double &Z, std::vector<Kept> &keep) {
  E0 = m->pairs.front().E;
  Z = 0.0;
  for (auto &p : m->pairs) Z += std::exp(-(p.E - E0) * beta);
  for (auto &p : m->pairs) {
    double bf = std::exp(-(p.E - E0) * beta);
    if (std::fabs(cutoff - bf) > std::numeric_limits<double>::epsilon() && bf < cutoff) continue;
    keep.push_back({&p, bf});
  }
}

static int diag_storage(const edgpu_model *m) { return m->diag_storage; }

// the eigenvector of a pair in precision T (converted through a scratch buffer if needed)
template <typename T>
const T *pair_vector(edgpu_model *m, const Pair &p, std::vector<DBuf> &scratch) {
  if (p.prec == (sizeof(T) == 8 ? EDGPU_FP64 : EDGPU_FP32)) return p.vec<T>();
  edgpu_ctx *c = m->ctx;
  scratch.emplace_back(c->alloc, sizeof(T) * p.n);
  T *dst = scratch.back().template as<T>();
  if (p.prec == EDGPU_FP64) launch_convert<T>(p.vec<double>(), dst, p.n, c->stream);
  else {
    DBuf tmp(c->alloc, sizeof(double) * p.n);
    launch_to_double<float>(p.vec<float>(), tmp.template as<double>(), p.n, c->stream);
    launch_convert<T>(tmp.template as<double>(), dst, p.n, c->stream);
    sync(c);
  }
  return dst;
}

template <typename T>
int gf_impl(edgpu_model *m, const edgpu_gf_params *p, double *G, double *Gij, double *Z_out) {
  edgpu_ctx *c = m->ctx;
  if (!m->have_pairs) throw ApiError(EDGPU_ERR_STATE, "diag() has not been run");
  if (m->evals_only) throw ApiError(EDGPU_ERR_STATE, "Eigenvectors have not been computed. Green's function can not be evaluated.");
  const int nint = m->interacting(), nw = p->nomega, nsp = 2;
  if (nw < 1 || p->nlanc < 1) throw ApiError(EDGPU_ERR_ARG, "NOMEGA and NLANC must be positive");
  std::vector<int> diag, pairs;
  orbital_lists(m, p, diag, pairs);
  const size_t n1 = (size_t)nw * nint * nsp * 2, n2 = (size_t)nw * nint * nint * nsp * 2;
  DBuf Gg(c->alloc, sizeof(double) * n1), Gl(c->alloc, sizeof(double) * n1), Ggij(c->alloc, sizeof(double) * n2),
      Glij(c->alloc, sizeof(double) * n2), Go(c->alloc, sizeof(double) * n1), Gijo(c->alloc, sizeof(double) * n2);
  for (DBuf *b : {&Gg, &Gl, &Ggij, &Glij}) CK(cudaMemsetAsync(b->p, 0, b->bytes, c->stream));
  double Z = 0.0, E0 = 0.0;
  std::vector<Kept> keep;
  if (!m->pairs.empty()) boltzmann(m, p->beta, p->cutoff, E0, Z, keep);
  std::vector<double> om(nw);
  for (int w = 0; w < nw; ++w) om[w] = (2.0 * w + 1) * M_PI / p->beta;
  DBuf dom = upload(c, om);
  const int storage = diag_storage(m);
  std::vector<DBuf> scratch;
  struct Start {
    std::unique_ptr<LzJob<T>> job;
    double E;
    int isign;
    double *out;
    long long stride;
  };
  std::vector<Start> starts;
  const int np = (int)pairs.size() / 2;
  DBuf norms(c->alloc, sizeof(double) * std::max<size_t>(1, keep.size() * (diag.size() + np) * 4));
  DBuf parts(c->alloc, sizeof(double) * 64 * std::max<size_t>(1, keep.size() * (diag.size() + np) * 4));
  for (auto &kp : keep) {
    const Pair &pr = *kp.pair;
    const T *src = pair_vector<T>(m, pr, scratch);
    Sector *ss = get_sector(m, storage, pr.nup, pr.ndn);
    auto add = [&](const std::vector<int> &orbs, int spin, bool create, double *out, long long stride) {
      int tu = pr.nup, td = pr.ndn;
      if (create) { tu += 1 - spin; td += spin; }
      else {
        if ((spin == 0 ? pr.nup : pr.ndn) <= 0) return;
        tu -= 1 - spin; td -= spin;
      }
      if (tu > m->ns || td > m->ns) return;
      Sector *ts = get_sector(m, storage, tu, td);
      Start st;
      st.job.reset(new LzJob<T>());
      st.job->s = ts;
      for (int b = 0; b < 3; ++b) st.job->buf[b] = DBuf(c->alloc, sizeof(T) * ts->dim);
      for (size_t q = 0; q < orbs.size(); ++q)
        launch_a_adag<T>(ss->op<T>(), ts->op<T>(), orbs[q] + spin * m->ns, create ? 0 : 1, src, st.job->buf[0].template as<T>(),
                         q > 0 ? 1 : 0, c->stream);
      const size_t k = starts.size();
      launch_dot_partials<T>(st.job->buf[0].template as<T>(), st.job->buf[0].template as<T>(), ts->dim, parts.template as<double>() + 64 * k, 64,
                             c->stream);
      launch_reduce(parts.template as<double>() + 64 * k, 64, norms.template as<double>() + k, c->stream);
      st.E = pr.E;
      st.isign = create ? 1 : -1;
      st.out = out;
      st.stride = stride;
      starts.push_back(std::move(st));
    };
    for (int orb : diag)
      for (int spin = 0; spin < nsp; ++spin) {
        add({orb}, spin, true, Gg.template as<double>() + 2 * ((long long)orb * nsp + spin), (long long)nint * nsp);
        add({orb}, spin, false, Gl.template as<double>() + 2 * ((long long)orb * nsp + spin), (long long)nint * nsp);
      }
    for (int q = 0; q < np; ++q) {
      int i = pairs[2 * q], j = pairs[2 * q + 1];
      for (int spin = 0; spin < nsp; ++spin) {
        long long idx = (long long)nint * i + j;
        add({i, j}, spin, true, Ggij.template as<double>() + 2 * (idx * nsp + spin), (long long)nint * nint * nsp);
        add({i, j}, spin, false, Glij.template as<double>() + 2 * (idx * nsp + spin), (long long)nint * nint * nsp);
      }
    }
  }
  std::vector<double> hn(starts.size());
  if (!starts.empty())
    CK(cudaMemcpyAsync(hn.data(), norms.p, sizeof(double) * hn.size(), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  std::vector<LzJob<T> *> run;
  std::vector<CfJob> cf;
  for (size_t k = 0; k < starts.size(); ++k) {
    if (!(std::fabs(hn[k]) > 1e-10)) continue;
    LzJob<T> &J = *starts[k].job;
    launch_scale<T>(J.buf[0].template as<T>(), J.s->dim, norms.template as<double>() + k, 1, c->stream);
    run.push_back(&J);
  }
  run_lanczos<T>(m, run, p->nlanc);
  for (size_t k = 0; k < starts.size(); ++k) {
    if (!(std::fabs(hn[k]) > 1e-10)) continue;
    LzJob<T> &J = *starts[k].job;
    CfJob jb;
    jb.alpha = J.alpha.template as<double>();
    jb.beta = J.beta.template as<double>();
    jb.state = J.state.template as<int>();
    jb.expectation = hn[k];
    jb.E = starts[k].E;
    jb.E0 = E0;
    jb.isign = starts[k].isign;
    jb.sym = 0;
    jb.out = starts[k].out;
    jb.out_stride = starts[k].stride;
    cf.push_back(jb);
  }
  DBuf dcf = upload(c, cf);
  launch_cf(dcf.template as<CfJob>(), (int)cf.size(), dom.template as<double>(), nw, p->beta, c->stream);
  DBuf ddiag = upload(c, diag), dpairs = upload(c, pairs);
  if (!keep.empty()) {
    k_gf_finalize<<<(nw + 127) / 128, 128, 0, c->stream>>>(Gg.template as<double>(), Gl.template as<double>(), Ggij.template as<double>(),
                                                           Glij.template as<double>(), Go.template as<double>(), Gijo.template as<double>(), nw, nint,
                                                           Z, ddiag.template as<int>(), (int)diag.size(), dpairs.template as<int>(), np, nsp); note_launch();
  } else {
    CK(cudaMemsetAsync(Go.p, 0, Go.bytes, c->stream));
    CK(cudaMemsetAsync(Gijo.p, 0, Gijo.bytes, c->stream));
  }
  CK(cudaGetLastError());
  if (G) CK(cudaMemcpyAsync(G, Go.p, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
  if (Gij) CK(cudaMemcpyAsync(Gij, Gijo.p, sizeof(double) * n2, cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  if (Z_out) *Z_out = Z;
  return EDGPU_OK;
}

template <typename T>
int chi_impl(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chiij, double *Z_out) {
  edgpu_ctx *c = m->ctx;
  if (!m->have_pairs) throw ApiError(EDGPU_ERR_STATE, "diag() has not been run");
  if (m->evals_only) throw ApiError(EDGPU_ERR_STATE, "Eigenvectors have not been computed. Green's function can not be evaluated.");
  if (op != EDGPU_OP_SZ && op != EDGPU_OP_N) throw ApiError(EDGPU_ERR_ARG, "unknown operator");
  const int nint = m->interacting(), nw = p->nomega;
  if (nw < 3 || p->nlanc < 1) throw ApiError(EDGPU_ERR_ARG, "NOMEGA must be >= 3 and NLANC positive");
  std::vector<int> diag, pairs;
  orbital_lists(m, p, diag, pairs);
  const int np = (int)pairs.size() / 2;
  const size_t n1 = (size_t)nw * nint * 2, n2 = (size_t)nw * nint * nint * 2;
  DBuf g(c->alloc, sizeof(double) * n1), gij(c->alloc, sizeof(double) * n2);
  CK(cudaMemsetAsync(g.p, 0, g.bytes, c->stream));
  CK(cudaMemsetAsync(gij.p, 0, gij.bytes, c->stream));
  double Z = 0.0, E0 = 0.0;
  std::vector<Kept> keep;
  if (!m->pairs.empty()) boltzmann(m, p->beta, p->cutoff, E0, Z, keep);
  std::vector<double> om(nw);
  for (int w = 0; w < nw; ++w) om[w] = (2.0 * w) * M_PI / p->beta;
  DBuf dom = upload(c, om);
  const int storage = diag_storage(m);
  std::vector<DBuf> scratch;
  struct Start {
    std::unique_ptr<LzJob<T>> job;
    double E;
    bool local;
    double *out;
    long long stride;
  };
  std::vector<Start> starts;
  const size_t maxs = std::max<size_t>(1, keep.size() * (diag.size() + np));
  DBuf norms(c->alloc, sizeof(double) * maxs), parts(c->alloc, sizeof(double) * 64 * maxs);
  for (auto &kp : keep) {
    const Pair &pr = *kp.pair;
    const T *src = pair_vector<T>(m, pr, scratch);
    Sector *ss = get_sector(m, storage, pr.nup, pr.ndn);
    auto add = [&](int mu, int nu, double *out, long long stride) {
      Start st;
      st.job.reset(new LzJob<T>());
      st.job->s = ss;
      for (int b = 0; b < 3; ++b) st.job->buf[b] = DBuf(c->alloc, sizeof(T) * ss->dim);
      launch_diag_op<T>(ss->op<T>(), op, mu, nu, src, st.job->buf[0].template as<T>(), c->stream);
      const size_t k = starts.size();
      launch_dot_partials<T>(st.job->buf[0].template as<T>(), st.job->buf[0].template as<T>(), ss->dim, parts.template as<double>() + 64 * k, 64,
                             c->stream);
      launch_reduce(parts.template as<double>() + 64 * k, 64, norms.template as<double>() + k, c->stream);
      st.E = pr.E;
      st.local = nu < 0;
      st.out = out;
      st.stride = stride;
      starts.push_back(std::move(st));
    };
    for (int orb : diag) add(orb, -1, g.template as<double>() + 2 * orb, nint);
    for (int q = 0; q < np; ++q)
      add(pairs[2 * q], pairs[2 * q + 1], gij.template as<double>() + 2 * ((long long)nint * pairs[2 * q] + pairs[2 * q + 1]),
          (long long)nint * nint);
  }
  std::vector<double> hn(starts.size());
  if (!starts.empty())
    CK(cudaMemcpyAsync(hn.data(), norms.p, sizeof(double) * hn.size(), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  std::vector<LzJob<T> *> run;
  std::vector<CfJob> cf;
  std::vector<char> use(starts.size(), 0);
  for (size_t k = 0; k < starts.size(); ++k) {
    use[k] = starts[k].local ? (hn[k] > 1e-9) : 1;
    if (!use[k]) continue;
    LzJob<T> &J = *starts[k].job;
    launch_scale<T>(J.buf[0].template as<T>(), J.s->dim, norms.template as<double>() + k, 1, c->stream);
    run.push_back(&J);
  }
  run_lanczos<T>(m, run, p->nlanc);
  for (size_t k = 0; k < starts.size(); ++k) {
    if (!use[k]) continue;
    LzJob<T> &J = *starts[k].job;
    CfJob jb;
    jb.alpha = J.alpha.template as<double>();
    jb.beta = J.beta.template as<double>();
    jb.state = J.state.template as<int>();
    jb.expectation = hn[k];
    jb.E = starts[k].E;
    jb.E0 = E0;
    jb.isign = 1;
    jb.sym = 1;
    jb.out = starts[k].out;
    jb.out_stride = starts[k].stride;
    cf.push_back(jb);
  }
  DBuf dcf = upload(c, cf);
  launch_cf(dcf.template as<CfJob>(), (int)cf.size(), dom.template as<double>(), nw, p->beta, c->stream);
  if (!keep.empty()) {
    k_div<<<(unsigned)((n1 + 255) / 256), 256, 0, c->stream>>>(g.template as<double>(), (long long)n1, Z); note_launch();
    k_div<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(gij.template as<double>(), (long long)n2, Z); note_launch();
    for (int orb : diag) launch_chi_tail(g.template as<double>() + 2 * orb, nint, nw, dom.template as<double>(), p->beta, avg, c->stream);
    for (int q = 0; q < np; ++q)
      launch_chi_tail(gij.template as<double>() + 2 * ((long long)nint * pairs[2 * q] + pairs[2 * q + 1]), (long long)nint * nint,
                      nw, dom.template as<double>(), p->beta, avg, c->stream);
    DBuf ddiag = upload(c, diag), dpairs = upload(c, pairs);
    k_chi_combine<<<(nw + 127) / 128, 128, 0, c->stream>>>(g.template as<double>(), gij.template as<double>(), nw, nint, ddiag.template as<int>(),
                                                           (int)diag.size(), dpairs.template as<int>(), np); note_launch();
    CK(cudaGetLastError());
    sync(c);
  }
  if (chi) CK(cudaMemcpyAsync(chi, g.p, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
  if (chiij) CK(cudaMemcpyAsync(chiij, gij.p, sizeof(double) * n2, cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  if (Z_out) *Z_out = Z;
  return EDGPU_OK;
}

int gf_dispatch(edgpu_model *m, const edgpu_gf_params *p, double *G, double *Gij, double *Z) {
  if (p->precision == EDGPU_FP32) return gf_impl<float>(m, p, G, Gij, Z);
  return gf_impl<double>(m, p, G, Gij, Z);
}

int chi_dispatch(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chiij, double *Z) {
  if (p->precision == EDGPU_FP32) return chi_impl<float>(m, p, op, avg, chi, chiij, Z);
  return chi_impl<double>(m, p, op, avg, chi, chiij, Z);
}

int static_obs(edgpu_model *m, double beta, double cutoff, double *n, double *n_up, double *n_dn, double *mag,
               double *d_occ, double *mimj, double *n_eff, double *energy) {
  edgpu_ctx *c = m->ctx;
  if (!m->have_pairs || m->pairs.empty()) throw ApiError(EDGPU_ERR_STATE, "diag() has not been run");
  if (m->evals_only) throw ApiError(EDGPU_ERR_STATE, "Eigenvectors have not been computed. StaticObservables can not continue.");
  const int nint = m->interacting();
  const int Q = 3 * nint + nint * nint + 1;
  const int gx = 64, gy = (Q + 7) / 8;
  double E0, Z;
  std::vector<Kept> keep;
  boltzmann(m, beta, cutoff, E0, Z, keep);
  std::vector<double> acc(Q + 1, 0.0);  // last: energy
  double tot = 0.0;
  DBuf part(c->alloc, sizeof(double) * (size_t)Q * gx);
  std::vector<double> hp((size_t)Q * gx);
  const int storage = diag_storage(m);
  for (auto &kp : keep) {
    const Pair &pr = *kp.pair;
    Sector *s = get_sector(m, storage, pr.nup, pr.ndn);
    if (pr.prec == EDGPU_FP64) {
      k_static<double><<<dim3(gx, gy), 256, 0, c->stream>>>(s->op<double>(), pr.vec<double>(), nint, Q, part.template as<double>()); note_launch();
    } else {
      k_static<float><<<dim3(gx, gy), 256, 0, c->stream>>>(s->op<float>(), pr.vec<float>(), nint, Q, part.template as<double>()); note_launch();
    }
    CK(cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (int q = 0; q < Q; ++q) {
      double s2 = 0.0;
      for (int x = 0; x < gx; ++x) s2 += hp[(size_t)q * gx + x];
      acc[q] += (q == Q - 1 ? 1.0 / s2 : s2) * kp.bf;
    }
    acc[Q] += pr.E * kp.bf;
    tot += kp.bf;
  }
  for (int o = 0; o < nint; ++o) {
    double up = acc[o] / tot, dn = acc[nint + o] / tot;
    if (n) n[o] = up + dn;
    if (n_up) n_up[o] = up;
    if (n_dn) n_dn[o] = dn;
    if (mag) mag[o] = up - dn;
    if (d_occ) d_occ[o] = acc[2 * nint + o] / tot;
  }
  if (mimj)
    for (int q = 0; q < nint * nint; ++q) mimj[q] = acc[3 * nint + q] / tot;
  if (n_eff) *n_eff = acc[Q - 1] / tot;
  if (energy) *energy = acc[Q] / tot;
  return EDGPU_OK;
}

template <typename T>
void lanczos_batch(edgpu_model *m, const std::vector<Sector *> &secs, const std::vector<T *> &starts, int nlanc,
                   std::vector<DBuf> &alpha, std::vector<DBuf> &beta, std::vector<DBuf> &state) {
  edgpu_ctx *c = m->ctx;
  std::vector<std::unique_ptr<LzJob<T>>> own;
  std::vector<LzJob<T> *> run;
  for (size_t q = 0; q < secs.size(); ++q) {
    own.emplace_back(new LzJob<T>());
    LzJob<T> &J = *own.back();
    J.s = secs[q];
    for (int b = 0; b < 3; ++b) J.buf[b] = DBuf(c->alloc, sizeof(T) * secs[q]->dim);
    CK(cudaMemcpyAsync(J.buf[0].p, starts[q], sizeof(T) * secs[q]->dim, cudaMemcpyDeviceToDevice, c->stream));
    run.push_back(&J);
  }
  run_lanczos<T>(m, run, nlanc);
  for (auto &J : own) {
    alpha.push_back(std::move(J->alpha));
    beta.push_back(std::move(J->beta));
    state.push_back(std::move(J->state));
  }
}

template void lanczos_batch<float>(edgpu_model *, const std::vector<Sector *> &, const std::vector<float *> &, int,
                                   std::vector<DBuf> &, std::vector<DBuf> &, std::vector<DBuf> &);
template void lanczos_batch<double>(edgpu_model *, const std::vector<Sector *> &, const std::vector<double *> &, int,
                                    std::vector<DBuf> &, std::vector<DBuf> &, std::vector<DBuf> &);

}  // namespace host
}  // namespace edgpu
