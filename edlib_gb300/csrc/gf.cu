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
// The start vectors of a call are built in groups bounded by device memory (and max_batch), their norms
// read back once per group, and every recurrence of a group advances together in one batched launch per
// phase; only the Lanczos coefficients are kept for the fractions.
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
  edgpu_model *m = nullptr;  // the model the sector belongs to (float-float tables are built from its data)
  DBuf buf[3];
  DBuf alpha, beta, part_a, part_b, scal, state;
};

// EDGPU_TRACE_LZ: the first recurrence coefficients of every job on stderr (after the recurrences, for diagnosis)
template <typename T>
void trace_coefficients(const std::vector<LzJob<T> *> &jobs, int nlanc, const char *tag) {
  if (!getenv("EDGPU_TRACE_LZ")) return;
  for (size_t q = 0; q < jobs.size(); ++q) {
    double a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
    CK(cudaMemcpy(a, jobs[q]->alpha.p, sizeof(double) * std::min(nlanc, 4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b, jobs[q]->beta.p, sizeof(double) * std::min(nlanc + 1, 4), cudaMemcpyDeviceToHost));
    fprintf(stderr, "lz %s job %zu sector (%d,%d): alpha %.17g %.17g %.17g beta %.17g %.17g %.17g\n", tag, q,
            jobs[q]->s->nup, jobs[q]->s->ndn, a[0], a[1], a[2], b[1], b[2], b[3]);
  }
}

// The recurrences of FP64 jobs in float-float (`ff`, the mixed mode on spin-resolved sectors): each job's
// normalised FP64 start vector is rewritten in place as float-float (the same 8 bytes per element), the three
// buffers are read as float-float, and the steps run on the sector's float-float tables; alpha / beta stay FP64.
void run_lanczos_ff(edgpu_model *m, std::vector<LzJob<double> *> &jobs, int nlanc) {
  edgpu_ctx *c = m->ctx;
  std::vector<LzTask<ffloat>> tasks(jobs.size());
  std::vector<int> item_task;
  MvShape shape{kSRS, 0};
  for (size_t q = 0; q < jobs.size(); ++q) {
    LzJob<double> &J = *jobs[q];
    Sector &s = *J.s;
    ensure_ff(J.m ? J.m : m, &s);
    launch_convert<ffloat>(J.buf[0].as<double>(), J.buf[0].as<ffloat>(), s.dim, c->stream);
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
    LzTask<ffloat> &t = tasks[q];
    t.op = s.dop<ffloat>();
    t.srs_rows = s.srs_rows;
    t.item_begin = (int)item_task.size();
    t.nitems = s.nitems;
    for (int b = 0; b < 3; ++b) t.buf[b] = J.buf[b].as<ffloat>();
    t.alpha = J.alpha.as<double>();
    t.beta = J.beta.as<double>();
    t.part_a = J.part_a.as<double>();
    t.part_b = J.part_b.as<double>();
    t.scal = J.scal.as<double>();
    t.state = J.state.as<int>();
    t.nlanc_max = nlanc;
    for (int it = 0; it < s.nitems; ++it) item_task.push_back((int)q);
    merge_shape(shape, mv_shape<double>(s));  // float-float elements take the room of FP64 ones
  }
  {
    const OpTuning &tu = m->op_tune[0];
    if (tu.done && tu.ms > 0 && !getenv("EDGPU_SRS_STAGE_KB")) shape.staged = tu.staged;
  }
  DBuf dt = upload(c, tasks), dm = upload(c, item_task);
  for (int it = 0; it < nlanc; ++it)
    launch_lz_step<ffloat>(dt.as<LzTask<ffloat>>(), dm.as<int>(), (int)item_task.size(), (int)jobs.size(), it, shape,
                           c->stream);
  CK(cudaGetLastError());
  sync(c);
  trace_coefficients(jobs, nlanc, "ff");
  m->st_steps += nlanc;
  for (auto *J : jobs) {
    m->st_work += (double)nlanc * (double)J->s->dim;
    m->st_spmv += nlanc;
  }
}

template <typename T>
void run_lanczos(edgpu_model *m, std::vector<LzJob<T> *> &jobs, int nlanc, bool ff = false) {
  edgpu_ctx *c = m->ctx;
  if (jobs.empty() || nlanc <= 0) return;
  if constexpr (std::is_same<T, double>::value) {
    bool all_srs = true;
    for (auto *J : jobs) all_srs = all_srs && J->s->storage == kSRS;
    if (ff && all_srs) {
      run_lanczos_ff(m, jobs, nlanc);
      return;
    }
  }
  std::vector<LzTask<T>> tasks(jobs.size());
  std::vector<int> item_task;
  MvShape shape{jobs[0]->s->storage, 0};
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
    merge_shape(shape, mv_shape<T>(s));
  }
  {  // the model's tuned source-row staging (the recurrence's own kernel has one register variant)
    const OpTuning &tu = m->op_tune[sizeof(T) == 4 ? 1 : 0];
    if (tu.done && tu.ms > 0 && !getenv("EDGPU_SRS_STAGE_KB")) shape.staged = tu.staged;
  }
  DBuf dt = upload(c, tasks), dm = upload(c, item_task);
  for (int it = 0; it < nlanc; ++it)
    launch_lz_step<T>(dt.template as<LzTask<T>>(), dm.template as<int>(), (int)item_task.size(), (int)jobs.size(), it, shape, c->stream);
  CK(cudaGetLastError());
  sync(c);
  trace_coefficients(jobs, nlanc, sizeof(T) == 8 ? "fp64" : "fp32");
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

// One model's share of a Green's-function or susceptibility call: its start vectors, output buffers and
// Boltzmann data.  Several plans share one batched Lanczos run.
template <typename T>
struct GfPlan {
  edgpu_model *m = nullptr;
  bool chi = false;
  int op = 0;
  double avg = 0.0;
  int nint = 0, nw = 0, np = 0;
  std::vector<int> diag, pairs;
  size_t n1 = 0, n2 = 0;
  DBuf Gg, Gl, Ggij, Glij, Go, Gijo, dom;
  double Z = 0.0, E0 = 0.0;
  std::vector<Kept> keep;
  // A start vector is described here and built only when its recurrence runs (groups bounded by memory):
  // kind 0 = sum over orbs of a / a+ of spin `spin` applied to the pair's vector, kind 1 = a diagonal
  // operator (mu, nu) applied in the same sector, kind 2 = sum_j w_j a / a+ of orbital j.
  struct Start {
    std::unique_ptr<LzJob<T>> job;  // job->s: the recurrence's sector
    double E;
    int isign;
    bool local;
    double *out;
    long long stride;
    const T *src;
    Sector *from;
    int kind, orbs[2], norb, spin, create, mu, nu;
    const double *w;  // kind 2: weights of the orbital combination (n_int_orb of them)
  };
  std::vector<Start> starts;
  std::vector<DBuf> scratch;
  std::vector<double> hn;
  std::vector<char> use;
};

template <typename T>
void plan_prepare(GfPlan<T> &P, edgpu_model *m, const edgpu_gf_params *p, bool chi, int op, double avg,
                  const double *weights = nullptr, int nrows = 0) {
  edgpu_ctx *c = m->ctx;
  if (!m->have_pairs) throw ApiError(EDGPU_ERR_STATE, "diag() has not been run");
  if (m->evals_only) throw ApiError(EDGPU_ERR_STATE, "Eigenvectors have not been computed. Green's function can not be evaluated.");
  if (chi && op != EDGPU_OP_SZ && op != EDGPU_OP_N) throw ApiError(EDGPU_ERR_ARG, "unknown operator");
  P.m = m;
  P.chi = chi;
  P.op = op;
  P.avg = avg;
  P.nint = m->interacting();
  P.nw = p->nomega;
  if (P.nw < (chi ? 3 : 1) || p->nlanc < 1) throw ApiError(EDGPU_ERR_ARG, "NOMEGA (>= 3 for chi) and NLANC must be positive");
  const int nint_model = P.nint;
  if (weights) {  // one output row per orbital combination, no pairs
    if (chi || nrows < 1) throw ApiError(EDGPU_ERR_ARG, "orbital combinations need at least one weight row");
    P.nint = nrows;
    for (int r = 0; r < nrows; ++r) P.diag.push_back(r);
  } else {
    orbital_lists(m, p, P.diag, P.pairs);
  }
  P.np = (int)P.pairs.size() / 2;
  const int nsp = chi ? 1 : 2;
  P.n1 = (size_t)P.nw * P.nint * nsp * 2;
  P.n2 = (size_t)P.nw * P.nint * P.nint * nsp * 2;
  P.Gg = DBuf(c->alloc, sizeof(double) * P.n1);
  P.Ggij = DBuf(c->alloc, sizeof(double) * P.n2);
  CK(cudaMemsetAsync(P.Gg.p, 0, P.Gg.bytes, c->stream));
  CK(cudaMemsetAsync(P.Ggij.p, 0, P.Ggij.bytes, c->stream));
  if (!chi) {
    P.Gl = DBuf(c->alloc, sizeof(double) * P.n1);
    P.Glij = DBuf(c->alloc, sizeof(double) * P.n2);
    P.Go = DBuf(c->alloc, sizeof(double) * P.n1);
    P.Gijo = DBuf(c->alloc, sizeof(double) * P.n2);
    CK(cudaMemsetAsync(P.Gl.p, 0, P.Gl.bytes, c->stream));
    CK(cudaMemsetAsync(P.Glij.p, 0, P.Glij.bytes, c->stream));
  }
  if (!m->pairs.empty()) boltzmann(m, p->beta, p->cutoff, P.E0, P.Z, P.keep);
  std::vector<double> om(P.nw);
  if (p->mesh == EDGPU_MESH_REAL) {
    // RealFreqMeshFactory (MeshFactory.h:27-34): linear grid EMIN..EMAX
    if (P.nw < 2 || !(p->emax > p->emin)) throw ApiError(EDGPU_ERR_ARG, "the real mesh needs NOMEGA >= 2 and EMAX > EMIN");
    for (int w = 0; w < P.nw; ++w) om[w] = p->emin + (p->emax - p->emin) * w / double(P.nw - 1);
  } else {
    for (int w = 0; w < P.nw; ++w) om[w] = (2.0 * w + (chi ? 0 : 1)) * M_PI / p->beta;
  }
  P.dom = upload(c, om);
  const int storage = diag_storage(m);
  for (auto &kp : P.keep) {
    const Pair &pr = *kp.pair;
    const T *src = pair_vector<T>(m, pr, P.scratch);
    Sector *ss = get_sector(m, storage, pr.nup, pr.ndn);
    auto finish_start = [&](typename GfPlan<T>::Start &st, Sector *) {
      st.E = pr.E;
      st.src = src;
      st.from = ss;
      P.starts.push_back(std::move(st));
    };
    if (!chi) {
      // GreensFunction::create_particles / annihilate_particles (GreensFunction.h:389-462)
      auto add = [&](const std::vector<int> &orbs, int spin, bool create, double *out, long long stride) {
        int tu = pr.nup, td = pr.ndn;
        if (create) {
          tu += 1 - spin;
          td += spin;
        } else {
          if ((spin == 0 ? pr.nup : pr.ndn) <= 0) return;
          tu -= 1 - spin;
          td -= spin;
        }
        if (tu > m->ns || td > m->ns) return;
        Sector *ts = get_sector(m, storage, tu, td);
        typename GfPlan<T>::Start st;
        st.job.reset(new LzJob<T>());
        st.job->s = ts;
        st.job->m = P.m;
        st.kind = 0;
        st.norb = (int)orbs.size();
        for (size_t q = 0; q < orbs.size(); ++q) st.orbs[q] = orbs[q];
        st.spin = spin;
        st.create = create ? 1 : 0;
        st.w = nullptr;
        st.isign = create ? 1 : -1;
        st.local = orbs.size() == 1;
        st.out = out;
        st.stride = stride;
        finish_start(st, ts);
      };
      if (weights) {
        // orbital combinations c_w = sum_j w_j c_j: start vectors sum_j w_j c+_j |n> and sum_j w_j c_j |n>
        for (int r = 0; r < nrows; ++r)
          for (int spin = 0; spin < 2; ++spin)
            for (int create = 1; create >= 0; --create) {
              const size_t before = P.starts.size();
              add({0}, spin, create != 0, (create ? P.Gg : P.Gl).template as<double>() + 2 * ((long long)r * 2 + spin),
                  (long long)P.nint * 2);
              if (P.starts.size() > before) {
                auto &st = P.starts.back();
                st.kind = 2;
                st.norb = nint_model;
                st.w = weights + (size_t)r * nint_model;
                st.local = false;
              }
            }
      }
      for (int orb : weights ? std::vector<int>() : P.diag)
        for (int spin = 0; spin < 2; ++spin) {
          add({orb}, spin, true, P.Gg.template as<double>() + 2 * ((long long)orb * 2 + spin), (long long)P.nint * 2);
          add({orb}, spin, false, P.Gl.template as<double>() + 2 * ((long long)orb * 2 + spin), (long long)P.nint * 2);
        }
      for (int q = 0; q < P.np; ++q) {
        int i = P.pairs[2 * q], j = P.pairs[2 * q + 1];
        for (int spin = 0; spin < 2; ++spin) {
          long long idx = (long long)P.nint * i + j;
          add({i, j}, spin, true, P.Ggij.template as<double>() + 2 * (idx * 2 + spin), (long long)P.nint * P.nint * 2);
          add({i, j}, spin, false, P.Glij.template as<double>() + 2 * (idx * 2 + spin), (long long)P.nint * P.nint * 2);
        }
      }
    } else {
      // ChiLoc::operation (ChiLoc.h:474-530): O|n> in the same sector
      auto add = [&](int mu, int nu, double *out, long long stride) {
        typename GfPlan<T>::Start st;
        st.job.reset(new LzJob<T>());
        st.job->s = ss;
        st.job->m = P.m;
        st.kind = 1;
        st.mu = mu;
        st.nu = nu;
        st.w = nullptr;
        st.isign = 1;
        st.local = nu < 0;
        st.out = out;
        st.stride = stride;
        finish_start(st, ss);
      };
      for (int orb : P.diag) add(orb, -1, P.Gg.template as<double>() + 2 * orb, P.nint);
      for (int q = 0; q < P.np; ++q)
        add(P.pairs[2 * q], P.pairs[2 * q + 1],
            P.Ggij.template as<double>() + 2 * ((long long)P.nint * P.pairs[2 * q] + P.pairs[2 * q + 1]),
            (long long)P.nint * P.nint);
    }
  }
  P.hn.assign(P.starts.size(), 0.0);
  P.use.assign(P.starts.size(), 0);
}

// The recurrences of every plan of a call, in groups whose three vectors each fit `cap` bytes (and of at most
// max_batch recurrences): build the group's start vectors, read their norms back, normalise the kept ones
// (fermionic |.|^2 > 1e-10, GreensFunction.h:418; local chi > 1e-9, pairs always), run their recurrences
// together and release the vectors.  Only alpha / beta stay for the fractions.
template <typename T>
void run_starts(std::vector<std::unique_ptr<GfPlan<T>>> &plans, const edgpu_gf_params *p, edgpu_model *m0) {
  edgpu_ctx *c = m0->ctx;
  struct Ref {
    GfPlan<T> *P;
    size_t k;
  };
  std::vector<Ref> all;
  for (auto &P : plans)
    for (size_t k = 0; k < P->starts.size(); ++k) all.push_back({P.get(), k});
  const size_t cap = (size_t)16 << 30;
  const size_t most = p->max_batch > 0 ? (size_t)p->max_batch : all.size();
  for (size_t i = 0; i < all.size();) {
    size_t j = i, bytes = 0;
    while (j < all.size() && j - i < most) {
      const size_t b = 3 * sizeof(T) * (size_t)all[j].P->starts[all[j].k].job->s->dim;
      if (j > i && bytes + b > cap) break;
      bytes += b;
      ++j;
    }
    const size_t ng = j - i;
    DBuf parts(c->alloc, sizeof(double) * 64 * ng), norms(c->alloc, sizeof(double) * ng);
    for (size_t q = 0; q < ng; ++q) {
      GfPlan<T> &P = *all[i + q].P;
      auto &st = P.starts[all[i + q].k];
      LzJob<T> &J = *st.job;
      const long long n = J.s->dim;
      for (int b = 0; b < 3; ++b) J.buf[b] = DBuf(c->alloc, sizeof(T) * n);
      T *v0 = J.buf[0].template as<T>();
      if (st.kind == 0) {
        for (int q2 = 0; q2 < st.norb; ++q2)
          launch_a_adag<T>(st.from->template op<T>(), J.s->template op<T>(), st.orbs[q2] + st.spin * P.m->ns,
                           st.create ? 0 : 1, st.src, v0, q2 > 0 ? 1 : 0, c->stream);
      } else if (st.kind == 2) {
        bool first = true;
        for (int o = 0; o < st.norb; ++o) {
          if (st.w[o] == 0.0) continue;
          launch_a_adag<T>(st.from->template op<T>(), J.s->template op<T>(), o + st.spin * P.m->ns,
                           st.create ? 0 : 1, st.src, v0, first ? 0 : 1, c->stream, st.w[o]);
          first = false;
        }
        if (first) CK(cudaMemsetAsync(v0, 0, sizeof(T) * n, c->stream));
      } else {
        launch_diag_op<T>(st.from->template op<T>(), P.op, st.mu, st.nu, st.src, v0, c->stream);
      }
      launch_dot_partials<T>(v0, v0, n, parts.template as<double>() + 64 * q, 64, c->stream);
      launch_reduce(parts.template as<double>() + 64 * q, 64, norms.template as<double>() + q, c->stream);
    }
    std::vector<double> hn(ng);
    CK(cudaMemcpyAsync(hn.data(), norms.p, sizeof(double) * ng, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    std::vector<LzJob<T> *> run;
    for (size_t q = 0; q < ng; ++q) {
      GfPlan<T> &P = *all[i + q].P;
      const size_t k = all[i + q].k;
      P.hn[k] = hn[q];
      P.use[k] = !P.chi ? (std::fabs(hn[q]) > 1e-10) : (P.starts[k].local ? (hn[q] > 1e-9) : 1);
      if (!P.use[k]) continue;
      LzJob<T> &J = *P.starts[k].job;
      launch_scale<T>(J.buf[0].template as<T>(), J.s->dim, norms.template as<double>() + q, 1, c->stream);
      run.push_back(&J);
    }
    run_lanczos<T>(m0, run, p->nlanc, p->precision == EDGPU_MIXED);
    sync(c);
    if (take_mv_stall()) throw ApiError(EDGPU_ERR_CUDA, "a bulk copy into shared memory did not complete");
    for (size_t q = 0; q < ng; ++q)
      for (int b = 0; b < 3; ++b) all[i + q].P->starts[all[i + q].k].job->buf[b] = DBuf();
    i = j;
  }
}

template <typename T>
void plan_finish(GfPlan<T> &P, const edgpu_gf_params *p, double *G, double *Gij, double *Z_out) {
  edgpu_ctx *c = P.m->ctx;
  std::vector<CfJob> cf;
  for (size_t k = 0; k < P.starts.size(); ++k) {
    if (!P.use[k]) continue;
    LzJob<T> &J = *P.starts[k].job;
    CfJob jb;
    jb.alpha = J.alpha.template as<double>();
    jb.beta = J.beta.template as<double>();
    jb.state = J.state.template as<int>();
    jb.expectation = P.hn[k];
    jb.E = P.starts[k].E;
    jb.E0 = P.E0;
    jb.isign = P.starts[k].isign;
    jb.sym = P.chi ? 1 : 0;
    jb.out = P.starts[k].out;
    jb.out_stride = P.starts[k].stride;
    cf.push_back(jb);
  }
  DBuf dcf = upload(c, cf);
  DBuf cfres(c->alloc, sizeof(double2) * std::max<size_t>(1, cf.size() * (size_t)P.nw));
  launch_cf(dcf.template as<CfJob>(), (int)cf.size(), P.dom.template as<double>(), P.nw, p->beta,
            p->mesh == EDGPU_MESH_REAL, cfres.template as<double2>(), c->stream);
  DBuf ddiag = upload(c, P.diag), dpairs = upload(c, P.pairs);
  const int nw = P.nw, nint = P.nint, np = P.np;
  if (!P.chi) {
    if (!P.keep.empty()) {
      k_gf_finalize<<<(nw + 127) / 128, 128, 0, c->stream>>>(
          P.Gg.template as<double>(), P.Gl.template as<double>(), P.Ggij.template as<double>(), P.Glij.template as<double>(),
          P.Go.template as<double>(), P.Gijo.template as<double>(), nw, nint, P.Z, ddiag.template as<int>(),
          (int)P.diag.size(), dpairs.template as<int>(), np, 2); note_launch();
    } else {
      CK(cudaMemsetAsync(P.Go.p, 0, P.Go.bytes, c->stream));
      CK(cudaMemsetAsync(P.Gijo.p, 0, P.Gijo.bytes, c->stream));
    }
    CK(cudaGetLastError());
    if (G) CK(cudaMemcpyAsync(G, P.Go.p, sizeof(double) * P.n1, cudaMemcpyDeviceToHost, c->stream));
    if (Gij) CK(cudaMemcpyAsync(Gij, P.Gijo.p, sizeof(double) * P.n2, cudaMemcpyDeviceToHost, c->stream));
  } else {
    double *g = P.Gg.template as<double>(), *gij = P.Ggij.template as<double>();
    if (!P.keep.empty()) {
      k_div<<<(unsigned)((P.n1 + 255) / 256), 256, 0, c->stream>>>(g, (long long)P.n1, P.Z); note_launch();
      k_div<<<(unsigned)((P.n2 + 255) / 256), 256, 0, c->stream>>>(gij, (long long)P.n2, P.Z); note_launch();
      if (p->mesh != EDGPU_MESH_REAL) {  // zero-frequency sum rule: Matsubara mesh only (ChiLoc.h:358-390)
        for (int orb : P.diag)
          launch_chi_tail(g + 2 * orb, nint, nw, P.dom.template as<double>(), p->beta, P.avg, c->stream);
        for (int q = 0; q < np; ++q)
          launch_chi_tail(gij + 2 * ((long long)nint * P.pairs[2 * q] + P.pairs[2 * q + 1]), (long long)nint * nint, nw,
                          P.dom.template as<double>(), p->beta, P.avg, c->stream);
      }
      k_chi_combine<<<(nw + 127) / 128, 128, 0, c->stream>>>(g, gij, nw, nint, ddiag.template as<int>(), (int)P.diag.size(),
                                                             dpairs.template as<int>(), np); note_launch();
    }
    CK(cudaGetLastError());
    if (G) CK(cudaMemcpyAsync(G, g, sizeof(double) * P.n1, cudaMemcpyDeviceToHost, c->stream));
    if (Gij) CK(cudaMemcpyAsync(Gij, gij, sizeof(double) * P.n2, cudaMemcpyDeviceToHost, c->stream));
  }
  sync(c);
  if (Z_out) *Z_out = P.Z;
}

// G (chi == false) or chi_Op (chi == true) for `count` models: the recurrences of every model in
// memory-bounded batched groups, then the fractions.
template <typename T>
int gf_many_impl(edgpu_model *const *ms, int count, const edgpu_gf_params *p, bool chi, int op, const double *avg,
                 double *const *G, double *const *Gij, double *Z, const double *weights = nullptr, int nrows = 0) {
  if (count < 1) throw ApiError(EDGPU_ERR_ARG, "no models");
  edgpu_ctx *c = ms[0]->ctx;
  for (int q = 0; q < count; ++q)
    if (!ms[q] || ms[q]->ctx != c) throw ApiError(EDGPU_ERR_ARG, "models of one batch must share a context");
  // FP64 recurrences start from FP64 eigenvectors: kept pairs of an FP32 eigen-solve are continued in FP64 first
  int status = EDGPU_OK;
  if (sizeof(T) == 8) status = refine_kept(ms, count, p->beta, p->cutoff);
  std::vector<std::unique_ptr<GfPlan<T>>> plans;
  for (int q = 0; q < count; ++q) {
    plans.emplace_back(new GfPlan<T>());
    plan_prepare<T>(*plans.back(), ms[q], p, chi, op, avg ? avg[q] : 0.0, weights, nrows);
  }
  sync(c);
  run_starts<T>(plans, p, ms[0]);
  for (int q = 0; q < count; ++q)
    plan_finish<T>(*plans[q], p, G ? G[q] : nullptr, Gij ? Gij[q] : nullptr, Z ? Z + q : nullptr);
  return status;
}

template <typename T>
int gf_impl(edgpu_model *m, const edgpu_gf_params *p, double *G, double *Gij, double *Z_out) {
  return gf_many_impl<T>(&m, 1, p, false, 0, nullptr, &G, &Gij, Z_out);
}

template <typename T>
int chi_impl(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chiij, double *Z_out) {
  return gf_many_impl<T>(&m, 1, p, true, op, &avg, &chi, &chiij, Z_out);
}

int gf_many_dispatch(edgpu_model *const *ms, int count, const edgpu_gf_params *p, int chi, int op, const double *avg,
                     double *const *G, double *const *Gij, double *Z) {
  if (p->precision == EDGPU_FP32) return gf_many_impl<float>(ms, count, p, chi != 0, op, avg, G, Gij, Z);
  return gf_many_impl<double>(ms, count, p, chi != 0, op, avg, G, Gij, Z);
}

int gf_weighted_dispatch(edgpu_model *m, const edgpu_gf_params *p, const double *weights, int nrows, double *G,
                         double *Z) {
  if (p->precision == EDGPU_FP32) return gf_many_impl<float>(&m, 1, p, false, 0, nullptr, &G, nullptr, Z, weights, nrows);
  return gf_many_impl<double>(&m, 1, p, false, 0, nullptr, &G, nullptr, Z, weights, nrows);
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
