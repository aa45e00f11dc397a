/*
 * edgpu.h -- C ABI of the GB300 (sm_103a) exact-diagonalisation library (libedgpu.so).
 *
 * The reference's plug-in point for this path is its compile-time Storage concept
 * (EDLib::Storage::{CRSStorage, SpinResolvedStorage, SOCRSStorage}, used by
 * EDLib::Hamiltonian<Storage>, EDLib::gf::Lanczos / GreensFunction / ChiLoc).  Every entry point
 * below replaces one member of that concept or one driver routine built on it; each declaration
 * cites the reference interface it stands in for (paths relative to the reference project root).
 *
 * Conventions
 *  - Every function returns an int status: EDGPU_OK (0), a negative EDGPU_ERR_* code, or
 *    EDGPU_NOT_CONVERGED (+1, ARPACK's info = 1: results are kept).  edgpu_last_error() gives the
 *    message.  No function throws.
 *  - Plain pointers and sizes only.  "host" arrays are ordinary host memory; the library owns all
 *    device memory through the opaque handles.
 *  - A context serves one host thread at a time; all work of a context runs on its stream.
 *  - Sector vectors are indexed as in the reference: i = ninv[N_up][up] * C(Ns, N_dn) + ninv[N_dn][dn].
 *  - Precision: EDGPU_FP64 keeps every vector in FP64; EDGPU_FP32 keeps vectors in FP32 with FP64
 *    (float-float) dot products, FP64 projected matrices, Boltzmann weights and continued fractions.
 */
#ifndef EDGPU_H
#define EDGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDGPU_OK 0
#define EDGPU_NOT_CONVERGED 1
#define EDGPU_ERR_ARG (-1)
#define EDGPU_ERR_CUDA (-2)
#define EDGPU_ERR_CAPACITY (-3)  /* MAX_DIM / MAX_SIZE / HBM budget exceeded (reference: std::runtime_error) */
#define EDGPU_ERR_COLLISION (-4) /* SOCRS duplicate element (reference: std::logic_error "Collision") */
#define EDGPU_ERR_STATE (-5)     /* call order (e.g. Green's function before diag, EIGENVALUES_ONLY) */

#define EDGPU_CRS 0
#define EDGPU_SRS 1
#define EDGPU_SOCRS 2

#define EDGPU_FP64 0
#define EDGPU_FP32 1
#define EDGPU_MIXED 2 /* Hamiltonian::diag only: FP32 vectors with FP64 Rayleigh-Ritz eigenvalues (FP64 vectors
                         for sectors asking for more than 32 pairs or of at most ncv states); FP64 Green's
                         functions, susceptibilities and edgpu_refine_eigenpairs continue the Boltzmann-kept
                         FP32 pairs in FP64 */

#define EDGPU_OP_SZ 0
#define EDGPU_OP_N 1
#define EDGPU_MESH_MATSUBARA 0
#define EDGPU_MESH_REAL 1

typedef struct edgpu_ctx edgpu_ctx;
typedef struct edgpu_model edgpu_model;
typedef struct edgpu_server edgpu_server;

/* ---------------------------------------------------------------- context */
/* One GPU, one stream.  hbm_budget = 0: no limit beyond the device. */
int edgpu_ctx_create(edgpu_ctx **ctx, int device, size_t hbm_budget);
int edgpu_ctx_destroy(edgpu_ctx *ctx);
const char *edgpu_last_error(const edgpu_ctx *ctx);
/* Bytes of device memory currently held by the context (allocated and cached). */
size_t edgpu_ctx_device_bytes(const edgpu_ctx *ctx);
/* The context's cudaStream_t (as void *), for callers that time or order work around the library's. */
void *edgpu_ctx_stream(const edgpu_ctx *ctx);

/* ---------------------------------------------------------------- models */
/* Hubbard model, include/edlib/HubbardModel.h:48-77.
 * t[ns*ns] hopping (H = -sum t_ij c+_j c_i over |t_ij| > 1e-10), U[ns], xmu[ns] (entries 0 and 1 are
 * used, indexed by spin as in the reference), hmag[ns] or NULL, J[ns*ns] or NULL. */
int edgpu_model_hubbard(edgpu_ctx *ctx, int ns, const double *t, const double *U, const double *xmu,
                        const double *hmag, const double *J, edgpu_model **out);
/* Single-impurity Anderson model, include/edlib/SingleImpurityAndersonModel.h:195-275.
 * epsk[(ns-ml)*2], vk[ml*(ns-ml)*2], h0[ml*ml*2], mu, U[2*2*ml^4] (row-major as the HDF5 datasets). */
int edgpu_model_siam(edgpu_ctx *ctx, int ns, int ml, const double *epsk, const double *vk, const double *h0,
                     double mu, const double *U, edgpu_model **out);
int edgpu_model_destroy(edgpu_model *m);
/* Number of hopping (which = 0) / interaction (which = 1) transitions (Model::T_states / V_states). */
int edgpu_model_transitions(const edgpu_model *m, int which);

/* Storage limits (storage.MAX_DIM / storage.MAX_SIZE, include/edlib/EDParams.h:21-22); 0 = no limit.
 * Checked like CRSStorage::reset/addElement (CRSStorage.h:38-52, 200-204) and SOCRSStorage::reset
 * (SOCRSStorage.h:92-112). */
int edgpu_model_set_limits(edgpu_model *m, size_t max_dim, size_t max_size);

/* ---------------------------------------------------------------- symmetry tables */
/* C(n, k) of SzSymmetry::comb() (Combination.h:13-78). */
long long edgpu_binom(const edgpu_model *m, int n, int k);
/* Device-built basis[k][r] masks (SzSymmetry.h:191-216), copied to host out[C(ns,k)]. */
int edgpu_basis(edgpu_model *m, int k, int *out);
/* Device-built ninv[k][mask] (SzSymmetry.h:123-133), copied to host out[2^ns]. */
int edgpu_ninv(edgpu_model *m, int k, int *out);
/* Sector iteration order of SzSymmetry (SzSymmetry.h:72-98): list == NULL for all (N_up, N_dn), or
 * n_in pairs.  out receives 2 ints per sector; returns the count through *n_out. */
int edgpu_sector_order(const edgpu_model *m, const int *list, int n_in, int *out, int *n_out);

/* ---------------------------------------------------------------- Storage concept */
/* Storage::fill for sector (N_up, N_dn) with the given storage (CRSStorage.h:66-83,
 * SpinResolvedStorage.h:120-155, SOCRSStorage.h:114-160); *dim receives ntot. */
int edgpu_fill(edgpu_model *m, int storage, int nup, int ndn, long long *dim);
/* Storage::av(v, w, n, clear) on host FP64 arrays of the current fill (CRSStorage.h:57-64,
 * SpinResolvedStorage.h:58-115, SOCRSStorage.h:46-87).  prec selects the device arithmetic. */
int edgpu_av(edgpu_model *m, const double *v, double *w, long long n, int clear, int prec);
/* Storage::av (CRSStorage.h:57-64, SpinResolvedStorage.h:58-115, SOCRSStorage.h:46-87) on caller-owned DEVICE
 * vectors, stream-ordered: for q < nvec, y_q = H x_q (accumulate = 0, the reference's clear = true) or
 * y_q += H x_q (accumulate = 1), with x_q = x + q * ldx and y_q = y + q * ldx (elements of the precision
 * prec: FP64 double, FP32 float; ldx >= the sector dimension).  The work is enqueued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) and the call returns without waiting for it; the sector's
 * tables are built on first use (synchronously on the context's stream).  x and y must not overlap. */
int edgpu_spmv(edgpu_model *m, int storage, int nup, int ndn, const void *x, void *y, int nvec, long long ldx, int prec,
               int accumulate, void *stream);
/* Storage::a_adag (CRSStorage.h:131-145, SpinResolvedStorage.h:293-381): out[index(c_i^(+) s)] = sign * in[s]
 * from sector (nup, ndn) into (tnup, tndn); spin_orbital = orbital + spin * ns. */
int edgpu_a_adag(edgpu_model *m, int spin_orbital, int nup, int ndn, int tnup, int tndn, const double *in,
                 double *out, int annihilate);
/* Storage::vv (CRSStorage.h:123-129): FP64 dot product (device, fixed-order reduction). */
int edgpu_vv(edgpu_model *m, const double *v, const double *w, long long n, double *out);

/* ---------------------------------------------------------------- Hamiltonian::diag */
typedef struct {
  int storage;           /* EDGPU_CRS / EDGPU_SRS / EDGPU_SOCRS */
  int precision;         /* EDGPU_FP64 / EDGPU_FP32 / EDGPU_MIXED */
  int nev;               /* arpack.NEV */
  int ncv;               /* arpack.NCV, 0 = 2*nev+3 (Storage.h:26-30) */
  int eigenvalues_only;  /* storage.EIGENVALUES_ONLY */
  double tol;            /* relative residual tolerance, 0 = default (1e-12 FP64, 2e-6 FP32 + FP64 refinement) */
  int maxitr;            /* restart cycles, 0 = 1000 (Storage.h:65) */
  const int *sectors;    /* NULL: all sectors; else n_sectors (N_up, N_dn) pairs (arpack.SECTOR) */
  int n_sectors;
  int multiplicity_check;  /* 0: after convergence, restart from a fresh random vector deflated against the
                              converged pairs and run until nev + 1 pairs converge, keeping any copy of a
                              degenerate eigenvalue a single-vector Krylov space misses (the multiplicities
                              of dense LAPACK); 1: no check; c >= 2: the check gets c - 1 restart cycles */
  int max_batch;         /* sectors solved together in one lock-step batch of launches: 0 = as many as fit
                            (every sector of every model of the call), 1 = one sector at a time (the
                            reference's loop order, Hamiltonian.h:66-86); results do not depend on it */
} edgpu_diag_params;

/* Hamiltonian::diag (Hamiltonian.h:54-101 with Storage::diag, Storage.h:43-146): every sector in the
 * reference order, nev = min(NEV, ncv-1), ncv = min(NCV, dim), dim 1 -> (H_00, [1]).  Eigen-pairs are
 * kept on the device, ordered ascending with ties in insertion order (the std::set<EigenPair> order). */
int edgpu_diag(edgpu_model *m, const edgpu_diag_params *p, int *npairs);
/* Hamiltonian::diag for `count` models of one context at once (independent impurity or cluster solves):
 * every sector of every model shares the batched eigen-solver launches; each model then holds its own
 * eigen-pairs exactly as after edgpu_diag.  npairs[count] receives the per-model counts. */
int edgpu_diag_many(edgpu_model *const *models, int count, const edgpu_diag_params *p, int *npairs);
/* Storage::diag for the single sector (nup, ndn) (Storage.h:43-146): up to nev eigenvalues ascending in
 * evals[], their count in *nconv, and -- unless evecs is NULL -- the Ritz vectors as FP64 host columns
 * evecs[q * ldv + i].  Returns EDGPU_NOT_CONVERGED when maxitr restart cycles were not enough (the
 * converged pairs are still returned, as the reference keeps ARPACK's info = 1 results). */
int edgpu_diag_sector(edgpu_model *m, const edgpu_diag_params *p, int nup, int ndn, double *evals, int *nconv,
                      double *evecs, long long ldv);
/* evals[npairs], sectors[2*npairs] (N_up, N_dn), ids[npairs] (insertion ids); any may be NULL. */
int edgpu_eigenpairs(const edgpu_model *m, double *evals, int *sectors, int *ids, int max_pairs);
/* EigenPair::eigenvector (EigenPair.h:31-33): copy pair `index` (sorted order) to host FP64 out[n]. */
int edgpu_eigenvector(edgpu_model *m, int index, double *out, long long n);

/* ---------------------------------------------------------------- Green's functions */
typedef struct {
  double beta;           /* lanc.BETA */
  int nomega;            /* lanc.NOMEGA */
  int nlanc;             /* lanc.NLANC */
  double cutoff;         /* lanc.BOLTZMANN_CUTOFF */
  int precision;         /* EDGPU_FP64 / EDGPU_FP32 Lanczos vectors; EDGPU_MIXED: FP64 start vectors (kept FP32
                            pairs continued in FP64 first), recurrences on float-float vectors (pairs of FP32
                            values, about 2^-48 relative; GB300 issues FP64 at 1/64 of its FP32 rate) for
                            spin-resolved sectors, FP64 for the other storages */
  const int *orbitals;   /* GreensFunction_orbitals / ChiLoc_orbitals pairs, NULL = all diagonal */
  int n_orbitals;
  int max_batch;         /* Lanczos recurrences advanced together per launch: 0 = all of the call, 1 = one
                            start vector at a time (the reference's loop order); results do not depend on it */
  int mesh;              /* EDGPU_MESH_MATSUBARA (MatsubaraMeshFactory) or EDGPU_MESH_REAL
                            (RealFreqMeshFactory: nomega points EMIN..EMAX, evaluated at w + i pi / beta) */
  double emin, emax;     /* lanc.EMIN, lanc.EMAX of the real mesh */
} edgpu_gf_params;

/* GreensFunction::compute (GreensFunction.h:109-159) on the Matsubara mesh w_n = (2n+1) pi / beta.
 * G[nomega][n_int_orb][2] and G_ij[nomega][n_int_orb^2][2] complex (re, im interleaved, may be NULL),
 * *Z = statistical sum. */
int edgpu_greens_function(edgpu_model *m, const edgpu_gf_params *p, double *G, double *G_ij, double *Z);
/* Green's functions of orbital combinations c_w = sum_j w_j c_j, one per row of weights[nrows][n_int_orb]:
 * start vectors sum_j w_j c+_j|n> and sum_j w_j c_j|n> per spin, the same recurrences and fractions as
 * GreensFunction::compute; G[nomega][nrows][2] complex, *Z.  For a translation-invariant cluster the rows
 * cos(k r_j) and sin(k r_j) give G(k) = (G_cos + G_sin) / N with 4 start vectors per spin instead of the
 * 2N - 1 orbital pairs of the reference's route (G_0j through GreensFunction_orbitals, then a Fourier sum).
 * No counterpart in the reference. */
int edgpu_greens_function_weighted(edgpu_model *m, const edgpu_gf_params *p, const double *weights, int nrows,
                                   double *G, double *Z);
/* GreensFunction::compute_selfenergy (GreensFunction.h:202-222): the model's bare Green's function G0
 * (HubbardModel.h:180-201; SingleImpurityAndersonModel.h:377-391, diagonal over the impurity orbitals) and
 * Sigma = G0^-1 - G_ij^-1 per frequency and spin (FermionicModel::solve_dyson, FermionicModel.h:83-108) on
 * the mesh p describes (beta, nomega, mesh, emin, emax are read).  G_ij[nomega][n_int_orb^2][2] complex as
 * edgpu_greens_function returns it; G0 and Sigma (either may be NULL) in the same layout.  A singular G_ij
 * (an orbital left out of GreensFunction_orbitals) is EDGPU_ERR_ARG. */
int edgpu_self_energy(edgpu_model *m, const edgpu_gf_params *p, const double *G_ij, double *G0, double *Sigma);
/* ChiLoc::compute<Op> (ChiLoc.h:180-233) on W_n = 2n pi / beta, op = EDGPU_OP_SZ / EDGPU_OP_N, avg =
 * operator average for the zero-frequency correction.  chi[nomega][n_int_orb], chi_ij[nomega][n_int_orb^2]. */
int edgpu_chiloc(edgpu_model *m, const edgpu_gf_params *p, int op, double avg, double *chi, double *chi_ij,
                 double *Z);
/* GreensFunction::compute for `count` models at once (all recurrences in one batched Lanczos run);
 * G[q] / G_ij[q] are the per-model outputs (entries may be NULL), Z[count]. */
int edgpu_greens_function_many(edgpu_model *const *models, int count, const edgpu_gf_params *p, double *const *G,
                               double *const *G_ij, double *Z);
/* ChiLoc::compute<Op> for `count` models at once; avg[count] operator averages. */
int edgpu_chiloc_many(edgpu_model *const *models, int count, const edgpu_gf_params *p, int op, const double *avg,
                      double *const *chi, double *const *chi_ij, double *Z);
/* FP64 continuation of an FP32 Hamiltonian::diag for the eigen-pairs a Boltzmann average at inverse temperature
 * beta keeps (weight exp(-beta (E - E0)) not below cutoff, GreensFunction.h:125-140), for `count` models of one
 * context at once.  An FP32 Ritz vector is accurate to about 1e-6, and G, chi and the static observables
 * inherit that at first order.  Each sector holding kept FP32 pairs runs its eigen-solve again in FP64,
 * started from a combination of its FP32 Ritz vectors (a degenerate eigenvalue from as many combinations as
 * its multiplicity); the kept pairs then hold FP64 eigenvectors, their eigenvalues and order unchanged.  The
 * FP64 Green's-function and susceptibility entry points do this themselves before their recurrences.
 * Returns EDGPU_NOT_CONVERGED when a sector's continuation did not converge (its pairs keep their FP32
 * vectors).  No counterpart in the reference (its ARPACK runs in one precision). */
int edgpu_refine_eigenpairs(edgpu_model *const *models, int count, double beta, double cutoff);
/* StaticObservables::calculate_static_observables (StaticObservables.h:106-158): Boltzmann averages over
 * the kept eigen-pairs.  n, n_up, n_dn, m, d_occ [n_int_orb]; mimj [n_int_orb^2]; n_eff, energy scalars. */
int edgpu_static_observables(edgpu_model *m, double beta, double cutoff, double *n, double *n_up, double *n_dn,
                             double *mag, double *d_occ, double *mimj, double *n_eff, double *energy);

/* The eigen-step operator variant the library's tuner chose for the model's first eigen batch (every
 * variant timed on the batch's own SRS sectors when the batch is built): resident blocks per SM (2 or 3) and
 * whether long rows stage their up-spin source rows in shared memory; *ms = the chosen variant's time per
 * operator launch, -1 when not tuned (no batch yet, no SRS storage, or EDGPU_OP_TUNE=0).  Every variant
 * computes the same sums in the same order.  No counterpart in the reference. */
int edgpu_operator_tuning(const edgpu_model *m, int prec, int *blocks_per_sm, int *staged, double *ms);

/* ---------------------------------------------------------------- device-level entry points */
/* Plain Lanczos recurrence of Lanczos::lanczos (Lanczos.h:36-77) for `count` normalised start vectors
 * given on the host (FP64), all in sector (nup, ndn) of the current storage: alpha[count][nlanc],
 * beta[count][nlanc+1], nl[count]. */
int edgpu_lanczos(edgpu_model *m, int storage, int nup, int ndn, const double *starts, int count, int nlanc,
                  int prec, double *alpha, double *beta, int *nl);
/* get_frac_point (Lanczos.h:201-224) for nz complex energies (re, im interleaved): out[nz] complex. */
int edgpu_frac_points(edgpu_ctx *ctx, const double *alpha, const double *beta, int nlanc, int isign,
                      double expectation, double expb, const double *ener, int nz, double *out);

/* ---------------------------------------------------------------- serving (continuous batching)
 * A request loop on one context (no counterpart in the reference, whose drivers solve one model at a time):
 * impurity / cluster solves of any size queue up; edgpu_server_step admits them in arrival order while
 * their eigen-solver footprint fits the device-memory budget, and their sectors join the running lock-step
 * eigen-solver batch between restart cycles, leaving it as they converge; a request's Green's function runs
 * as soon as its spectrum is complete.  Each result is the same as the request solved alone.  Single host
 * thread, like the reference's API.  hbm_budget = 0: 80 % of the free device memory at creation.  precision:
 * EDGPU_FP32, EDGPU_FP64, or EDGPU_MIXED (sectors routed as edgpu_diag routes them in that precision). */
int edgpu_server_create(edgpu_ctx *ctx, int precision, size_t hbm_budget, edgpu_server **out);
int edgpu_server_destroy(edgpu_server *s);
/* Queue Hamiltonian::diag of model m (created on the server's context; dp as for edgpu_diag, precision =
 * the server's, ncv <= 64) and, when gp != NULL, GreensFunction::compute into the caller's host arrays G,
 * G_ij, *Z (shapes of edgpu_greens_function; they must stay valid until the request is done). */
int edgpu_server_submit(edgpu_server *s, edgpu_model *m, const edgpu_diag_params *dp, const edgpu_gf_params *gp,
                        double *G, double *G_ij, double *Z, long long *ticket);
/* One scheduling round: admission, one restart cycle of every admitted sector, eigen-pairs of the requests
 * whose sectors all converged, their Green's functions.  *running / *queued: requests in each state. */
int edgpu_server_step(edgpu_server *s, int *running, int *queued);
/* *state: 0 queued, 1 running, 2 done (the model holds its *npairs eigen-pairs, G written), < 0 failed. */
int edgpu_server_poll(edgpu_server *s, long long ticket, int *state, int *npairs);

/* Batched Hamiltonian-times-vector throughput probe: `nvec` independent vectors of sector (nup, ndn)
 * in one launch (the batched form the Lanczos recurrences use), `reps` timed launches after two
 * warm-up launches, CUDA events on the context's stream.  Returns the mean launch time and the
 * algorithmic bytes of one launch (x read and y written per vector, the shared diagonal once). */
int edgpu_bench_spmv(edgpu_model *m, int storage, int nup, int ndn, int nvec, int prec, int reps,
                     double *ms_per_launch, double *bytes_per_launch);
/* Throughput probe of the Hamiltonian-times-vector as one eigen-solver step of Hamiltonian::diag launches it
 * for `count` models at once: one vector of every sector (more than one state) of every model, all in one
 * launch of the operator (the model's tuned variant), `reps` timed launches after two warm-up launches, CUDA
 * events on the context's stream.  Returns the mean launch time, the algorithmic bytes of one launch (per
 * sector: x read, y written and the diagonal read, states x element size each) and the states covered.  No
 * counterpart in the reference (it measures this library's kernel). */
int edgpu_bench_spmv_batch(edgpu_model *const *models, int count, int storage, int prec, int reps, double *ms_per_launch,
                           double *bytes_per_launch, long long *states);
/* Throughput probe of the eigen-solver's two Gram-Schmidt passes (the dominant kernels of a solve):
 * `ntasks` independent bases of `nbasis` columns of sector (nup, ndn) filled with seeded values, one
 * dot pass (s = V^T w, g = V^T V[j]) and one update pass (w -= V h) per round, `reps` timed rounds after
 * two untimed ones, CUDA events on the context's stream around each pass.  Returns the mean time of each
 * pass and its algorithmic bytes: (nbasis + 1) x states x element size per task for the dot pass (the
 * columns and w), (nbasis + 2) x ... for the update (the columns, w read and written).  No counterpart in
 * the reference (it measures this library's kernels). */
int edgpu_bench_cgs(edgpu_model *m, int storage, int nup, int ndn, int nbasis, int ntasks, int prec, int reps,
                    double *ms_dot, double *ms_upd, double *bytes_dot, double *bytes_upd);
/* <v, w> of caller-owned FP64 device arrays, written to the device scalar *out, enqueued on `stream`
 * (a cudaStream_t; NULL = the legacy default stream).  Unlike every other entry point this one
 * allocates nothing -- no cudaMalloc, cudaFree or allocating library call -- for callers that cannot
 * allocate device memory (a serving loop held to a fixed memory budget, stream-ordered code that cannot
 * take the device synchronisation an allocation may cause).  No counterpart in the reference: it is the
 * device-pointer form of Storage::vv.  Its partial sums live in a 16 KiB static device array that every
 * GPU loading the library keeps until exit; the first call on a device looks that array up (make it
 * before any stream capture).  All calls on a device share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.  n above EDGPU_VV_NOALLOC_MAX_N is rejected with
 * EDGPU_ERR_CAPACITY before any work is enqueued. */
#define EDGPU_VV_NOALLOC_MAX_N 8388608LL
int edgpu_vv_noalloc(const double *v, const double *w, long long n, double *out, void *stream);

/* Number of kernels launched by this library in the calling process so far. */
long long edgpu_launch_count(void);

/* Self-test of the device-side failure path (no counterpart in the reference): one block waits on a
 * bulk-copy barrier that no copy completes, `rounds` try_wait rounds (1 .. 2^22) twice, as the operator
 * kernels do for a copy that does not arrive.  *gave_up = 1 when the kernel's waits gave up and it
 * returned; *flagged = 1 when the stall flag the library checks after every batch step was set (and is
 * now cleared).  The context stays usable.
 * The stall flags are per device, not per context: every context on a device reads and clears the same
 * flags after its batch steps.  Run this self-test only while no other work of the library is in flight on
 * the device, or another context may take its flag (and fail a healthy step) or it may take another's. */
int edgpu_selftest_bulk_wait(edgpu_ctx *ctx, int rounds, int *gave_up, int *flagged);

/* Counters since the last diag: operator applications issued, Lanczos steps, restart cycles, and
 * element-steps (sum over operator applications of the sector dimension). */
int edgpu_stats(const edgpu_model *m, long long *spmv_vectors, long long *lanczos_steps, long long *restarts,
                double *element_steps);

#ifdef __cplusplus
}
#endif

#endif /* EDGPU_H */
