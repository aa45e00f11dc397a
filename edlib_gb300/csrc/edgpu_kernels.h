// Host-side declarations shared by the library's translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "edgpu_internal.cuh"

namespace edgpu {

// Number of kernels this library has launched in the process (every launch site increments it).
long long launch_count();
// Persistent grid: as many blocks of `fn` (block threads, smem dynamic bytes) as are resident on the
// current GPU at once -- one wave, blocks walk their work in a grid-stride loop -- but never more than
// `nitems`.  Cached per (device, kernel, shared memory).
int occupancy_grid(const void *fn, int block, size_t smem, int nitems);
void note_launch(long long n = 1);

inline long long binom_at_host(int n, int k) {
  if (n < 0 || k < 0 || k > n) return 0;
  long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

// Caching device allocator of a context: blocks are kept per size after free and reused, so the
// steady state of a solve performs no cudaMalloc.  Tracks the bytes held against an HBM budget.
class DeviceAllocator {
 public:
  void *alloc(size_t bytes);
  void free(void *p);
  void release_all();
  size_t in_use() const { return in_use_; }
  size_t held() const { return held_; }
  size_t budget = 0;  // 0 = unlimited
  std::string last_error;

 private:
  std::multimap<size_t, void *> free_;
  std::map<void *, size_t> live_;
  size_t in_use_ = 0, held_ = 0;
};

// items: every operator kernel walks a sector in "items" (row groups) so that batches of uneven
// sectors share one launch and per-item partial sums are reduced in a fixed order.
constexpr int kItemElems = 2048;  // target vector elements per item

template <typename T>
struct SectorItems {
  int nitems;
  int srs_rows;  // SRS: up-rows per item
};

// ---- tables.cu
void build_tables(const DevModel &m, long long *basis_off_host, int *basis, int *ninv, cudaStream_t st);
long long scan_tmp_size(long long n);
void exclusive_scan(const long long *in, long long *out, long long n, long long *tmp, cudaStream_t st);
void launch_spin_csr(const DevModel &m, int spin, int k, long long rows, const int *basis_k, long long *count,
                     long long *rp, long long *scan_tmp, int *rp32, int **col, double **val64, float **val32,
                     long long *nnz_out, int *err, DeviceAllocator &alloc, cudaStream_t st);
// k-major ("ELL") copy of a per-spin CSR: len[d], col/val[k * ld + d]; the padding stays as memset (0)
void launch_spin_ell(const int *rp, const int *col, const double *v64, const float *v32, int rows, int ld, int *len,
                     int *ell_col, double *ell_v64, float *ell_v32, cudaStream_t st);
void launch_crs(const DevModel &m, const SectorOp<double> &op, long long *count, long long *rp, long long *scan_tmp,
                int **col, double **val64, float **val32, long long *nnz_out, int *err, DeviceAllocator &alloc,
                cudaStream_t st);
void launch_diag(const DevModel &m, const SectorOp<double> &op, double *d64, float *d32, cudaStream_t st);
void launch_socrs_check(const DevModel &m, const SectorOp<double> &op, int *err, cudaStream_t st);

// ---- spmv.cu / krylov.cu : batched operator kernels
// Element range of item li of a sector operator.
// SRS sectors whose rows (down-spin dimension) are at least this long are swept by thread-per-column
// tiles of several rows; shorter rows are spread flat over the block.
constexpr int kSrsLongRow = 128;
// Up-spin rows per SRS work item: long rows are swept in groups of 4 rows, about 8192 elements per item
// (EDGPU_SRS_ITEM_ELEMS; at most 24576, as many rows as fit 96 KB of FP32, so that they still stage in
// shared memory; rows longer than 6144 elements one or a few per item); short rows take about kItemElems
// elements per item.  Measured on Anderson-12 (FP32 eigen-solve of all sectors): 0.575 s with 4096, 0.531 s
// with 8192, 0.543 s with 16384, 0.595 s with 2048 elements per item.
inline int srs_item_rows(int up_rows, int dn_rows) {
  static const int target = [] {  // elements per item of long rows (EDGPU_SRS_ITEM_ELEMS, for measurements)
    const char *e = getenv("EDGPU_SRS_ITEM_ELEMS");
    const int v = e ? atoi(e) : 0;
    return v >= 512 && v <= 24576 ? v : 8192;  // 8192: 8 % less eigen-solve time than 4096 on Anderson-12
  }();
  int r;
  if (dn_rows >= kSrsLongRow && 4 * dn_rows <= 24576) r = std::max(4, std::min(24576 / dn_rows, target / dn_rows) & ~3);
  else if (dn_rows >= kSrsLongRow) r = std::max(1, 24576 / dn_rows);  // very long rows: as many as stage in 96 KB
  else r = kItemElems / std::max(1, dn_rows);
  return std::max(1, std::min(r, up_rows));
}

template <typename T>
__host__ __device__ inline void item_range(const SectorOp<T> &op, int srs_rows, long long li, long long &lo, long long &hi) {
  if (op.storage == kSRS) {
    long long u0 = li * srs_rows;
    long long u1 = u0 + srs_rows;
    if (u1 > op.up_rows) u1 = op.up_rows;
    lo = u0 * op.dn_rows;
    hi = u1 * op.dn_rows;
  } else {
    lo = li * (long long)kItemElems;
    hi = lo + kItemElems;
    if (hi > op.dim) hi = op.dim;
  }
}

// One Hamiltonian-times-vector work unit of a batch: y = H x (+ c z), optional per-item <x,y>.
template <typename T>
struct MvTask {
  const SectorOp<T> *op;  // device pointer
  int srs_rows;
  int item_begin;
  const T *x;
  T *y;
  const T *z;
  double c;
  double *dot_partial;  // [nitems] or null
};

// Plain Lanczos recurrence (include/edlib/Lanczos.h:36-77) over rotating buffers.
template <typename T>
struct LzTask {
  const SectorOp<T> *op;
  int srs_rows;
  int item_begin;
  int nitems;
  T *buf[3];
  double *alpha;      // [nlanc]
  double *beta;       // [nlanc + 1]
  double *part_a;     // [nitems]
  double *part_b;     // [nitems]
  double *scal;       // [0] alf, [1] bet
  int *state;         // [0] done, [1] nlanc
  int nlanc_max;
};

// Restarted Lanczos eigen-solver task with full classical Gram-Schmidt (twice).
#ifndef EDGPU_SRS_STAGE_KB
// shared memory an SRS item may use for its up-spin source rows staged by bulk copies.  0 (the default):
// the hops gather the source rows from L2, which measured 3-5 % faster on GB300 than staging them (112)
#define EDGPU_SRS_STAGE_KB 0
#endif
#ifndef EDGPU_CGS_CHUNK
#define EDGPU_CGS_CHUNK 4096
#endif
#ifndef EDGPU_CGS_STAGES
#define EDGPU_CGS_STAGES 4  // shared-memory stages of the FP32 Gram-Schmidt slice stream
#endif
#ifndef EDGPU_CGS_MIN_BLOCKS
#define EDGPU_CGS_MIN_BLOCKS 2
#endif
constexpr int kCgsChunk = EDGPU_CGS_CHUNK;  // vector elements per Gram-Schmidt chunk
constexpr int kCgsSup = 64;                  // chunks per split of the dot pass's partials reduction
__host__ __device__ inline int cgs_nsup(int nchunks) { return (nchunks + kCgsSup - 1) / kCgsSup; }
constexpr int kMaxLd = 128;      // largest projected-matrix dimension (ncv + 1)
constexpr int kGramPairs = 64 * 65 / 2;  // pairs of a restart Gram block: basis of at most 64 vectors
constexpr int kGramSmem = 64 * 1024;         // shared memory of one Gram slice
constexpr int kEigDone = -0x40000000;  // restart code of a finished sector (k_eig_reset)

template <typename T>
struct EigTask {
  const SectorOp<T> *op;
  int srs_rows;
  int item_begin;
  int nitems;
  int chunk_begin;   // first entry of this task in the chunk map
  int nchunks;       // ceil(n / kCgsChunk)
  long long n;
  long long ldv;     // column stride of V (n rounded up to 16 bytes)
  int m;             // basis vectors before a restart (ncv, clamped to n)
  int ld;            // leading dimension of Tm (mmax + 1)
  T *V;              // (m + 1) columns, ldv apart
  T *w;              // ldv
  double *Tm;        // ld x ld column-major projected matrix
  double *hpart;     // [nchunks][ld] partials of s = V^T w
  double *hpart2;    // [nchunks][ld] partials of g = V^T V[j]
  double *spart;     // [nsup][2 ld + 2] superchunk sums of s, g and |w|^2 (kCgsSup chunks each)
  double *hv;        // [ld] projection coefficients h = (I - E) s of the step
  int *ord;          // [ld + 1] update order: [0] columns subtracted exactly, then the column indices
  int *cnt;          // [nsup + 1] arrival counters of the dot reduction, zero between launches
  double *npart;     // [2][nchunks] |w|^2 before and after the projection
  double *E;         // ld x ld Gram deviation V^T V - I of the basis (column-major)
  double *gpart;     // [nchunks][gstride] partial Gram blocks after a restart
  int gstride;       // (m + 1)(m + 2) / 2: pairs of the largest basis
  double *nsc;       // [1] beta of the last step
  // st: [0] basis size j + 1 so far (-1 before the first vector), [1] mode (0 Lanczos, 1 orthogonalising a
  // random vector), [2] not growing (basis full or given up), [3] random draws, [4] action of the last
  // step (0 none, 1 accept w, 2 draw), [5] sector finished
  int *st;
  unsigned long long seed;
  const T *start;    // first basis vector (before orthogonalisation); nullptr: a seeded random vector
};

// FP64 Rayleigh-Ritz refinement of k FP32 Ritz vectors of one sector (items of kItemElems elements)
struct RrTask {
  long long n;
  int k;             // <= 32
  int item_begin, nitems;
  const double *X;   // k x n
  const double *W;   // k x n, H X
  double *part;      // [nitems][2 k k]
  double *theta;     // [k]
  double *Y;         // [k][k], column i = coefficients of refined vector i
  float *out;        // k x n refined vectors
  int *status;       // [1] 0 ok, 1 Gram matrix not positive definite
};
void launch_rr(const RrTask *tasks_dev, const int *item_task_dev, int nitems, int ntasks, double *work, cudaStream_t st);

// Shared-memory shape of an operator launch (all tasks of a launch share one storage kind):
// xs_elems vector elements for the staged rows of an item; plain = 1 when no task of a launch_mv has a
// z term or wants dot products.
struct MvShape {
  int storage;
  int xs_elems;       // staging elements of an item's own rows
  int plain = 0;
  int xs_staged = 0;  // with the up-spin source rows of long SRS rows beside them (0: never fits)
  int staged = 0;     // stage the source rows (1) or gather them from L2 (0)
  int mb = 2;         // resident blocks per SM of the eigen-step operator kernel: 2 or 3 (plain launches: 3)
};
// Operator variants the tuner chooses between for the eigen step (spmv.cu, tune_eig_mv): blocks per SM
// {2, 3} x source-row staging {off, on}; all compute the same sums in the same order, so the choice
// changes speed only.
struct OpTuning {
  int mb = 2, staged = 0;
  double ms = 0.0;  // time of the chosen variant on the tuning launch
  bool done = false;
};

template <typename T>
void launch_mv(const MvTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, cudaStream_t st);

// True (and cleared) when an operator kernel gave up waiting for a bulk copy into shared memory.
bool take_mv_stall();
// One block that waits (bounded) on a bulk-copy barrier no copy completes: *gave_up_dev = 1 when both waits
// gave up (spmv.cu, k_wait_selftest).
void launch_wait_selftest(int rounds, int *gave_up_dev, cudaStream_t st);
// true (and cleared) when a bounded wait of the Gram-Schmidt dot pass gave up on a bulk copy
bool take_cgs_stall();
template <typename T>
void launch_lz_mv(const LzTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int it, MvShape sh,
                  cudaStream_t st);
template <typename T>
void launch_eig_mv(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, cudaStream_t st,
                   T *probe_y = nullptr);
// The operator tuner on an eigen-step batch: every variant timed on the batch's own tasks (probe mode: x =
// V[0] of every task, into the scratch probe_y of the largest task's length); returns the fastest.
template <typename T>
OpTuning tune_eig_mv(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, T *probe_y,
                     cudaStream_t st);
template <typename T>
void launch_lz_step(const LzTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int ntasks, int it,
                    MvShape sh, cudaStream_t st);
// Kernel attributes the step kernels need for this shape; call before launch_eig_step (and before a
// step is captured into a graph).
template <typename T>
void prepare_eig_step(MvShape sh);
template <typename T>
void prepare_eig_mv(MvShape sh);
template <typename T>
void launch_eig_step(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, const int *chunk_task_dev,
                     int nchunks, const int *leaders_dev, int nleaders, int ntasks, MvShape sh, cudaStream_t st);
template <typename T>
void launch_eig_jacobi(const EigTask<T> *tasks_dev, int ntasks, double *theta, double *Y, double *resid, int ld,
                       double *work, int *status, cudaStream_t st);
template <typename T>
void launch_eig_restart(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, const int *keep,
                        const double *Y, int ld, T *const *outV, cudaStream_t st);

template <typename T>
void launch_eig_reset(const EigTask<T> *tasks_dev, int ntasks, const int *rk, const double *theta, int ld,
                      cudaStream_t st);

// Fresh deterministic random vector in w of every task in restart mode (w <- hash(seed, draw, i) - 0.5)
template <typename T>
void launch_eig_random(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st);
// out[i] = sum_q coef[q] * vecs[q][i], i < n, vecs[q] FP64 where is64[q] else FP32 (Ritz vectors -> one FP64 vector)
void launch_seed_combine(const void *const *vecs, const int *is64, const double *coef, int k, long long n, double *out,
                         cudaStream_t st);
// y -= c[0] * x (c a device scalar)
void launch_axpy_dev(double *y, const double *x, const double *c, long long n, cudaStream_t st);
// The two Gram-Schmidt passes of an eigen-solver step on their own (launch_eig_step runs them).
template <typename T>
void launch_cgs_dot(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st);
// kernel attributes of launch_cgs_dot (its staging buffers); call once before launching or capturing it
template <typename T>
void prepare_cgs();
template <typename T>
void launch_cgs_upd(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st);
// between the two: the chunk partials of the dot pass reduced per task and the projection coefficients
template <typename T>
// leaders_dev: the chunk indices (into chunk_task_dev) whose chunk starts a split of kCgsSup chunks of its task
void launch_cgs_coef(const EigTask<T> *tasks_dev, const int *chunk_task_dev, const int *leaders_dev, int nleaders,
                     cudaStream_t st);
// Gram block of every restarted task's basis (rk[b] != 0, != kEigDone) into EigTask::E.
template <typename T>
void launch_eig_gram(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, int ntasks, const int *rk,
                     cudaStream_t st);
// The same Gram block from the old one and the restart's Y (before launch_eig_reset); see k_eig_gram_proj.
template <typename T>
void launch_eig_gram_proj(const EigTask<T> *tasks_dev, int ntasks, const int *rk, const double *Y, int ld,
                          cudaStream_t st);

// a / a+ (gather form), diagonal operators, dot products, scaling, continued fraction
template <typename T>
void launch_a_adag(const SectorOp<T> &src, const SectorOp<T> &dst, int im, int annihilate, const T *in, T *out,
                   int accumulate, cudaStream_t st, double weight = 1.0);
template <typename T>
void launch_diag_op(const SectorOp<T> &op, int opkind, int mu, int nu, const T *in, T *out, cudaStream_t st);
template <typename T>
void launch_dot_partials(const T *a, const T *b, long long n, double *partial, int nparts, cudaStream_t st);
void launch_reduce(const double *partial, int nparts, double *out, cudaStream_t st);
template <typename T>
void launch_scale(T *x, long long n, const double *norm2, int divide_sqrt, cudaStream_t st);
template <typename T>
void launch_convert(const double *in, T *out, long long n, cudaStream_t st);
template <typename T>
void launch_to_double(const T *in, double *out, long long n, cudaStream_t st);

struct CfJob {
  const double *alpha;
  const double *beta;
  const int *state;     // [1] = nlanc
  double expectation;   // <n|O+O|n>
  double E, E0;
  int isign;
  int sym;              // 0: fermionic fraction; 1: symmetrised bosonic fraction
  double *out;          // complex (re, im) output array base
  long long out_stride; // complex elements between consecutive frequencies
};
// real = 0: z = i omega (Matsubara, static term at index 0 of a symmetrised fraction); real = 1: z = omega + i pi/beta
// res: scratch of njobs * nw complex values
void launch_cf(const CfJob *jobs_dev, int njobs, const double *omega, int nw, double beta_T, int real, double2 *res,
               cudaStream_t st);
void launch_chi_tail(double *chi, long long stride, int nw, const double *omega, double beta_T, double avg,
                     cudaStream_t st);

}  // namespace edgpu
