// Krylov kernels: the plain Lanczos recurrence of the Green's-function path, the restarted Lanczos
// eigen-solver that replaces ARPACK, the small dense Jacobi eigen-solver, a / a+ and diagonal
// operators, and the continued-fraction evaluation.
//
// * Lanczos recurrence  -- include/edlib/Lanczos.h:36-77 (no re-orthogonalisation, break on beta < 1e-10), on
//                          FP32, FP64 or float-float vectors
// * eigen-solver        -- replaces the dsaupd/dseupd loop of include/edlib/Storage.h:43-146: thick-restart
//                          Lanczos with one Gram-corrected classical Gram-Schmidt pass per step against the
//                          whole basis (h = (I - E) s with the Gram deviation E = V^T V - I kept current: the
//                          orthogonality of a second pass with two passes over the basis instead of four);
//                          dependent residuals are replaced by fresh random vectors so the basis can grow to
//                          the full sector (exact multiplicities when ncv >= dim).
// * a / a+              -- FermionicModel::a/adag + a_adag of the storages (FermionicModel.h:45-68,
//                          CRSStorage.h:131-145), written as a gather over the target sector
// * diagonal operators  -- ChiLoc SzOperator / NOperator and operation() (ChiLoc.h:40-91, 474-530)
// * continued fraction  -- get_frac_point, compute_(sym_)continued_fraction, update_static
//                          (Lanczos.h:83-124, 166-169, 201-224); zero_freq_contribution / get_tail (ChiLoc.h:358-411)
#include <cfloat>

#include "edgpu_kernels.h"

namespace edgpu {

constexpr int kBlk = 256;

__device__ __forceinline__ double sum_partials(const double *p, int n, double *red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
  s = block_sum<kBlk>(s, red);
  __syncthreads();
  if (threadIdx.x == 0) red[0] = s;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// ================================================================ plain Lanczos recurrence

// phase 2: alf = <v, w>; w -= alf v; |w|^2 per item
template <typename T>
__global__ void __launch_bounds__(kBlk) k_lz_alpha(const LzTask<T> *tasks, const int *item_task, int nitems, int iter) {
  __shared__ double red[kBlk / 32];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const LzTask<T> &t = tasks[item_task[it]];
    if (t.state[0]) continue;
    const long long li = it - t.item_begin;
    const double alf = sum_partials(t.part_a, t.nitems, red);
    if (li == 0 && threadIdx.x == 0) {
      t.alpha[iter] = alf;
      t.scal[0] = alf;
    }
    long long lo, hi;
    item_range(*t.op, t.srs_rows, li, lo, hi);
    const T *v = t.buf[iter % 3];
    T *w = t.buf[(iter + 1) % 3];
    const T a = (T)alf;
    DotAcc acc;
    dot_init(acc);
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const T x = renorm(w[i] - a * v[i]);  // float-float: hi restored after the cancellation against a v
      w[i] = x;
      dot_add(acc, x, x);
    }
    double s = block_sum<kBlk>(dot_value(acc), red);
    if (threadIdx.x == 0) t.part_b[li] = s;
  }
}

// phase 3: bet = sqrt(|w|^2); store; stop below 1e-10; else w /= bet becomes the next v
template <typename T>
__global__ void __launch_bounds__(kBlk) k_lz_beta(const LzTask<T> *tasks, const int *item_task, int nitems, int iter) {
  __shared__ double red[kBlk / 32];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const LzTask<T> &t = tasks[item_task[it]];
    if (t.state[0]) continue;
    const long long li = it - t.item_begin;
    const double bet = sqrt(sum_partials(t.part_b, t.nitems, red));
    const bool stop = fabs(bet) < 1e-10;
    if (li == 0 && threadIdx.x == 0) {
      t.scal[1] = bet;
      if (iter + 1 != t.nlanc_max) t.beta[iter + 1] = bet;
      t.state[1] = iter + 1;
      if (stop || iter + 1 == t.nlanc_max) t.state[0] = 1;
    }
    if (stop || iter + 1 == t.nlanc_max) continue;
    long long lo, hi;
    item_range(*t.op, t.srs_rows, li, lo, hi);
    T *w = t.buf[(iter + 1) % 3];
    // one reciprocal per block and a multiply per element: GB300 issues FP64 at 2 lanes per clock per SM, and a
    // division per element made this pass FP64-bound (it differs from w / b by at most one rounding)
    const T rb = (T)(1.0 / bet);
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) w[i] = renorm(w[i] * rb);
  }
}

static int grid_items(int nitems) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 148;
  }
  int g = nsm * 8;
  return nitems < g ? (nitems > 0 ? nitems : 1) : g;
}

template <typename T>
void launch_lz_step(const LzTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int ntasks, int it,
                    MvShape sh, cudaStream_t st) {
  launch_lz_mv<T>(tasks_dev, item_task_dev, nitems_total, it, sh, st);
  k_lz_alpha<T><<<grid_items(nitems_total), kBlk, 0, st>>>(tasks_dev, item_task_dev, nitems_total, it); note_launch();
  k_lz_beta<T><<<grid_items(nitems_total), kBlk, 0, st>>>(tasks_dev, item_task_dev, nitems_total, it); note_launch();
}

// ================================================================ eigen-solver step
// One Lanczos step of every task that still grows its basis, with one-pass classical Gram-Schmidt made
// exact by the Gram matrix of the basis:
//   k_eig_mv (spmv.cu)  w = H V[j]
//   k_cgs_dot           per chunk: s = V^T w, g = V^T V[j] (the Gram column of the newest vector), |w|^2
//   k_cgs_upd           every block reduces s and g over the chunks in a fixed order, completes
//                       E = V^T V - I with column j, and takes the projection coefficients
//                       h = (I - E) s = (V^T V)^{-1} s + O(|E|^2 |s|); then w -= V h, accumulated in
//                       float-float for FP32 vectors (so the only rounding is the final one), |w|^2 per chunk
//   k_eig_norm          accept V[j+1] = w / |w|, or declare w dependent and draw a random vector
//   k_eig_scale         apply the decision
// Two passes over the basis per step (classical Gram-Schmidt with a second pass needs four) with the
// orthogonality of the second pass: the coefficients are the exact projection for the basis as stored,
// and the update adds no rounding of the size of |w| before the cancellation.  After a restart the
// kept vectors' Gram block is formed from the old one and the restart's coefficients (k_eig_gram_proj).
// The Gram-Schmidt kernels walk vectors in chunks
// of kCgsChunk elements, independent of the operator's items.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double rand_elem(unsigned long long seed, int draw, long long i) {
  unsigned long long h = mix64(seed ^ mix64((unsigned long long)draw * 0x100000001b3ull + (unsigned long long)i));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5;
}

__device__ __forceinline__ void chunk_range(long long n, long long ci, long long &lo, long long &hi) {
  lo = ci * (long long)kCgsChunk;
  hi = lo + kCgsChunk;
  if (hi > n) hi = n;
}

// Element layout of a chunk: thread t owns the 16-byte groups starting at lo + VEC t + g VEC kBlk for
// g < G (VEC = 16 / sizeof(T), G = kCgsChunk / (VEC kBlk)), so each warp load is 512 contiguous bytes.
// Basis columns have a stride ldv that is a multiple of VEC, so every group load is aligned; elements past
// n (the padding) are loaded but never used.
template <typename T>
struct CgsGeom {
  static constexpr int VEC = 16 / sizeof(T);
  static constexpr int G = kCgsChunk / (VEC * kBlk);
  __device__ static long long at(long long lo, int g) { return lo + (long long)VEC * threadIdx.x + (long long)g * VEC * kBlk; }
};

// Warp sums of NB (a power of two, <= 32) values per lane by a transposing butterfly: the exchanges 16,
// 8, ... lanes apart each hand over half of the values still held, until one is left; ordinary steps
// finish.  Eight sums take 9 exchanges instead of 40.  Afterwards every lane holds in slot 0 the warp
// total of value (lane >> (5 - log2 NB)) & (NB - 1), each total by a fixed tree.  FP32 values travel as
// float-float pairs (h, l).
template <int NB>
__device__ __forceinline__ void warp_sum_t(float (&h)[NB], float (&l)[NB]) {
  const int lane = threadIdx.x & 31;
  int o = 16;
#pragma unroll
  for (int half = NB / 2; half >= 1; half >>= 1, o >>= 1) {
    const bool up = lane & o;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      const float sh = up ? h[k] : h[k + half], sl = up ? l[k] : l[k + half];
      float kh = up ? h[k + half] : h[k], kl = up ? l[k + half] : l[k];
      ff_add(kh, kl, __shfl_xor_sync(0xffffffffu, sh, o), __shfl_xor_sync(0xffffffffu, sl, o));
      h[k] = kh;
      l[k] = kl;
    }
  }
#pragma unroll
  for (; o >= 1; o >>= 1)
    ff_add(h[0], l[0], __shfl_xor_sync(0xffffffffu, h[0], o), __shfl_xor_sync(0xffffffffu, l[0], o));
}
template <int NB>
__device__ __forceinline__ void warp_sum_t(double (&h)[NB]) {
  const int lane = threadIdx.x & 31;
  int o = 16;
#pragma unroll
  for (int half = NB / 2; half >= 1; half >>= 1, o >>= 1) {
    const bool up = lane & o;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      const double send = up ? h[k] : h[k + half];
      h[k] = (up ? h[k + half] : h[k]) + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
#pragma unroll
  for (; o >= 1; o >>= 1) h[0] += __shfl_xor_sync(0xffffffffu, h[0], o);
}

// Projection coefficients of the step from s = V^T w, g = V^T V[j] and n0 = |w|^2 summed over the task:
// h = s - E s with E = V^T V - I (entries (c, d < j) from earlier steps, column j from g), a warp per row;
// records column j of E and, in Lanczos mode, column j of the projected matrix.  Then the column order
// of the update: for FP32 vectors the columns whose |h| exceeds 1/64 of the estimated residual
// sqrt(n0 - |s|^2) come first and are subtracted exactly (float-float), the rest afterwards by single
// fused multiply-adds on a running value that is already of the residual's size; a residual below 1e-3
// |w| (near dependence) keeps every column exact.  FP64 vectors keep the index order.
template <typename T>
__device__ void cgs_coefficients(const EigTask<T> &t, int j, const double *sv, const double *gv, double *hs,
                                 double n0) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, mode = t.st[1];
  for (int c = warp; c <= j; c += kBlk / 32) {
    double a = 0.0;
    for (int d = lane; d <= j; d += 32) {
      double e;
      if (c == j && d == j) e = gv[j] - 1.0;
      else if (c == j) e = gv[d];
      else if (d == j) e = gv[c];
      else e = t.E[(long long)d * t.ld + c];
      a += e * sv[d];
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double h = sv[c] - a;
      hs[c] = h;
      t.hv[c] = h;
      if (mode == 0) t.Tm[(long long)j * t.ld + c] = h;
    }
  }
  for (int c = threadIdx.x; c <= j; c += blockDim.x) {
    const double e = c == j ? gv[j] - 1.0 : gv[c];
    t.E[(long long)j * t.ld + c] = e;
    t.E[(long long)c * t.ld + j] = e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int *ord = t.ord;
    double lim = -1.0;  // every column exact
    if (sizeof(T) == 4) {
      double ss = 0.0;
      for (int c = 0; c <= j; ++c) ss += sv[c] * sv[c];
      const double b2 = n0 - ss;
      if (b2 > 1e-6 * n0) lim = 0.015625 * sqrt(b2);
    }
    int k = 1;
    for (int c = 0; c <= j; ++c)
      if (!(fabs(hs[c]) <= lim)) ord[k++] = c;
    ord[0] = k - 1;
    for (int c = 0; c <= j; ++c)
      if (fabs(hs[c]) <= lim) ord[k++] = c;
  }
}

// The reduction of one split (kCgsSup consecutive chunks of a task) of the chunk partials of s, g and
// |w|^2, and, in the block of the task's last split to finish, the sum over the splits and the projection
// coefficients.  Values v < nv = 2 nc + 1: s (v < nc), g, then n0; a split row of spart holds them at
// [0, nc), [ld, ld + nc) and 2 ld.  Each sum runs in a fixed order (P interleaved parts, then the parts
// in order), so the result depends only on the chunk partials, not on which block finished last or on
// what else shares the launch.  The split count is an atomic after a memory fence; the last arrival
// resets it, so it is zero again for the next launch.  No block waits for another.
template <typename T>
__device__ void cgs_split(const EigTask<T> &t, int sc, int j, double *part, double *sv, double *gv, double *hs,
                          int &flag) {
  const int nsup = cgs_nsup(t.nchunks), ld = t.ld, nc = j + 1, nv = 2 * nc + 1;
  const long long S = 2 * (long long)ld + 2;
  const int P = max(1, (int)blockDim.x / nv);
  const int v = (int)threadIdx.x % nv, p = (int)threadIdx.x / nv;
  const int off = v < nc ? v : (v < 2 * nc ? ld + v - nc : 2 * ld);
  {
    const int q0 = sc * kCgsSup, q1 = min(q0 + kCgsSup, t.nchunks);
    double a = 0.0;
    if (p < P) {
      const double *src;
      long long stride;
      if (v < nc) src = t.hpart + v, stride = ld;
      else if (v < 2 * nc) src = t.hpart2 + (v - nc), stride = ld;
      else src = t.npart, stride = 1;
#pragma unroll 4
      for (int q = q0 + p; q < q1; q += P) a += src[(long long)q * stride];
    }
    part[threadIdx.x] = a;
  }
  __syncthreads();
  if (nsup == 1) {  // the split is the task: straight to the coefficients (the same sums, bit for bit)
    if ((int)threadIdx.x < nv) {
      double a = 0.0;
      for (int q = 0; q < P; ++q) a += part[q * nv + threadIdx.x];
      if (v < nc) sv[v] = a;
      else if (v < 2 * nc) gv[v - nc] = a;
      else part[kBlk] = a;
    }
    __syncthreads();
    cgs_coefficients(t, j, sv, gv, hs, part[kBlk]);
    __syncthreads();
    return;
  }
  if ((int)threadIdx.x < nv) {
    double a = 0.0;
    for (int q = 0; q < P; ++q) a += part[q * nv + threadIdx.x];
    t.spart[sc * S + off] = a;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) flag = atomicAdd(&t.cnt[nsup], 1) == nsup - 1;
  __syncthreads();
  if (!flag) return;  // uniform
  __threadfence();
  if (threadIdx.x == 0) t.cnt[nsup] = 0;
  {
    double a = 0.0;
    if (p < P)
#pragma unroll 4
      for (int q = p; q < nsup; q += P) a += __ldcg(t.spart + q * S + off);
    part[threadIdx.x] = a;
  }
  __syncthreads();
  if ((int)threadIdx.x < nv) {
    double a = 0.0;
    for (int q = 0; q < P; ++q) a += part[q * nv + threadIdx.x];
    if (v < nc) sv[v] = a;
    else if (v < 2 * nc) gv[v - nc] = a;
    else part[kBlk] = a;
  }
  __syncthreads();
  cgs_coefficients(t, j, sv, gv, hs, part[kBlk]);
  __syncthreads();
}

// One block per split leader (the chunk that starts a split of a task), taken from the batch's leader map
// (chunk indices of the leaders, built with the chunk map): cgs_split for the tasks still growing.
template <typename T>
__global__ void __launch_bounds__(kBlk, 1) k_cgs_coef(const EigTask<T> *tasks, const int *chunk_task, const int *leaders,
                                                     int nleaders) {
  __shared__ double part[kBlk + 1];
  __shared__ double sv[kMaxLd], gv[kMaxLd], hs[kMaxLd];
  __shared__ int flag;
  for (int li = blockIdx.x; li < nleaders; li += gridDim.x) {
    const int it = leaders[li];
    const EigTask<T> &t = tasks[chunk_task[it]];
    if (t.st[2]) continue;  // uniform across the block
    cgs_split(t, (it - t.chunk_begin) / kCgsSup, t.st[0], part, sv, gv, hs, flag);
  }
}

// ---------------------------------------------------------------- bulk-copy slice pipelines
// Kernels that stream vector slices (the Gram-Schmidt passes, the thick restart) pass them through S
// shared-memory stages filled by bulk (TMA) copies that the first lane of a producer warp issues S slices
// ahead, across chunk boundaries, so that S - 1 slices per block are in flight while the compute warps
// work on the last one (ProdPipe).  Every compute warp waits for a slice on the stage's full barrier (one
// arrival with the byte count) and, when done with it, arrives on the stage's empty barrier (one arrival
// per warp); the producer refills a stage once all compute warps have arrived.  No block-wide barrier per
// slice.  Waits are bounded: after one gave up a thread stops waiting (its results are void, and the host
// is told through g_cgs_stall), and before the block's shared memory is released each stage's last copy
// gets one more bounded wait.
__device__ int g_cgs_stall = 0;
constexpr int kCgsSpin = 1 << 22;  // try_wait rounds before a stage is declared stalled

__device__ __forceinline__ bool cgs_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < kCgsSpin; ++it) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory geometry of a slice stream: S stages of STAGE bytes, a full and an empty barrier per stage
// behind them (SMEM bytes in all).  ProdPipe runs the stream.
template <int S_, int STAGE_>
struct StageGeom {
  static constexpr int S = S_, STAGE = STAGE_;
  static constexpr size_t SMEM = (size_t)S * STAGE + 16 * S;
};

// The Gram-Schmidt passes' stream: per chunk of the block (it = blockIdx.x, + gridDim.x, ...) the
// chunk's slice of w, then of the columns.  Dot pass: k = 0 w, 1 V[j], 2 + c V[c]; update pass: 0 w,
// 1 + q V[ord[1 + q]].  Chunks of tasks that do not grow have no slices.
template <typename T>
using CgsPipeT = StageGeom<sizeof(T) == 4 ? EDGPU_CGS_STAGES : 2, kCgsChunk * (int)sizeof(T)>;

template <typename T, bool UPD>
struct CgsIssue {
  const EigTask<T> *tasks;
  const int *chunk_task;
  int nchunks, it, k;
  __device__ __forceinline__ bool operator()(unsigned dst, unsigned bar) {
    while (it < nchunks) {
      const EigTask<T> &t = tasks[chunk_task[it]];
      const int j = t.st[0];
      const int nslices = t.st[2] ? 0 : (j >= 0 ? j + 2 : 1);
      if (k >= nslices) {
        it += gridDim.x;
        k = 0;
        continue;
      }
      long long lo, hi;
      chunk_range(t.n, it - t.chunk_begin, lo, hi);
      const int col = UPD ? (k > 0 ? t.ord[k] : 0) : (k == 1 ? j : k - 2);
      const T *src = k == 0 ? t.w : t.V + (long long)col * t.ldv;
      stage_copy(dst, src + lo, (unsigned)((((hi - lo) * (long long)sizeof(T)) + 15) & ~15LL), bar);  // in the padding
      ++k;
      return true;
    }
    return false;
  }
};

// A slice pipe with a producer warp: kBlk consumer threads (8 warps) and one more warp whose
// first lane issues every slice of the block's stream, refilling a stage once all 8 consumer warps have
// released it (its empty barrier).  The consumers only wait on full barriers and release: no thread of
// theirs waits for the others per slice.  Consumer-only block synchronisation uses named barrier 1
// (cgs_csync), so the producer warp can leave as soon as its stream is issued.
template <int S_, int STAGE_>
struct ProdPipe {
  static constexpr int S = S_, STAGE = STAGE_;
  static constexpr size_t SMEM = (size_t)S * STAGE + 16 * S;
  unsigned char *mem;
  unsigned base, bars, empties;
  int used;
  bool stalled;
  __device__ void init(unsigned char *m) {
    mem = m;
    base = (unsigned)__cvta_generic_to_shared(mem);
    bars = base + (unsigned)(S * STAGE);
    empties = bars + 8u * S;
    if (threadIdx.x == 0) {
      for (int q = 0; q < S; ++q) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bars + 8u * q) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(empties + 8u * q), "r"(kBlk / 32) : "memory");
      }
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();  // every thread of the block, the producer warp included
    used = 0;
    stalled = false;
  }
  // the producer warp: lane 0 issues the whole stream.  When a bounded wait for a free stage gives up it
  // issues nothing more (no full barrier is armed again and no stage a consumer may still read is
  // overwritten), flags the host and gives each slice already issued one more bounded wait before leaving;
  // the consumers then give up once on the slices that never come.
  template <class Issue>
  __device__ void produce(Issue &issue) {
    if ((threadIdx.x & 31) != 0) return;
    bool gave_up = false;
    int u = 0;
    for (;; ++u) {
      const int q = u % S;
      if (u >= S && !cgs_wait(empties + 8u * q, (unsigned)(((u - S) / S) & 1))) {
        gave_up = true;
        break;
      }
      if (!issue(base + (unsigned)(q * STAGE), bars + 8u * q)) break;
    }
    if (gave_up) {
      atomicExch(&g_cgs_stall, 1);
      for (int v = max(0, u - S); v < u; ++v) cgs_wait(bars + 8u * (v % S), (unsigned)((v / S) & 1));
    }
  }
  __device__ const unsigned char *take() {
    const int stage = used % S;
    if (!stalled) stalled = !cgs_wait(bars + 8u * stage, (unsigned)((used / S) & 1));
    return mem + stage * STAGE;
  }
  __device__ void release() {
    const int stage = used % S;
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
      unsigned long long state;
      asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];\n" : "=l"(state) : "r"(empties + 8u * stage) : "memory");
    }
    ++used;
  }
  // a consumer whose bounded wait gave up flags the host and, before the block's shared memory can be
  // released, gives each stage's last slice (consumers take every issued slice, in issue order) one more
  // bounded wait
  __device__ void finish() {
    if (stalled) {
      atomicExch(&g_cgs_stall, 1);
      for (int v = max(0, used - S); v < used; ++v) cgs_wait(bars + 8u * (v % S), (unsigned)((v / S) & 1));
    }
  }
};

// the Gram-Schmidt passes' producer pipe, slices read as T
template <typename T>
struct CgsProdPipe : ProdPipe<CgsPipeT<T>::S, CgsPipeT<T>::STAGE> {
  __device__ const T *take() { return reinterpret_cast<const T *>(ProdPipe<CgsPipeT<T>::S, CgsPipeT<T>::STAGE>::take()); }
};

// barrier of the kBlk consumer threads only (named barrier 1)
__device__ __forceinline__ void cgs_csync() { asm volatile("bar.sync 1, %0;\n" ::"n"(kBlk) : "memory"); }

// block_sum over the consumer threads
__device__ inline double cgs_csum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  cgs_csync();
  if (lane == 0) red[warp] = v;
  cgs_csync();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlk / 32; ++w) r += red[w];
  return r;
}

// The thread's G groups of the staged slice (16 bytes each, kBlk * 16 bytes apart); with MASK the
// elements at or past rem read as zeros (the padding of the last chunk holds arbitrary bits).
template <typename T, bool MASK>
__device__ __forceinline__ void stage_read(const T *slice, int rem, Lanes<T> (&x)[CgsGeom<T>::G]) {
  constexpr int VEC = CgsGeom<T>::VEC, G = CgsGeom<T>::G, GS = VEC * kBlk;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    x[g] = *reinterpret_cast<const Lanes<T> *>(slice + VEC * threadIdx.x + g * GS);
    if (MASK) {
#pragma unroll
      for (int v = 0; v < VEC; ++v)
        if (g * GS + v >= rem) x[g].v[v] = T(0);
    }
  }
}

// The column part of the dot pass for one chunk: positions p = 0..j in batches of NB (FP32: 8, FP64: 2,
// bounded by registers); position 0 is V[j] itself (taken into vj), position p > 0 column p - 1.  Per
// warp and column the two sums go to ps / pg.  MASK: the chunk is the vector's last and partial, elements
// at or past rem read as zeros (a separate instantiation, so full chunks carry no selects).
template <typename T, bool MASK, class Pipe>
__device__ __forceinline__ void cgs_dot_columns(Pipe &pipe, const Lanes<T> (&w)[CgsGeom<T>::G],
                                                Lanes<T> (&vj)[CgsGeom<T>::G], int rem, int j,
                                                double (*ps)[kMaxLd], double (*pg)[kMaxLd]) {
  using Geo = CgsGeom<T>;
  constexpr int VEC = Geo::VEC, G = Geo::G;
  constexpr bool F32 = sizeof(T) == 4;
  constexpr int NB = F32 ? 8 : 2, LB = F32 ? 3 : 1;
  using Acc = typename std::conditional<F32, float, double>::type;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int p0 = 0; p0 <= j; p0 += NB) {
    Acc sh[NB], gh[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int p = p0 + q;
      sh[q] = gh[q] = Acc(0);
      if (p > j) continue;
      const T *sl = pipe.take();
      if (p == 0) stage_read<T, MASK>(sl, rem, vj);
      // group by group from the stage (FP64 has no registers for a whole slice)
#pragma unroll
      for (int g = 0; g < G; ++g) {
        Lanes<T> x = *reinterpret_cast<const Lanes<T> *>(sl + VEC * threadIdx.x + g * (VEC * kBlk));
        if (MASK) {
#pragma unroll
          for (int v = 0; v < VEC; ++v)
            if (g * (VEC * kBlk) + v >= rem) x.v[v] = T(0);
        }
        T s = x.v[0] * w[g].v[0], r = x.v[0] * vj[g].v[0];
#pragma unroll
        for (int v = 1; v < VEC; ++v) {
          s = fma(x.v[v], w[g].v[v], s);
          r = fma(x.v[v], vj[g].v[v], r);
        }
        sh[q] += s;
        gh[q] += r;
      }
      pipe.release();
    }
    const int p = p0 + ((lane >> (5 - LB)) & (NB - 1));
    const int c = p == 0 ? j : p - 1;
    const bool writer = (lane & ((32 >> LB) - 1)) == 0 && p <= j;
    if constexpr (F32) {
      float sl[NB], gl[NB];
#pragma unroll
      for (int q = 0; q < NB; ++q) sl[q] = gl[q] = 0.f;
      warp_sum_t<NB>(sh, sl);
      warp_sum_t<NB>(gh, gl);
      if (writer) {
        ps[warp][c] = (double)sh[0] + (double)sl[0];
        pg[warp][c] = (double)gh[0] + (double)gl[0];
      }
    } else {
      warp_sum_t<NB>(sh);
      warp_sum_t<NB>(gh);
      if (writer) {
        ps[warp][c] = sh[0];
        pg[warp][c] = gh[0];
      }
    }
  }
}

// Per chunk: s = V^T w, g = V^T V[j] and |w|^2.  The slices of w and V[j] are taken into registers;
// every other column's slice is used from its stage.  A thread's products of one column are summed by
// fused multiply-adds (G * VEC = 16 terms), the warp sums taken a batch of columns at a time by a
// transposing butterfly in float-float (FP32 data), the warps and chunks added in FP64.  The roundings
// of the 16-term sums are independent from thread to thread, so their total stays far below the FP32
// rounding of the vectors being orthogonalised.  Column order within the chunk: j, 0, 1, ..., j - 1.
template <typename T>
__global__ void __launch_bounds__(kBlk + 32, sizeof(T) == 4 ? EDGPU_CGS_MIN_BLOCKS : 1) k_cgs_dot(const EigTask<T> *tasks, const int *chunk_task, int nchunks) {
  using Geo = CgsGeom<T>;
  constexpr int VEC = Geo::VEC, G = Geo::G;
  extern __shared__ __align__(128) unsigned char cgs_stage[];
  __shared__ double ps[kBlk / 32][kMaxLd], pg[kBlk / 32][kMaxLd];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  CgsProdPipe<T> pipe;
  pipe.init(cgs_stage);
  if (threadIdx.x >= kBlk) {  // the producer warp
    CgsIssue<T, false> iss{tasks, chunk_task, nchunks, (int)blockIdx.x, 0};
    pipe.produce(iss);
    return;
  }
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const EigTask<T> &t = tasks[chunk_task[it]];
    if (t.st[2]) continue;
    const long long ci = it - t.chunk_begin;
    const int j = t.st[0];
    long long lo, hi;
    chunk_range(t.n, ci, lo, hi);
    const int rem = (int)(hi - (lo + (long long)VEC * threadIdx.x));
    const bool full = hi - lo == kCgsChunk;
    Lanes<T> w[G], vj[G];
    {
      const T *sl = pipe.take();
      if (full) stage_read<T, false>(sl, rem, w);
      else stage_read<T, true>(sl, rem, w);
      pipe.release();
    }
    // |w|^2: the warp's sum goes to the spare slot kMaxLd - 1 of ps and is summed over the warps with the
    // columns at the end of the chunk
    {
      DotAcc acc;
      dot_init(acc);
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int v = 0; v < VEC; ++v) dot_add(acc, w[g].v[v], w[g].v[v]);
      dot_warp_sum<T>(acc);
      if (lane == 0) ps[warp][kMaxLd - 1] = dot_value(acc);
    }
    if (full) cgs_dot_columns<T, false>(pipe, w, vj, rem, j, ps, pg);
    else cgs_dot_columns<T, true>(pipe, w, vj, rem, j, ps, pg);
    cgs_csync();
    // value c <= j: s and g of column c; c = j + 1: |w|^2
    for (int c = threadIdx.x; c <= j + 1; c += kBlk) {
      double a = 0.0, b = 0.0;
      const int cs = c <= j ? c : kMaxLd - 1;
      for (int q = 0; q < kBlk / 32; ++q) {
        a += ps[q][cs];
        if (c <= j) b += pg[q][c];
      }
      if (c <= j) {
        t.hpart[ci * (long long)t.ld + c] = a;
        t.hpart2[ci * (long long)t.ld + c] = b;
      } else {
        t.npart[ci] = a;
      }
    }
    cgs_csync();  // ps / pg are reused by the next chunk
  }
  pipe.finish();
}

// Running value of w[i] - sum_c h[c] V[c][i]: FP32 keeps it in float-float with h in float-float (one
// final rounding); FP64 uses plain fused multiply-adds.
struct CgsAcc32 {
  float hi, lo;
};
__device__ __forceinline__ void cgs_sub(CgsAcc32 &a, float hh, float hl, float v) {
  const float p = hh * v;
  const float pe = fmaf(hh, v, -p) + hl * v;
  const float t = a.hi - p;
  const float bb = t - a.hi;
  const float e = (a.hi - (t - bb)) - (p + bb);
  a.hi = t;
  a.lo += e - pe;
}
struct CgsAcc64 {
  double hi;
};
__device__ __forceinline__ void cgs_sub(CgsAcc64 &a, double hh, double, double v) { a.hi = fma(-hh, v, a.hi); }
template <typename T>
struct CgsAcc;
template <>
struct CgsAcc<float> {
  using type = CgsAcc32;
  __device__ static type init(float x) { return {x, 0.f}; }
  __device__ static float value(const type &a) { return a.hi + a.lo; }
};
template <>
struct CgsAcc<double> {
  using type = CgsAcc64;
  __device__ static type init(double x) { return {x}; }
  __device__ static double value(const type &a) { return a.hi; }
};

// w -= V h over the chunk, the columns in the order the coefficient step chose: the first ord[0] into a
// float-float running value for FP32 vectors (exact subtraction, one rounding at the end), the rest by
// single fused multiply-adds once the running value is rounded to the vectors' type.  The chunk's slices
// of w and of the columns arrive through the block's bulk-copy stream; w is taken into registers, every
// column used from its stage.  |w|^2 partials per chunk for the acceptance test.
template <typename T>
__global__ void __launch_bounds__(kBlk + 32, EDGPU_CGS_MIN_BLOCKS) k_cgs_upd(const EigTask<T> *tasks, const int *chunk_task, int nchunks) {
  using Geo = CgsGeom<T>;
  constexpr int VEC = Geo::VEC, G = Geo::G, GS = VEC * kBlk;
  using Acc = CgsAcc<T>;
  extern __shared__ __align__(128) unsigned char cgs_stage[];
  __shared__ double red[kBlk / 32];
  __shared__ T hh[kMaxLd], hl[kMaxLd];
  CgsProdPipe<T> pipe;
  pipe.init(cgs_stage);
  if (threadIdx.x >= kBlk) {  // the producer warp
    CgsIssue<T, true> iss{tasks, chunk_task, nchunks, (int)blockIdx.x, 0};
    pipe.produce(iss);
    return;
  }
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const EigTask<T> &t = tasks[chunk_task[it]];
    if (t.st[2]) continue;
    const long long ci = it - t.chunk_begin;
    const int j = t.st[0];
    long long lo, hi;
    chunk_range(t.n, ci, lo, hi);
    const long long first = lo + (long long)VEC * threadIdx.x;
    const int rem = (int)(hi - first);
    const bool full = hi - lo == kCgsChunk;
    cgs_csync();
    for (int q = threadIdx.x; q <= j; q += kBlk) {
      const double h = t.hv[t.ord[1 + q]];
      hh[q] = (T)h;
      hl[q] = (T)(h - (double)(T)h);
    }
    const int nbig = sizeof(T) == 8 ? j + 1 : (j >= 0 ? t.ord[0] : 0);  // FP64: one loop of plain FMAs
    cgs_csync();
    typename Acc::type a[G][VEC];
    {
      Lanes<T> wq[G];
      const T *sl = pipe.take();
      if (full) stage_read<T, false>(sl, rem, wq);
      else stage_read<T, true>(sl, rem, wq);
      pipe.release();
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int v = 0; v < VEC; ++v) a[g][v] = Acc::init(wq[g].v[v]);
    }
    // column slices past the end of the vector hold arbitrary bits; only the elements below rem are kept
    int q = 0;
    for (; q < nbig; ++q) {
      const T *sl = pipe.take();
      const T h0 = hh[q], h1 = hl[q];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const Lanes<T> x = *reinterpret_cast<const Lanes<T> *>(sl + VEC * threadIdx.x + g * GS);
#pragma unroll
        for (int v = 0; v < VEC; ++v) cgs_sub(a[g][v], h0, h1, x.v[v]);
      }
      pipe.release();
    }
    Lanes<T> x[G];
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int v = 0; v < VEC; ++v) x[g].v[v] = Acc::value(a[g][v]);
    if constexpr (sizeof(T) == 4) {
      for (; q <= j; ++q) {
        const T *sl = pipe.take();
        const T h0 = -hh[q];
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const Lanes<T> c = *reinterpret_cast<const Lanes<T> *>(sl + VEC * threadIdx.x + g * GS);
#pragma unroll
          for (int v = 0; v < VEC; ++v) x[g].v[v] = fma(h0, c.v[v], x[g].v[v]);
        }
        pipe.release();
      }
    }
    DotAcc acc;
    dot_init(acc);
#pragma unroll
    for (int g = 0; g < G; ++g) {
#pragma unroll
      for (int v = 0; v < VEC; ++v) {
        if (!full && g * GS + v >= rem) x[g].v[v] = T(0);  // padding
        dot_add(acc, x[g].v[v], x[g].v[v]);
      }
      if (g * GS < rem) store_lanes(t.w + first + g * GS, x[g].v);
    }
    const double s2 = cgs_csum(dot_value(acc), red);
    if (threadIdx.x == 0) t.npart[t.nchunks + ci] = s2;
  }
  pipe.finish();
}

// one block per task: accept the new basis vector, or declare the residual dependent
template <typename T>
__global__ void k_eig_norm(const EigTask<T> *tasks) {
  __shared__ double red[kBlk / 32];
  const EigTask<T> &t = tasks[blockIdx.x];
  if (t.st[2]) {  // not growing: nothing for k_eig_scale to apply (uniform across the block)
    if (threadIdx.x == 0) t.st[4] = 0;
    return;
  }
  const double n0 = sum_partials(t.npart, t.nchunks, red);
  const double b2 = sum_partials(t.npart + t.nchunks, t.nchunks, red);
  if (threadIdx.x != 0) return;
  const int j = t.st[0];
  const int mode = t.st[1];
  const double beta = sqrt(b2);
  const double w0 = sqrt(n0);  // before orthogonalisation
  t.st[4] = 0;
  if (j + 1 >= t.n) {  // the basis spans the whole sector: exact, no residual
    t.st[0] = j + 1;
    t.st[2] = 1;
    t.nsc[1] = 0.0;
    return;
  }
  // w lies in the span when the projection removed all but a small part of it: the new vector would keep
  // an orthogonality error of (rounding) * |w| / beta.  The bound is 1e-6 for FP32 vectors (rounding 6e-8)
  // and 1e-9 for FP64 ones (rounding 1e-16): a basis started from a vector that is already an eigenvector to
  // FP32 accuracy (the FP64 continuation of an FP32 solve) has a first residual of about 1e-6 |w|, which must
  // be taken as the next Lanczos vector, not replaced by a random one.
  const bool dependent = !(beta > (sizeof(T) == 8 ? 1e-9 : 1e-6) * w0) || !(beta > 1e-300);
  if (!dependent) {
    if (j >= 0) {
      double cpl = mode == 0 ? beta : 0.0;
      t.Tm[(long long)j * t.ld + (j + 1)] = cpl;
      t.Tm[(long long)(j + 1) * t.ld + j] = cpl;
    }
    t.nsc[1] = beta;
    t.st[0] = j + 1;
    t.st[1] = 0;
    t.st[4] = 1;
    if (j + 1 == t.m) t.st[2] = 1;
  } else {
    if (j >= 0 && mode == 0) {
      t.Tm[(long long)j * t.ld + (j + 1)] = 0.0;
      t.Tm[(long long)(j + 1) * t.ld + j] = 0.0;
    }
    t.st[1] = 1;
    t.st[3] += 1;
    t.st[4] = 2;
    if (t.st[3] > 64) t.st[2] = 1;  // give up growing (reported through the basis size)
  }
}

// apply the decision: V[j] = w / beta, or a fresh random w
template <typename T>
__global__ void __launch_bounds__(kBlk) k_eig_scale(const EigTask<T> *tasks, const int *chunk_task, int nchunks) {
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const EigTask<T> &t = tasks[chunk_task[it]];
    const int act = t.st[4];
    if (act == 0) continue;
    const long long ci = it - t.chunk_begin;
    long long lo, hi;
    chunk_range(t.n, ci, lo, hi);
    if (act == 1) {  // 16-byte groups; the last group of the vector runs into its padding (ldv)
      constexpr int C = Lanes<T>::C;
      T *dst = t.V + (long long)t.st[0] * t.ldv;
      const T b = (T)t.nsc[1];
      for (long long i = lo + (long long)C * threadIdx.x; i < hi; i += (long long)C * blockDim.x) {
        Lanes<T> q = load16(t.w + i);
#pragma unroll
        for (int v = 0; v < C; ++v) q.v[v] = q.v[v] / b;
        store_lanes(dst + i, q.v);
      }
    } else {
      const int draw = t.st[3];
      for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) t.w[i] = (T)rand_elem(t.seed, draw, i);
    }
  }
}

// a fresh random w for every task that is about to orthogonalise one (mode 1)
template <typename T>
__global__ void k_eig_random(const EigTask<T> *tasks, const int *chunk_task, int nchunks) {
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const EigTask<T> &t = tasks[chunk_task[it]];
    if (t.st[5] || t.st[1] != 1) continue;
    const long long ci = it - t.chunk_begin;
    long long lo, hi;
    chunk_range(t.n, ci, lo, hi);
    const int draw = t.st[3];
    if (t.start && draw == 0) {  // the task's given start vector
      for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) t.w[i] = t.start[i];
      continue;
    }
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) t.w[i] = (T)rand_elem(t.seed, draw, i);
  }
}

__global__ void k_seed_combine(const void *const *vecs, const int *is64, const double *coef, int k, long long n,
                               double *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < k; ++q) {
      const double x = is64[q] ? static_cast<const double *>(vecs[q])[i] : (double)static_cast<const float *>(vecs[q])[i];
      s = fma(coef[q], x, s);
    }
    out[i] = s;
  }
}

void launch_seed_combine(const void *const *vecs, const int *is64, const double *coef, int k, long long n, double *out,
                         cudaStream_t st) {
  k_seed_combine<<<grid_items((int)std::min<long long>((n + kBlk - 1) / kBlk, 1 << 20)), kBlk, 0, st>>>(vecs, is64, coef,
                                                                                                        k, n, out);
  note_launch();
}

__global__ void k_axpy_dev(double *y, const double *x, const double *c, long long n) {
  const double a = c[0];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = fma(-a, x[i], y[i]);
}

void launch_axpy_dev(double *y, const double *x, const double *c, long long n, cudaStream_t st) {
  k_axpy_dev<<<grid_items((int)std::min<long long>((n + kBlk - 1) / kBlk, 1 << 20)), kBlk, 0, st>>>(y, x, c, n);
  note_launch();
}

template <typename T>
void launch_eig_random(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st) {
  k_eig_random<T><<<grid_items(nchunks), kBlk, 0, st>>>(tasks_dev, chunk_task_dev, nchunks); note_launch();
}

template <typename T>
void prepare_cgs();

template <typename T>
void prepare_eig_step(MvShape sh) {
  prepare_eig_mv<T>(sh);
  prepare_cgs<T>();
}

template <typename T>
void launch_eig_step(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, const int *chunk_task_dev,
                     int nchunks, const int *leaders_dev, int nleaders, int ntasks, MvShape sh, cudaStream_t st) {
  const int g = grid_items(nchunks);
  launch_eig_mv<T>(tasks_dev, item_task_dev, nitems_total, sh, st);
  launch_cgs_dot<T>(tasks_dev, chunk_task_dev, nchunks, st);
  launch_cgs_coef<T>(tasks_dev, chunk_task_dev, leaders_dev, nleaders, st);
  launch_cgs_upd<T>(tasks_dev, chunk_task_dev, nchunks, st);
  k_eig_norm<T><<<ntasks, kBlk, 0, st>>>(tasks_dev); note_launch();
  k_eig_scale<T><<<g, kBlk, 0, st>>>(tasks_dev, chunk_task_dev, nchunks); note_launch();
}

template <typename T>
void prepare_cgs() {
  cudaFuncSetAttribute(k_cgs_dot<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CgsPipeT<T>::SMEM);
  cudaFuncSetAttribute(k_cgs_upd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CgsPipeT<T>::SMEM);
}

template <typename T>
void launch_cgs_dot(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st) {
  const size_t smem = CgsPipeT<T>::SMEM;
  k_cgs_dot<T><<<occupancy_grid((const void *)k_cgs_dot<T>, kBlk + 32, smem, nchunks), kBlk + 32, smem, st>>>(
      tasks_dev, chunk_task_dev, nchunks);
  note_launch();
}

bool take_cgs_stall() {
  int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_cgs_stall, sizeof(int)) != cudaSuccess) return false;
  if (v) cudaMemcpyToSymbol(g_cgs_stall, &zero, sizeof(int));
  return v != 0;
}
template <typename T>
void launch_cgs_coef(const EigTask<T> *tasks_dev, const int *chunk_task_dev, const int *leaders_dev, int nleaders,
                     cudaStream_t st) {
  k_cgs_coef<T><<<grid_items(nleaders), kBlk, 0, st>>>(tasks_dev, chunk_task_dev, leaders_dev, nleaders);
  note_launch();
}

template <typename T>
void launch_cgs_upd(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, cudaStream_t st) {
  const size_t smem = CgsPipeT<T>::SMEM;
  k_cgs_upd<T><<<occupancy_grid((const void *)k_cgs_upd<T>, kBlk + 32, smem, nchunks), kBlk + 32, smem, st>>>(
      tasks_dev, chunk_task_dev, nchunks);
  note_launch();
}

// Gram block of the basis after a restart: E[a][b] = V[a].V[b] - delta_ab for a, b <= j (j = st[0]) of every
// task with rk != 0 (and not finished).  Per chunk, the vectors are staged in shared memory in slices; the
// pairs are taken in 4 x 4 tiles (a-block <= b-block), a warp per tile: each lane loads 4 + 4 elements per
// position and makes the 16 products (register blocking, 2 FMAs per shared-memory load), its running sums
// are plain FMAs over its positions of the slice, and the 16 warp sums come out of one transposing
// butterfly (float-float for FP32 data), accumulated per pair in FP64 over the slices; partials per chunk.
template <typename T>
__global__ void __launch_bounds__(kBlk) k_eig_gram(const EigTask<T> *tasks, const int *chunk_task, int nchunks,
                                                   const int *rk_all) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double gacc[kGramPairs];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const int b = chunk_task[it];
    const EigTask<T> &t = tasks[b];
    const int rk = rk_all[b];
    if (rk == 0 || rk == kEigDone) continue;
    const int nv = t.st[0] + 1;
    const int npair = nv * (nv + 1) / 2;
    const int nt = (nv + 3) / 4, ntile = nt * (nt + 1) / 2;
    const long long ci = it - t.chunk_begin;
    long long lo, hi;
    chunk_range(t.n, ci, lo, hi);
    const int slice = (kGramSmem / (int)sizeof(T) / nv) & ~3;  // elements per staged slice (16-byte rows)
    T *vs = reinterpret_cast<T *>(smem_raw);
    __syncthreads();
    for (int p = threadIdx.x; p < npair; p += blockDim.x) gacc[p] = 0.0;
    for (long long s0 = lo; s0 < hi; s0 += slice) {
      const int ns = (int)min((long long)slice, hi - s0);
      __syncthreads();
      for (int a = 0; a < nv; ++a) stage_async(vs + a * slice, t.V + (long long)a * t.ldv + s0, ns);
      cp_async_wait_all();
      __syncthreads();
      for (int tile = warp; tile < ntile; tile += nwarp) {
        // tile -> (ta, tb), ta <= tb, row-major over the upper triangle of tiles
        int ta = 0, rem = tile;
        while (rem >= nt - ta) {
          rem -= nt - ta;
          ++ta;
        }
        const int tb = ta + rem;
        const T *ra[4], *rb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          // rows past the basis read row 0 (their sums are dropped)
          ra[i] = vs + (ta * 4 + i < nv ? ta * 4 + i : 0) * slice;
          rb[i] = vs + (tb * 4 + i < nv ? tb * 4 + i : 0) * slice;
        }
        using Acc = typename std::conditional<sizeof(T) == 4, float, double>::type;
        Acc acc[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = Acc(0);
        for (int k = lane; k < ns; k += 32) {
          T x[4], y[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            x[i] = ra[i][k];
            y[i] = rb[i][k];
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) acc[i * 4 + jj] = fma(x[i], y[jj], acc[i * 4 + jj]);
        }
        // lane l then holds in slot 0 the warp sum of product (l >> 1) & 15
        double v;
        if constexpr (sizeof(T) == 4) {
          float lo16[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) lo16[q] = 0.f;
          warp_sum_t<16>(acc, lo16);
          v = (double)acc[0] + (double)lo16[0];
        } else {
          warp_sum_t<16>(acc);
          v = acc[0];
        }
        const int q = (lane >> 1) & 15, a = ta * 4 + q / 4, bb = tb * 4 + q % 4;
        if ((lane & 1) == 0 && a <= bb && bb < nv) gacc[a * nv - a * (a - 1) / 2 + (bb - a)] += v;
      }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < npair; p += blockDim.x) t.gpart[ci * (long long)t.gstride + p] = gacc[p];
  }
}

template <typename T>
__global__ void k_eig_gram_reduce(const EigTask<T> *tasks, const int *rk_all) {
  const int b = blockIdx.x;
  const int rk = rk_all[b];
  if (rk == 0 || rk == kEigDone) return;
  const EigTask<T> &t = tasks[b];
  const int nv = t.st[0] + 1;
  const int npair = nv * (nv + 1) / 2;
  for (int p = threadIdx.x; p < npair; p += blockDim.x) {
    int a = 0, rem = p;
    while (rem >= nv - a) {
      rem -= nv - a;
      ++a;
    }
    const int bb = a + rem;
    double v = 0.0;
    for (int q = 0; q < t.nchunks; ++q) v += t.gpart[(long long)q * t.gstride + p];
    if (a == bb) v -= 1.0;
    t.E[(long long)bb * t.ld + a] = v;
    t.E[(long long)a * t.ld + bb] = v;
  }
}

// Gram block of the basis after a restart, from the projected quantities alone (one block per restarting
// task; launched before k_eig_reset, while st[0] still holds the old basis size nb).  The restart wrote
// V'[r] = sum_c V[c] Ys[c][r] (r < k; Ys = Y rounded to the vector type, as the restart applied it) and, when
// rk > 0, V'[k] = V[nb]; with the old Gram block G = I + E over V[0..nb):
//   V'[a].V'[b] = (Ys^T G Ys)[a][b]   (a, b < k).
// The column of V'[k], the newest vector, is measured by the next step's dot pass before any use
// (cgs_coefficients takes column j from g), as it would be for any new vector; it is written as zero here.
// Left out are the roundings of the restart's own sums: independent from element to element, they change a
// Gram entry by about eps / sqrt(n), far below the orthogonality the vectors' precision allows.  This
// replaces a pass over the k + 1 new vectors (k_eig_gram).
template <typename T>
__global__ void __launch_bounds__(kBlk) k_eig_gram_proj(const EigTask<T> *tasks, const int *rk_all, const double *Y_all,
                                                        int ld) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.x;
  const int rk = rk_all[b];
  if (rk == 0 || rk == kEigDone) return;
  const EigTask<T> &t = tasks[b];
  const int nb = t.st[0], n1 = nb + 1;
  const int k = rk > 0 ? rk : -rk;
  double *Eo = reinterpret_cast<double *>(smem_raw);  // old E over V[0..nb], column-major (leading dim n1)
  double *Ys = Eo + (size_t)n1 * n1;                    // nb x k: Ys[c + r nb]
  double *T1 = Ys + (size_t)nb * k;                     // nb x k: (I + E) Ys
  const double *Y = Y_all + (size_t)b * ld * ld;
  for (int e = threadIdx.x; e < n1 * n1; e += blockDim.x) {
    const int c = e / n1, r = e - c * n1;
    Eo[e] = t.E[(long long)c * t.ld + r];
  }
  for (int e = threadIdx.x; e < nb * k; e += blockDim.x) {
    const int r = e / nb, c = e - r * nb;
    Ys[e] = (double)(T)Y[c + (size_t)r * ld];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * k; e += blockDim.x) {
    const int r = e / nb, c = e - r * nb;
    double v = Ys[e];
    for (int d = 0; d < nb; ++d) v = fma(Eo[c + (size_t)d * n1], Ys[d + (size_t)r * nb], v);
    T1[e] = v;
  }
  __syncthreads();
  const int nv = rk > 0 ? k + 1 : k;
  for (int e = threadIdx.x; e < nv * nv; e += blockDim.x) {
    const int bb = e / nv, a = e - bb * nv;
    if (a > bb) continue;  // upper triangle, mirrored
    double v = 0.0;
    if (bb < k) {
      for (int c = 0; c < nb; ++c) v = fma(Ys[c + (size_t)a * nb], T1[c + (size_t)bb * nb], v);
      if (a == bb) v -= 1.0;
    }
    t.E[(long long)bb * t.ld + a] = v;
    t.E[(long long)a * t.ld + bb] = v;
  }
}

template <typename T>
void launch_eig_gram_proj(const EigTask<T> *tasks_dev, int ntasks, const int *rk, const double *Y, int ld,
                          cudaStream_t st) {
  const size_t sm = sizeof(double) * (size_t)3 * ld * ld;
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_eig_gram_proj<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_eig_gram_proj<T><<<ntasks, kBlk, sm, st>>>(tasks_dev, rk, Y, ld); note_launch();
}

template <typename T>
void launch_eig_gram(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, int ntasks, const int *rk,
                     cudaStream_t st) {
  if (kGramSmem > 48 * 1024) cudaFuncSetAttribute(k_eig_gram<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmem);
  k_eig_gram<T><<<grid_items(nchunks), kBlk, kGramSmem, st>>>(tasks_dev, chunk_task_dev, nchunks, rk); note_launch();
  k_eig_gram_reduce<T><<<ntasks, kBlk, 0, st>>>(tasks_dev, rk); note_launch();
}

// ================================================================ dense symmetric eigen-solver (one block per task)
// Cyclic Jacobi with a round-robin pairing (all np/2 rotations of a round are disjoint), FP64, on the
// np x np column-major matrix A (np even; a padding index stays decoupled); Q accumulates the rotations.
constexpr size_t kJacobiSmem = 96 * 1024;  // projected-matrix workspaces in shared memory up to this size

struct JacobiSmem {
  double cs[512], sn[512];
  int pp[512], qq[512];
  int rotated;  // rotations applied in the current sweep
};

// Cyclic Jacobi in the round-robin order: round r pairs the players at positions k and np - 1 - k, where
// position 0 holds player 0 and position i >= 1 holds ((i - 1 - r) mod (np - 1)) + 1 (a rotation of all
// but player 0 per round); the np / 2 rotations of a round touch disjoint rows and columns.
// Rutishauser's threshold: an off-diagonal entry that adding a hundred times it would not change either
// diagonal entry it couples (|a_pp| + 100 |a_pq| == |a_pp| and the same for a_qq) is set to zero and not
// rotated; the iteration ends after a sweep without rotations.  That stops at the rounding level of the
// matrix instead of at a fixed relative off-diagonal norm, which entries at rounding level (about
// n eps |A|) can keep above any bound fixed in advance.
__device__ int jacobi_core(double *A, double *Q, int np, JacobiSmem &sm) {
  int sweep = 0;
  for (; sweep < 60; ++sweep) {
    if (threadIdx.x == 0) sm.rotated = 0;
    __syncthreads();
    const int half = np / 2;
    for (int round = 0; round < np - 1; ++round) {
      for (int k = threadIdx.x; k < half; k += blockDim.x) {
        const int m = np - 1;
        int p = k == 0 ? 0 : ((k - 1 - round) % m + m) % m + 1;
        int q = ((np - 2 - k - round) % m + m) % m + 1;
        if (p > q) { int tmp = p; p = q; q = tmp; }
        sm.pp[k] = p;
        sm.qq[k] = q;
        double apq = A[p + (size_t)q * np];
        double app = A[p + (size_t)p * np], aqq = A[q + (size_t)q * np];
        double c = 1.0, s = 0.0;
        const double g = 100.0 * fabs(apq);
        if (fabs(app) + g == fabs(app) && fabs(aqq) + g == fabs(aqq)) {
          // negligible: zero it (this thread alone owns the pair in this round)
          A[p + (size_t)q * np] = 0.0;
          A[q + (size_t)p * np] = 0.0;
        } else {
          double th = (aqq - app) / (2.0 * apq);
          double tt = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
          c = 1.0 / sqrt(tt * tt + 1.0);
          s = tt * c;
          atomicAdd(&sm.rotated, 1);
        }
        sm.cs[k] = c;
        sm.sn[k] = s;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < half * np; e += blockDim.x) {  // rows: A <- J^T A
        int k = e / np, col = e % np;
        if (sm.sn[k] == 0.0) continue;
        int p = sm.pp[k], q = sm.qq[k];
        double c = sm.cs[k], s = sm.sn[k];
        double ap = A[p + (size_t)col * np], aq = A[q + (size_t)col * np];
        A[p + (size_t)col * np] = c * ap - s * aq;
        A[q + (size_t)col * np] = s * ap + c * aq;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < half * np; e += blockDim.x) {  // columns: A <- A J, Q <- Q J
        int k = e / np, row = e % np;
        if (sm.sn[k] == 0.0) continue;
        int p = sm.pp[k], q = sm.qq[k];
        double c = sm.cs[k], s = sm.sn[k];
        double ap = A[row + (size_t)p * np], aq = A[row + (size_t)q * np];
        A[row + (size_t)p * np] = c * ap - s * aq;
        A[row + (size_t)q * np] = s * ap + c * aq;
        double qp = Q[row + (size_t)p * np], qv = Q[row + (size_t)q * np];
        Q[row + (size_t)p * np] = c * qp - s * qv;
        Q[row + (size_t)q * np] = s * qp + c * qv;
      }
      __syncthreads();
    }
    if (sm.rotated == 0) break;  // uniform: read after the round's last barrier
    __syncthreads();             // every thread has read it before thread 0 clears it
  }
  return sweep;
}

// ---------------------------------------------------------------- projected eigenproblem of the restart
// One block per task, in two precisions: cyclic Jacobi in FP32 (Rutishauser's threshold, as jacobi_core) to the
// FP32 rounding level, then in FP64: the FP32 eigenvectors Q are made orthonormal by Newton-Schulz steps
// Q <- Q (3 I - Q^T Q) / 2 (each squares the orthogonality error), B = Q^T A Q is formed from the FP64 matrix,
// and FP64 Jacobi on B -- off-diagonal entries at the FP32 level, so one sweep of small rotations and one that
// finds none -- finishes eigenvalues and eigenvectors to the FP64 rounding level.  GB300 issues FP64 at a small
// fraction of its FP32 rate and the projected problem is solved once per restart cycle for every sector of
// a batch: the FP64 work is now about one sweep and a few small matrix products instead of every sweep.
// (One warp per task, without block barriers, measured slower: 620 us against 420 us for the FP64 block
// Jacobi, every round's index arithmetic and shared-memory round trips on one warp's critical path.)
struct JacSmem {
  float cs32[40], sn32[40];
  double cs[40], sn[40];
  int pp[40], qq[40];
  double red[kBlk / 32];
};

template <typename R>
__device__ int block_jacobi(R *A, R *Q, int np, R *cs, R *sn, int *pp, int *qq, int max_sweeps) {
  const int half = np / 2, m = np - 1;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int any = 0;
    for (int round = 0; round < np - 1; ++round) {
      for (int k = threadIdx.x; k < half; k += blockDim.x) {
        int p = k == 0 ? 0 : ((k - 1 - round) % m + m) % m + 1;
        int q = ((np - 2 - k - round) % m + m) % m + 1;
        if (p > q) {
          const int tmp = p;
          p = q;
          q = tmp;
        }
        pp[k] = p;
        qq[k] = q;
        const R apq = A[p + q * np], app = A[p + p * np], aqq = A[q + q * np];
        R c = (R)1, sn_ = (R)0;
        const R g = (R)100 * fabs(apq);
        if (fabs(app) + g == fabs(app) && fabs(aqq) + g == fabs(aqq)) {
          A[p + q * np] = (R)0;  // negligible (this thread alone owns the pair in this round)
          A[q + p * np] = (R)0;
        } else {
          const R th = (aqq - app) / ((R)2 * apq);
          const R tt = (th >= (R)0 ? (R)1 : (R)-1) / (fabs(th) + sqrt(th * th + (R)1));
          c = (R)1 / sqrt(tt * tt + (R)1);
          sn_ = tt * c;
          any = 1;
        }
        cs[k] = c;
        sn[k] = sn_;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < half * np; e += blockDim.x) {  // rows: A <- J^T A
        const int k = e / np, col = e - k * np;
        const R s_ = sn[k];
        if (s_ == (R)0) continue;
        const int p = pp[k], q = qq[k];
        const R c = cs[k], ap = A[p + col * np], aq = A[q + col * np];
        A[p + col * np] = c * ap - s_ * aq;
        A[q + col * np] = s_ * ap + c * aq;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < half * np; e += blockDim.x) {  // columns: A <- A J, Q <- Q J
        const int k = e / np, row = e - k * np;
        const R s_ = sn[k];
        if (s_ == (R)0) continue;
        const int p = pp[k], q = qq[k];
        const R c = cs[k];
        const R ap = A[row + p * np], aq = A[row + q * np];
        A[row + p * np] = c * ap - s_ * aq;
        A[row + q * np] = s_ * ap + c * aq;
        const R qp = Q[row + p * np], qv = Q[row + q * np];
        Q[row + p * np] = c * qp - s_ * qv;
        Q[row + q * np] = s_ * qp + c * qv;
      }
      __syncthreads();
    }
    if (!__syncthreads_or(any)) break;
  }
  return sweep;
}

// C = op(X) Y for np x np column-major matrices, op = transpose when TX (the block)
template <bool TX>
__device__ __forceinline__ void block_matmul(const double *X, const double *Y, double *C, int np) {
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
    const int c = e / np, r = e - c * np;
    double a = 0.0;
    for (int k = 0; k < np; ++k) a = fma(TX ? X[k + r * np] : X[r + k * np], Y[k + c * np], a);
    C[e] = a;
  }
  __syncthreads();
}

// A: nb x nb (from the upper triangle of Tm), eigenvalues ascending into theta, vectors into Y
// (column i = eigenvector i, leading dimension ld).  resid[i] = |beta_m * Y[nb-1][i]|.  Workspace 4 ld^2
// doubles per task: in shared memory when it fits, else work_all.
template <typename T>
__global__ void __launch_bounds__(kBlk) k_eig_jacobi(const EigTask<T> *tasks, double *theta_all, double *Y_all,
                                                     double *resid_all, int ld, double *work_all, int *status,
                                                     int in_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ JacSmem sm;
  const EigTask<T> &t = tasks[blockIdx.x];
  if (t.st[5]) return;  // finished sector (uniform)
  const int nb = t.st[0];
  const size_t per = (size_t)4 * ld * ld;
  double *A = in_smem ? reinterpret_cast<double *>(smem_raw) : work_all + (size_t)blockIdx.x * per;
  const int np = (nb + 1) & ~1;  // padded to even
  double *Q = A + (size_t)np * np, *Tq = Q + (size_t)np * np, *F = Tq + (size_t)np * np;
  float *A32 = reinterpret_cast<float *>(F), *Q32 = A32 + (size_t)np * np;
  double *theta = theta_all + (size_t)blockIdx.x * ld;
  double *Y = Y_all + (size_t)blockIdx.x * ld * ld;
  double *resid = resid_all + (size_t)blockIdx.x * ld;
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
    const int c = e / np, r = e - c * np;
    double v = 0.0;
    if (r < nb && c < nb) v = r <= c ? t.Tm[(long long)c * t.ld + r] : t.Tm[(long long)r * t.ld + c];
    A[e] = v;
    A32[e] = (float)v;
    Q32[e] = r == c ? 1.f : 0.f;
  }
  __syncthreads();
  const int s32 = block_jacobi<float>(A32, Q32, np, sm.cs32, sm.sn32, sm.pp, sm.qq, 40);
  // FP64: Q from the FP32 eigenvectors, made orthonormal: Newton-Schulz steps G = Q^T Q, Q <- Q (3 I - G) / 2
  // until max |G - I| reaches the FP64 rounding level.  The FP32 rotations leave an orthogonality error that
  // grows with their number (about 1e-6 after a few hundred; one step left 6e-12, and eigenvalues off by
  // 1e-11 relative): two or three steps.
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) Q[e] = (double)Q32[e];
  __syncthreads();
  for (int it = 0; it < 5; ++it) {
    block_matmul<true>(Q, Q, Tq, np);
    double dev = 0.0;
    for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
      const int c = e / np, r = e - c * np;
      const double g = Tq[e] - (r == c ? 1.0 : 0.0);
      dev = fmax(dev, fabs(g));
      Tq[e] = (r == c ? 1.0 : 0.0) - 0.5 * g;  // (3 I - G) / 2
    }
    for (int o = 16; o > 0; o >>= 1) dev = fmax(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5] = dev;
    __syncthreads();
    double d = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) d = fmax(d, sm.red[w]);
    __syncthreads();
    if (d <= 1e-15 * np) break;  // uniform across the block
    block_matmul<false>(Q, Tq, F, np);  // F overwrites A32 / Q32, no longer needed
    for (int e = threadIdx.x; e < np * np; e += blockDim.x) Q[e] = F[e];
    __syncthreads();
  }
  // B = Q^T A Q (symmetrised) into A, then FP64 Jacobi on it, accumulating into Q
  block_matmul<false>(A, Q, Tq, np);
  block_matmul<true>(Q, Tq, F, np);
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
    const int c = e / np, r = e - c * np;
    A[e] = 0.5 * (F[e] + F[c + r * np]);
  }
  __syncthreads();
  const int s64 = block_jacobi<double>(A, Q, np, sm.cs, sm.sn, sm.pp, sm.qq, 30);
  // sort eigenvalues ascending (rank by value, ties by index), skipping the padding slot
  const double beta_m = (nb > 0 && nb < t.ld && nb < t.n) ? t.Tm[(long long)(nb - 1) * t.ld + nb] : 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const double vi = A[i + (size_t)i * np];
    int rank = 0;
    for (int k = 0; k < nb; ++k) {
      const double vk = A[k + (size_t)k * np];
      if (vk < vi || (vk == vi && k < i)) ++rank;
    }
    theta[rank] = vi;
    for (int r = 0; r < nb; ++r) Y[r + (size_t)rank * ld] = Q[r + (size_t)i * np];
    resid[rank] = fabs(beta_m * Q[(nb - 1) + (size_t)i * np]);
  }
  if (threadIdx.x == 0) status[blockIdx.x] = s32 * 100 + s64;
}

// ================================================================ FP64 Rayleigh-Ritz refinement of FP32 Ritz vectors
// For k vectors X (FP64 copies of the FP32 Ritz vectors) and W = H X (FP64 H*v):
// G = X^T X, M = X^T W; G = L L^T; C = L^-1 M L^-T = Z diag(theta) Z^T; Y = L^-T Z; X' = X Y.
// The refined eigenvalues carry the square of the FP32 vectors' error.
__global__ void __launch_bounds__(kBlk) k_rr_gram(const RrTask *tasks, const int *item_task, int nitems) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const RrTask &t = tasks[item_task[it]];
    const long long li = it - t.item_begin;
    const long long lo = li * (long long)kItemElems;
    long long hi = lo + kItemElems;
    if (hi > t.n) hi = t.n;
    const int k = t.k;
    for (int q = warp; q < 2 * k * k; q += nwarp) {
      const int which = q / (k * k), r = q % (k * k), a = r % k, b = r / k;
      const double *xa = t.X + (long long)a * t.n;
      const double *yb = (which ? t.W : t.X) + (long long)b * t.n;
      double s = 0.0;
      for (long long i = lo + lane; i < hi; i += 32) s = fma(xa[i], yb[i], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) t.part[li * 2 * k * k + q] = s;
    }
  }
}

__global__ void k_rr_small(const RrTask *tasks, double *work) {
  const RrTask &t = tasks[blockIdx.x];
  const int k = t.k;
  const int np = (k + 1) & ~1;
  double *G = work + (size_t)blockIdx.x * 4 * 64 * 64;
  double *M = G + 64 * 64, *A = M + 64 * 64, *Q = A + 64 * 64;
  __shared__ JacobiSmem sm;
  for (int q = threadIdx.x; q < 2 * k * k; q += blockDim.x) {
    double s = 0.0;
    for (int li = 0; li < t.nitems; ++li) s += t.part[(long long)li * 2 * k * k + q];
    if (q < k * k) G[q] = s; else M[q - k * k] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // symmetrise M, Cholesky G = L L^T in place (lower), C = L^-1 M L^-T into A (np x np, padded)
    for (int a = 0; a < k; ++a)
      for (int b = a + 1; b < k; ++b) {
        double v = 0.5 * (M[a + b * k] + M[b + a * k]);
        M[a + b * k] = M[b + a * k] = v;
      }
    bool ok = true;
    for (int j = 0; j < k; ++j) {
      double d = G[j + j * k];
      for (int p = 0; p < j; ++p) d -= G[j + p * k] * G[j + p * k];
      if (!(d > 0)) { ok = false; d = 1.0; }
      d = sqrt(d);
      G[j + j * k] = d;
      for (int i = j + 1; i < k; ++i) {
        double v = G[i + j * k];
        for (int p = 0; p < j; ++p) v -= G[i + p * k] * G[j + p * k];
        G[i + j * k] = v / d;
      }
    }
    t.status[0] = ok ? 0 : 1;
    // B = L^-1 M  (column by column forward substitution), then C = B L^-T = (L^-1 B^T)^T
    for (int c = 0; c < k; ++c)
      for (int i = 0; i < k; ++i) {
        double v = M[i + c * k];
        for (int p = 0; p < i; ++p) v -= G[i + p * k] * A[p + c * np];
        A[i + c * np] = v / G[i + i * k];
      }
    for (int c = 0; c < k; ++c)  // rows of C: C[c][:] = L^-1 B[c][:]^T
      for (int i = 0; i < k; ++i) {
        double v = A[c + i * np];
        for (int p = 0; p < i; ++p) v -= G[i + p * k] * Q[c + p * np];
        Q[c + i * np] = v / G[i + i * k];
      }
    for (int c = 0; c < np; ++c)
      for (int i = 0; i < np; ++i) {
        double v = (c < k && i < k) ? 0.5 * (Q[c + i * np] + Q[i + c * np]) : 0.0;
        A[i + c * np] = v;
      }
    for (int c = 0; c < np; ++c)
      for (int i = 0; i < np; ++i) Q[i + c * np] = i == c ? 1.0 : 0.0;
  }
  __syncthreads();
  jacobi_core(A, Q, np, sm);
  // sort, then Y = L^-T Z (back substitution with L^T)
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    double vi = A[i + (size_t)i * np];
    int rank = 0;
    for (int q = 0; q < k; ++q) {
      double vq = A[q + (size_t)q * np];
      if (vq < vi || (vq == vi && q < i)) ++rank;
    }
    t.theta[rank] = vi;
    double *y = t.Y + (size_t)rank * k;
    for (int r = k - 1; r >= 0; --r) {
      double v = Q[r + (size_t)i * np];
      for (int p = r + 1; p < k; ++p) v -= G[p + r * k] * y[p];
      y[r] = v / G[r + r * k];
    }
  }
}

__global__ void __launch_bounds__(kBlk) k_rr_rotate(const RrTask *tasks, const int *item_task, int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const RrTask &t = tasks[item_task[it]];
    if (t.status[0]) continue;  // Gram matrix not positive definite: keep the FP32 vectors
    const long long li = it - t.item_begin;
    const long long lo = li * (long long)kItemElems;
    long long hi = lo + kItemElems;
    if (hi > t.n) hi = t.n;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x)
      for (int r = 0; r < t.k; ++r) {
        double acc = 0.0;
        for (int c = 0; c < t.k; ++c) acc = fma(t.Y[c + (size_t)r * t.k], t.X[(long long)c * t.n + i], acc);
        t.out[(long long)r * t.n + i] = (float)acc;
      }
  }
}

void launch_rr(const RrTask *tasks_dev, const int *item_task_dev, int nitems, int ntasks, double *work, cudaStream_t st) {
  k_rr_gram<<<grid_items(nitems), kBlk, 0, st>>>(tasks_dev, item_task_dev, nitems); note_launch();
  k_rr_small<<<ntasks, kBlk, 0, st>>>(tasks_dev, work); note_launch();
  k_rr_rotate<<<grid_items(nitems), kBlk, 0, st>>>(tasks_dev, item_task_dev, nitems); note_launch();
}

template <typename T>
void launch_eig_jacobi(const EigTask<T> *tasks_dev, int ntasks, double *theta, double *Y, double *resid, int ld,
                       double *work, int *status, cudaStream_t st) {
  // work: ntasks x 4 ld^2 doubles (used when one task's workspace does not fit in shared memory)
  const size_t want = (size_t)4 * ld * ld * sizeof(double);
  const size_t sm = want <= kJacobiSmem ? want : 0;
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_eig_jacobi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_eig_jacobi<T><<<ntasks, kBlk, sm, st>>>(tasks_dev, theta, Y, resid, ld, work, status, sm ? 1 : 0);
  note_launch();
}

// Thick restart / Ritz vectors: for task b with keep[b] = k > 0: outV[b][i] = V Y[:, i] (i < k) and
// outV[b][k] = V[nb] (the residual), columns ldv apart (the next basis); keep[b] = -k: outV[b][i] = V Y[:, i]
// for i < k only, packed n apart (the eigenvectors); 0: nothing.
// Each chunk is taken in sub-chunks of one 16-byte group per thread; the basis columns' slices of a
// sub-chunk stream through shared-memory stages, four columns per stage and barrier (bulk copies issued
// by a producer warp, ProdPipe), and each thread accumulates up to RC outputs of its group in registers
// (FP32 FMAs in FP32 mode), k > RC in further passes.  Y is
// staged in shared memory in vector precision behind the stages.
template <typename T>
struct RstGeom {
  static constexpr int VEC = 16 / (int)sizeof(T);
  static constexpr int SUB = VEC * kBlk;          // elements of a sub-chunk
  static constexpr int NSUB = kCgsChunk / SUB;    // sub-chunks of a chunk
  static constexpr int RC = sizeof(T) == 4 ? 12 : 8;  // outputs per pass
  static constexpr int CPS = 4;                   // column slices per stage (one barrier)
};
template <typename T>
using RstPipe = ProdPipe<6, RstGeom<T>::CPS * RstGeom<T>::SUB * (int)sizeof(T)>;

template <typename T>
struct RstIssue {
  const EigTask<T> *tasks;
  const int *chunk_task, *keep;
  int nchunks, it, sub, r0, c;
  __device__ __forceinline__ bool operator()(unsigned dst, unsigned bar) {
    using RG = RstGeom<T>;
    while (it < nchunks) {
      const int b = chunk_task[it];
      const EigTask<T> &t = tasks[b];
      const int kk = keep[b], k = kk > 0 ? kk : -kk, nb = t.st[0];
      long long lo, hi;
      chunk_range(t.n, it - t.chunk_begin, lo, hi);
      const long long s0 = lo + (long long)sub * RG::SUB;
      if (kk == 0 || sub >= RG::NSUB || s0 >= hi) {  // next chunk
        it += gridDim.x;
        sub = r0 = c = 0;
        continue;
      }
      if (r0 >= k) {  // next sub-chunk
        ++sub;
        r0 = c = 0;
        continue;
      }
      if (c >= nb) {  // next pass of outputs
        r0 += RG::RC;
        c = 0;
        continue;
      }
      // up to CPS columns' slices of the sub-chunk, one barrier
      const long long e = min(hi, s0 + RG::SUB);
      const unsigned bytes = (unsigned)((((e - s0) * (long long)sizeof(T)) + 15) & ~15LL);  // inside the padding
      const int n = min(RG::CPS, nb - c);
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      unsigned long long state;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;\n" : "=l"(state) : "r"(bar), "r"(bytes * n) : "memory");
      for (int i = 0; i < n; ++i)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                         dst + (unsigned)(i * RG::SUB * (int)sizeof(T))),
                     "l"(t.V + (long long)(c + i) * t.ldv + s0), "r"(bytes), "r"(bar)
                     : "memory");
      c += n;
      return true;
    }
    return false;
  }
};

template <typename T>
__global__ void __launch_bounds__(kBlk + 32, 2) k_eig_restart(const EigTask<T> *tasks, const int *chunk_task, int nchunks,
                                                           const int *keep, const double *Y_all, int ld, T *const *outV) {
  using RG = RstGeom<T>;
  constexpr int VEC = RG::VEC, RC = RG::RC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T *ys = reinterpret_cast<T *>(smem_raw + RstPipe<T>::SMEM);  // [nb][k] row-major: ys[c * k + r] = Y[c][r]
  RstPipe<T> pipe;
  pipe.init(smem_raw);
  if (threadIdx.x >= kBlk) {  // the producer warp
    RstIssue<T> iss{tasks, chunk_task, keep, nchunks, (int)blockIdx.x, 0, 0, 0};
    pipe.produce(iss);
    return;
  }
  int cur_b = -1;
  for (int it = blockIdx.x; it < nchunks; it += gridDim.x) {
    const int b = chunk_task[it];
    const EigTask<T> &t = tasks[b];
    const int kk = keep[b];
    if (kk == 0) continue;
    const int k = kk > 0 ? kk : -kk;
    const int nb = t.st[0];
    const long long ldo = kk > 0 ? t.ldv : t.n;  // next basis (padded columns) or packed Ritz vectors
    const bool vec_out = ((ldo * (long long)sizeof(T)) & 15) == 0;
    if (b != cur_b) {
      cgs_csync();
      const double *Y = Y_all + (size_t)b * ld * ld;
      for (int e = threadIdx.x; e < nb * k; e += kBlk) {
        int c = e / k, r = e % k;
        ys[e] = (T)Y[c + (size_t)r * ld];
      }
      cgs_csync();
      cur_b = b;
    }
    T *out = outV[b];
    long long lo, hi;
    chunk_range(t.n, it - t.chunk_begin, lo, hi);
    for (int sub = 0; sub < RG::NSUB; ++sub) {
      const long long s0 = lo + (long long)sub * RG::SUB;
      if (s0 >= hi) break;
      const long long i = s0 + (long long)VEC * threadIdx.x;  // this thread's group
      for (int r0 = 0; r0 < k; r0 += RC) {
        T acc[RC][VEC];
#pragma unroll
        for (int q = 0; q < RC; ++q)
#pragma unroll
          for (int v = 0; v < VEC; ++v) acc[q][v] = (T)0;
        for (int c0 = 0; c0 < nb; c0 += RG::CPS) {
          // padding elements of a slice hold arbitrary bits; their outputs are not stored
          const unsigned char *stg = pipe.take();
          const int n = min(RG::CPS, nb - c0);
#pragma unroll
          for (int i = 0; i < RG::CPS; ++i) {
            if (i >= n) break;
            const Lanes<T> x = *reinterpret_cast<const Lanes<T> *>(stg + i * RG::SUB * (int)sizeof(T) + 16 * threadIdx.x);
            const T *yr = ys + (c0 + i) * k + r0;
#pragma unroll
            for (int q = 0; q < RC; ++q) {
              if (r0 + q < k) {
                const T y = yr[q];
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[q][v] = fma(y, x.v[v], acc[q][v]);
              }
            }
          }
          pipe.release();
        }
        if (i < hi) {
#pragma unroll
          for (int q = 0; q < RC; ++q) {
            if (r0 + q < k) {
              T *o = out + (long long)(r0 + q) * ldo + i;
              if (vec_out && i + VEC <= hi) {
                store_lanes(o, acc[q]);
              } else {
#pragma unroll
                for (int v = 0; v < VEC; ++v)
                  if (i + v < hi) o[v] = acc[q][v];
              }
            }
          }
        }
      }
      if (kk > 0 && i < hi) {  // the residual becomes basis vector k
        const Lanes<T> rq = load16(t.V + (long long)nb * t.ldv + i);
        store_lanes(out + (long long)k * ldo + i, rq.v);
      }
    }
  }
  pipe.finish();
}

template <typename T>
void launch_eig_restart(const EigTask<T> *tasks_dev, const int *chunk_task_dev, int nchunks, const int *keep,
                        const double *Y, int ld, T *const *outV, cudaStream_t st) {
  const size_t sm = RstPipe<T>::SMEM + sizeof(T) * (size_t)ld * ld;
  cudaFuncSetAttribute(k_eig_restart<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_eig_restart<T><<<occupancy_grid((const void *)k_eig_restart<T>, kBlk + 32, sm, nchunks), kBlk + 32, sm, st>>>(
      tasks_dev, chunk_task_dev, nchunks, keep, Y, ld, outV);
  note_launch();
}

// After a restart: projected matrix = diag(theta[0..k)), basis size k (or k-1 with a pending random
// vector when rk < 0, the multiplicity check), mode and draw counter updated; rk == 0: untouched;
// rk == kEigDone: the sector finished, every later kernel of the batch skips it.
template <typename T>
__global__ void k_eig_reset(const EigTask<T> *tasks, const int *rk_all, const double *theta_all, int ld) {
  const int b = blockIdx.x;
  const int rk = rk_all[b];
  if (rk == 0) return;
  const EigTask<T> &t = tasks[b];
  if (rk == kEigDone) {
    if (threadIdx.x == 0) {
      t.st[2] = 1;
      t.st[4] = 0;
      t.st[5] = 1;
    }
    return;
  }
  const int k = rk > 0 ? rk : -rk;
  const double *theta = theta_all + (size_t)b * ld;
  for (int e = threadIdx.x; e < t.ld * t.ld; e += blockDim.x) {
    int r = e % t.ld, c = e / t.ld;
    t.Tm[e] = (r == c && r < k) ? theta[r] : 0.0;
  }
  if (threadIdx.x == 0) {
    const int draws = t.st[3];
    t.st[0] = rk > 0 ? k : k - 1;
    t.st[1] = rk > 0 ? 0 : 1;
    t.st[2] = 0;
    t.st[3] = rk > 0 ? draws : draws + 1;
    t.st[4] = 0;
  }
}

template <typename T>
void launch_eig_reset(const EigTask<T> *tasks_dev, int ntasks, const int *rk, const double *theta, int ld,
                      cudaStream_t st) {
  k_eig_reset<T><<<ntasks, kBlk, 0, st>>>(tasks_dev, rk, theta, ld); note_launch();
}

// ================================================================ a / a+, diagonal operators
template <typename T>
__global__ void k_a_adag(SectorOp<T> src, SectorOp<T> dst, int im, int annihilate, const T *in, T *out, int accumulate,
                         T weight) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= dst.dim) return;
  const state_t s1 = sector_state(dst, i);
  const state_t bit = 1ll << (dst.ip - 1 - im);
  T v = (T)0;
  const bool has = (s1 & bit) != 0;
  if (annihilate ? !has : has) {
    const state_t s0 = annihilate ? (s1 + bit) : (s1 - bit);
    const int sign = parity_sign(s0, im, dst.ip);
    v = (T)sign * in[sector_index(src, s0)];
  }
  if (weight != (T)1) v = weight * v;
  out[i] = accumulate ? out[i] + v : v;
}

template <typename T>
void launch_a_adag(const SectorOp<T> &src, const SectorOp<T> &dst, int im, int annihilate, const T *in, T *out,
                   int accumulate, cudaStream_t st, double weight) {
  if (dst.dim == 0) return;
  k_a_adag<T><<<(unsigned)((dst.dim + 255) / 256), 256, 0, st>>>(src, dst, im, annihilate, in, out, accumulate,
                                                                 (T)weight);
  note_launch();
}

template <typename T>
__global__ void k_diag_op(SectorOp<T> op, int kind, int mu, int nu, const T *in, T *out) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= op.dim) return;
  const state_t s = sector_state(op, i);
  auto act = [&](int o) -> T {
    int up = occ(s, o, op.ip), dn = occ(s, o + op.ns, op.ip);
    return kind == 0 ? (T)(0.5 * (up - dn)) : (T)(up + dn);
  };
  T f = act(mu);
  if (nu >= 0) f = f + act(nu);
  out[i] = f * in[i];
}

template <typename T>
void launch_diag_op(const SectorOp<T> &op, int opkind, int mu, int nu, const T *in, T *out, cudaStream_t st) {
  if (op.dim == 0) return;
  k_diag_op<T><<<(unsigned)((op.dim + 255) / 256), 256, 0, st>>>(op, opkind, mu, nu, in, out); note_launch();
}

// ================================================================ small vector helpers
template <typename T>
__global__ void k_dot_partials(const T *a, const T *b, long long n, double *partial) {
  __shared__ double red[kBlk / 32];
  DotAcc acc;
  dot_init(acc);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dot_add(acc, a[i], b[i]);
  double s = block_sum<kBlk>(dot_value(acc), red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <typename T>
void launch_dot_partials(const T *a, const T *b, long long n, double *partial, int nparts, cudaStream_t st) {
  k_dot_partials<T><<<nparts, kBlk, 0, st>>>(a, b, n, partial); note_launch();
}

__global__ void k_reduce(const double *p, int n, double *out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += p[i];
    *out = s;
  }
}

void launch_reduce(const double *partial, int nparts, double *out, cudaStream_t st) {
  k_reduce<<<1, 32, 0, st>>>(partial, nparts, out); note_launch();
}

template <typename T>
__global__ void k_scale(T *x, long long n, const double *norm2, int divide_sqrt) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = *norm2;
  const T d = (T)(divide_sqrt ? sqrt(v) : v);
  x[i] = x[i] / d;
}

template <typename T>
void launch_scale(T *x, long long n, const double *norm2, int divide_sqrt, cudaStream_t st) {
  if (n <= 0) return;
  k_scale<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, norm2, divide_sqrt); note_launch();
}

template <typename T>
__global__ void k_convert(const double *in, T *out, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)in[i];
}
template <typename T>
void launch_convert(const double *in, T *out, long long n, cudaStream_t st) {
  if (n <= 0) return;
  k_convert<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n); note_launch();
}
template <typename T>
__global__ void k_to_double(const T *in, double *out, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}
template <typename T>
void launch_to_double(const T *in, double *out, long long n, cudaStream_t st) {
  if (n <= 0) return;
  k_to_double<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n); note_launch();
}

// ================================================================ continued fraction
// dl_i = z - alpha_i*isign; det_{n-1} = dl_{n-1}; det_{n-2} = dl_{n-2} dl_{n-1} - beta_{n-1}^2;
// det_i = dl_i det_{i+1} - beta_{i+1}^2 det_{i+2}, rescaling det_i and det_{i+1} by 1000/FLT_MAX when
// |det_i| > FLT_MAX/2 (i != 0); result = norm * expb * det_1 / det_0 (n == 1: norm * expb / dl_0).
// thread per frequency, jobs in order (deterministic accumulation)
// One continued fraction per (job, omega) pair (the symmetrised pair of a bosonic job summed), into
// res[q * nw + w]: every SM busy, where one thread per omega over all jobs left most of the GPU idle.
__global__ void k_cf_eval(const CfJob *jobs, int njobs, const double *omega, int nw, double beta_T, int real,
                          double2 *res) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)njobs * nw) return;
  const int q = (int)(t / nw), w = (int)(t - (long long)q * nw);
  const CfJob &jb = jobs[q];
  // Lanczos::freq_point (Lanczos.h:146-148): i w on the Matsubara mesh, w + i pi / beta on the real one
  const double2 zw = real ? make_double2(omega[w], M_PI / beta_T) : make_double2(0.0, omega[w]);
  const int nl = jb.state[1];
  const double de = jb.E - jb.E0;
  const double expb = (beta_T * de > 25) ? 0.0 : exp(-beta_T * de);
  const double scale = jb.expectation * expb;
  double2 r = make_double2(0.0, 0.0);
  if (!jb.sym) {
    r = frac_point(jb.alpha, jb.beta, nl, jb.isign, scale, make_double2(jb.E * jb.isign + zw.x, zw.y));
  } else if (!(w == 0 && !real)) {
    const double2 r1 = frac_point(jb.alpha, jb.beta, nl, jb.isign, scale, make_double2(jb.E * jb.isign + zw.x, zw.y));
    const double2 r2 = frac_point(jb.alpha, jb.beta, nl, jb.isign, scale, make_double2(jb.E * jb.isign - zw.x, -zw.y));
    r = make_double2(r1.x + r2.x, r1.y + r2.y);
  }
  res[t] = r;
}

// The jobs' fractions added into their outputs in job order per omega, so every output sums its terms in the
// same order (and with the same expressions) as a loop over the jobs would.
__global__ void k_cf_sum(const CfJob *jobs, int njobs, int nw, double beta_T, int real, const double2 *res) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  for (int q = 0; q < njobs; ++q) {
    const CfJob &jb = jobs[q];
    double *o = jb.out + 2 * (long long)w * jb.out_stride;
    if (jb.sym && w == 0 && !real) {
      const double de = jb.E - jb.E0;
      const double expb = (beta_T * de > 25) ? 0.0 : exp(-beta_T * de);
      o[0] -= jb.expectation * beta_T * expb;
    } else {
      const double2 r = res[(long long)q * nw + w];
      o[0] += r.x;
      o[1] += r.y;
    }
  }
}

void launch_cf(const CfJob *jobs_dev, int njobs, const double *omega, int nw, double beta_T, int real, double2 *res,
               cudaStream_t st) {
  if (njobs <= 0) return;
  const long long n = (long long)njobs * nw;
  k_cf_eval<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(jobs_dev, njobs, omega, nw, beta_T, real, res); note_launch();
  k_cf_sum<<<(nw + 127) / 128, 128, 0, st>>>(jobs_dev, njobs, nw, beta_T, real, res); note_launch();
}

// chi(w_0) -= 2 sum_{n>=1} (Re chi_n - c2/w^2 - c4/w^4) + 2 tail - avg^2 beta, c2/c4 from the last two points
__global__ void k_chi_tail(double *chi, long long stride, int nw, const double *om, double beta, double avg) {
  // the terms' quotients are formed in parallel a chunk at a time; one thread then adds them in index order with
  // the expressions of the sequential sum, so the result is that sum's to the last bit
  constexpr int kChunk = 256;
  __shared__ double re_s[kChunk], q2_s[kChunk], q4_s[kChunk];
  if (nw < 3) return;
  auto re = [&](int w) { return chi[2 * (long long)w * stride]; };
  const int f = nw - 1;
  double om1 = om[f], om2 = om[f - 1];
  double om1_2 = om1 * om1, om2_2 = om2 * om2;
  double g1 = re(f), g2 = re(f - 1);
  double c2 = -(g2 * om2_2 * om2_2 - g1 * om1_2 * om1_2) / (om1_2 - om2_2);
  double c4 = -(g1 * om1_2 * om1_2 * om2_2 - g2 * om2_2 * om2_2 * om1_2) / (om1_2 - om2_2);
  double s = 0.0;
  for (int k0 = 1; k0 < nw; k0 += kChunk) {
    const int k = k0 + (int)threadIdx.x;
    if (threadIdx.x < kChunk && k < nw) {
      const double o = om[k];
      re_s[threadIdx.x] = re(k);
      q2_s[threadIdx.x] = c2 / (o * o);
      q4_s[threadIdx.x] = c4 / (o * o * o * o);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int n = min(kChunk, nw - k0);
      for (int j = 0; j < n; ++j) s = s + re_s[j] - q2_s[j] - q4_s[j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double tail = c2 * beta * beta / 24.0 + c4 * beta * beta * beta * beta / 1440.0;
    chi[0] -= 2 * s + 2 * tail - avg * avg * beta;
  }
}

void launch_chi_tail(double *chi, long long stride, int nw, const double *omega, double beta_T, double avg,
                     cudaStream_t st) {
  k_chi_tail<<<1, 256, 0, st>>>(chi, stride, nw, omega, beta_T, avg); note_launch();
}

// ================================================================ instantiations
#define EDGPU_INST(T)                                                                                              \
  template void launch_lz_step<T>(const LzTask<T> *, const int *, int, int, int, MvShape, cudaStream_t);           \
  template void prepare_eig_step<T>(MvShape);                                                                      \
  template void launch_eig_step<T>(const EigTask<T> *, const int *, int, const int *, int, const int *, int, int,  \
                                   MvShape, cudaStream_t);                                                         \
  template void launch_eig_jacobi<T>(const EigTask<T> *, int, double *, double *, double *, int, double *, int *,  \
                                     cudaStream_t);                                                                \
  template void launch_eig_restart<T>(const EigTask<T> *, const int *, int, const int *, const double *, int,      \
                                      T *const *, cudaStream_t);                                                   \
  template void launch_eig_random<T>(const EigTask<T> *, const int *, int, cudaStream_t);                          \
  template void prepare_cgs<T>();                                                                                  \
  template void launch_cgs_dot<T>(const EigTask<T> *, const int *, int, cudaStream_t);                             \
  template void launch_cgs_coef<T>(const EigTask<T> *, const int *, const int *, int, cudaStream_t);               \
  template void launch_cgs_upd<T>(const EigTask<T> *, const int *, int, cudaStream_t);                             \
  template void launch_eig_gram<T>(const EigTask<T> *, const int *, int, int, const int *, cudaStream_t);         \
  template void launch_eig_gram_proj<T>(const EigTask<T> *, int, const int *, const double *, int, cudaStream_t);  \
  template void launch_eig_reset<T>(const EigTask<T> *, int, const int *, const double *, int, cudaStream_t);      \
  template void launch_a_adag<T>(const SectorOp<T> &, const SectorOp<T> &, int, int, const T *, T *, int,          \
                                 cudaStream_t, double);                                                            \
  template void launch_diag_op<T>(const SectorOp<T> &, int, int, int, const T *, T *, cudaStream_t);              \
  template void launch_dot_partials<T>(const T *, const T *, long long, double *, int, cudaStream_t);              \
  template void launch_scale<T>(T *, long long, const double *, int, cudaStream_t);                                \
  template void launch_convert<T>(const double *, T *, long long, cudaStream_t);                                   \
  template void launch_to_double<T>(const T *, double *, long long, cudaStream_t);
EDGPU_INST(float)
EDGPU_INST(double)
// float-float recurrences (the mixed mode's Green's functions and susceptibilities on spin-resolved sectors)
template void launch_lz_step<ffloat>(const LzTask<ffloat> *, const int *, int, int, int, MvShape, cudaStream_t);
template void launch_convert<ffloat>(const double *, ffloat *, long long, cudaStream_t);

}  // namespace edgpu
