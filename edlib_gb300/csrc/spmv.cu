// Hamiltonian-times-vector kernels for the three storages, batched over work items.
//
// * SRS   -- SpinResolvedStorage::av (include/edlib/SpinResolvedStorage.h:58-115): the sector vector is the
//            row-major N_up x N_dn matrix X (d fastest) and
//            Y = D o X + X H_dn^T + H_up X + H_loc X,
//            accumulated per element in the reference order (diagonal, down hops, up hops, interaction).
//            A work item is a group of up-rows; its rows of X are staged in shared memory so the H_dn
//            gather reads shared memory, and the H_up term reads whole rows of X (coalesced in d).
//            The off-diagonal interaction (H_loc) is applied matrix-free from the transition list.
// * CRS   -- CRSStorage::av (include/edlib/CRSStorage.h:57-64): one thread per row, diagonal first.
// * SOCRS -- SOCRSStorage::av (include/edlib/SOCRSStorage.h:46-87): matrix-free; each row re-derives its
//            state from the combinadic tables, tests every transition, ranks the target with ninv and
//            takes the fermion sign from one popc; nothing but the tables is stored.
// Every kernel optionally emits <x, y> per item (FP64 / float-float accumulation, fixed order).
#include "edgpu_kernels.h"

namespace edgpu {

constexpr int kMvBlock = 256;

template <typename T>
__device__ __forceinline__ T transitions_term(const SectorOp<T> &op, state_t s, const Transition *L, const T *vals, int nL,
                                              const T *__restrict__ x, T acc) {
  for (int q = 0; q < nL; ++q) {
    if (!trans_valid(L[q], s, op.ip)) continue;
    int sign;
    state_t k = trans_apply(L[q], s, op.ip, sign);
    acc += vals[q] * (T)sign * x[sector_index(op, k)];
  }
  return acc;
}

// One item of a sector: y[lo:hi) = (H x)[lo:hi) + c z[lo:hi); accumulates <x, y> into acc.
template <typename T>
__device__ void mv_item(const SectorOp<T> &op, int srs_rows, long long li, const T *__restrict__ x, T *__restrict__ y,
                        const T *__restrict__ z, T c, bool want_dot, DotAcc &acc, T *xs, int xs_cap) {
  long long lo, hi;
  item_range(op, srs_rows, li, lo, hi);
  const int tid = threadIdx.x;
  if (op.storage == kSRS) {
    const int Nd = op.dn_rows;
    const long long u0 = lo / Nd;
    const int nel = (int)(hi - lo);
    const bool staged = nel <= xs_cap;
    __syncthreads();
    if (staged)
      for (int e = tid; e < nel; e += blockDim.x) xs[e] = x[lo + e];
    __syncthreads();
    const T *xr = staged ? xs : x + lo;
    for (int e = tid; e < nel; e += blockDim.x) {
      const int r = e / Nd;
      const int d = e - r * Nd;
      const long long u = u0 + r;
      const long long gi = lo + e;
      const T xv = xr[e];
      T v = op.diag[gi] * xv;
      if (z) v = v + c * z[gi];
      const T *xrow = xr + (long long)r * Nd;
      for (int j = op.dn_rp[d]; j < op.dn_rp[d + 1]; ++j) v += op.dn_val[j] * xrow[op.dn_col[j]];
      for (int j = op.up_rp[u]; j < op.up_rp[u + 1]; ++j) v += op.up_val[j] * x[(long long)op.up_col[j] * Nd + d];
      if (op.nV) {
        state_t s = ((state_t)op.up_basis[u] << op.ns) | (state_t)op.dn_basis[d];
        v = transitions_term(op, s, op.V_, op.V_val, op.nV, x, v);
      }
      y[gi] = v;
      if (want_dot) dot_add(acc, xv, v);
    }
  } else if (op.storage == kCRS) {
    for (long long i = lo + tid; i < hi; i += blockDim.x) {
      T v = z ? c * z[i] : (T)0;
      for (long long j = op.crs_rp[i]; j < op.crs_rp[i + 1]; ++j) v = v + op.crs_val[j] * x[op.crs_col[j]];
      y[i] = v;
      if (want_dot) dot_add(acc, x[i], v);
    }
  } else {
    for (long long i = lo + tid; i < hi; i += blockDim.x) {
      const state_t s = sector_state(op, i);
      const T xv = x[i];
      T v = op.diag[i] * xv;
      if (z) v = v + c * z[i];
      v = transitions_term(op, s, op.T_, op.T_val, op.nT, x, v);
      if (op.nV) v = transitions_term(op, s, op.V_, op.V_val, op.nV, x, v);
      y[i] = v;
      if (want_dot) dot_add(acc, xv, v);
    }
  }
}

template <typename T>
__device__ __forceinline__ void emit_dot(bool want, DotAcc &acc, double *dst, double *red) {
  if (!want) return;  // uniform across the block
  double s = block_sum<kMvBlock>(dot_value(acc), red);
  if (threadIdx.x == 0) *dst = s;
}

// ---------------------------------------------------------------- generic batch: y = H x (+ c z)
template <typename T>
__global__ void __launch_bounds__(kMvBlock) k_mv(const MvTask<T> *tasks, const int *item_task, int nitems, int xs_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[kMvBlock / 32];
  T *xs = reinterpret_cast<T *>(smem_raw);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const MvTask<T> &t = tasks[item_task[it]];
    const long long li = it - t.item_begin;
    DotAcc acc;
    dot_init(acc);
    const bool want = t.dot_partial != nullptr;
    mv_item<T>(*t.op, t.srs_rows, li, t.x, t.y, t.z, (T)t.c, want, acc, xs, xs_cap);
    emit_dot<T>(want, acc, want ? t.dot_partial + li : nullptr, red);
  }
}

// ---------------------------------------------------------------- Lanczos recurrence, phase 1
// Iteration it (0-based) of Lanczos.h:44-68: v = buf[it%3], w = buf[(it+1)%3] <- H v - bet * buf[(it+2)%3].
template <typename T>
__global__ void __launch_bounds__(kMvBlock) k_lz_mv(const LzTask<T> *tasks, const int *item_task, int nitems, int iter,
                                                    int xs_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[kMvBlock / 32];
  T *xs = reinterpret_cast<T *>(smem_raw);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const LzTask<T> &t = tasks[item_task[it]];
    if (t.state[0]) continue;  // recurrence finished (uniform per block)
    const long long li = it - t.item_begin;
    const T *x = t.buf[iter % 3];
    T *y = t.buf[(iter + 1) % 3];
    const T *z = iter == 0 ? nullptr : t.buf[(iter + 2) % 3];
    const T c = (T)(-t.scal[1]);
    DotAcc acc;
    dot_init(acc);
    mv_item<T>(*t.op, t.srs_rows, li, x, y, z, c, true, acc, xs, xs_cap);
    emit_dot<T>(true, acc, t.part_a + li, red);
  }
}

// ---------------------------------------------------------------- eigen-solver step, phase 1
// w = H V[j] for tasks in Lanczos mode that still grow their basis; |w|^2 per item.
template <typename T>
__global__ void __launch_bounds__(kMvBlock) k_eig_mv(const EigTask<T> *tasks, const int *item_task, int nitems, int xs_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[kMvBlock / 32];
  T *xs = reinterpret_cast<T *>(smem_raw);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const EigTask<T> &t = tasks[item_task[it]];
    if (t.st[2] || t.st[1] != 0) continue;  // full, or orthogonalising a random vector (uniform)
    const long long li = it - t.item_begin;
    const T *x = t.V + (long long)t.st[0] * t.n;
    DotAcc acc;
    dot_init(acc);
    long long lo, hi;
    mv_item<T>(*t.op, t.srs_rows, li, x, t.w, nullptr, (T)0, false, acc, xs, xs_cap);
    // |w|^2 of this item (second sweep over the freshly written, cache-resident slice)
    __syncthreads();
    item_range(*t.op, t.srs_rows, li, lo, hi);
    dot_init(acc);
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) dot_add(acc, t.w[i], t.w[i]);
    emit_dot<T>(true, acc, t.npart + li, red);
  }
}

static int grid_for(int nitems) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 148;
  }
  int g = nsm * 4;
  return nitems < g ? (nitems > 0 ? nitems : 1) : g;
}

template <typename K>
static void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T>
void launch_mv(const MvTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int smem_elems, cudaStream_t st) {
  size_t sm = sizeof(T) * (size_t)smem_elems;
  set_smem(k_mv<T>, sm);
  k_mv<T><<<grid_for(nitems_total), kMvBlock, sm, st>>>(tasks_dev, item_task_dev, nitems_total, smem_elems); note_launch();
}

template <typename T>
void launch_lz_mv(const LzTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int it, int smem_elems,
                  cudaStream_t st) {
  size_t sm = sizeof(T) * (size_t)smem_elems;
  set_smem(k_lz_mv<T>, sm);
  k_lz_mv<T><<<grid_for(nitems_total), kMvBlock, sm, st>>>(tasks_dev, item_task_dev, nitems_total, it, smem_elems); note_launch();
}

template <typename T>
void launch_eig_mv(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int smem_elems,
                   cudaStream_t st) {
  size_t sm = sizeof(T) * (size_t)smem_elems;
  set_smem(k_eig_mv<T>, sm);
  k_eig_mv<T><<<grid_for(nitems_total), kMvBlock, sm, st>>>(tasks_dev, item_task_dev, nitems_total, smem_elems); note_launch();
}

template void launch_mv<float>(const MvTask<float> *, const int *, int, int, cudaStream_t);
template void launch_mv<double>(const MvTask<double> *, const int *, int, int, cudaStream_t);
template void launch_lz_mv<float>(const LzTask<float> *, const int *, int, int, int, cudaStream_t);
template void launch_lz_mv<double>(const LzTask<double> *, const int *, int, int, int, cudaStream_t);
template void launch_eig_mv<float>(const EigTask<float> *, const int *, int, int, cudaStream_t);
template void launch_eig_mv<double>(const EigTask<double> *, const int *, int, int, cudaStream_t);

}  // namespace edgpu
