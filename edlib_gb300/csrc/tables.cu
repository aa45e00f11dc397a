// Sector bookkeeping on the device: combinadic tables, per-spin hopping CSR, full CSR, diagonal.
//
// * basis / ninv        -- SzSymmetry::initial_fill / next_basis (include/edlib/SzSymmetry.h:191-216):
//                          the r-th state with k particles is the r-th k-combination of bit positions in
//                          lexicographic order of the sorted position tuple; ninv is its inverse.
// * spin CSR            -- SpinResolvedStorage::fill_spin (include/edlib/SpinResolvedStorage.h:622-638)
//                          with CRSMatrix::addElement/endLine merging (include/edlib/CRSMatrix.h:46-98)
// * full CSR            -- CRSStorage::fill / addElement (include/edlib/CRSStorage.h:66-83, 169-205)
// * diagonal            -- Model::diagonal for every state of a sector
// * SOCRS collision test -- SOCRSStorage::addElement (include/edlib/SOCRSStorage.h:303-317)
#include "edgpu_kernels.h"

namespace edgpu {

// ------------------------------------------------------------------ combinadic tables
__global__ void k_unrank(int ns, int k, long long count, const long long *binom, int *out) {
  long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= count) return;
  int mask = 0, x = 0;
  long long rem = r;
  for (int i = 0; i < k; ++i) {
    while (true) {
      long long c = binom_at(binom, ns - 1 - x, k - 1 - i);
      if (rem < c) break;
      rem -= c;
      ++x;
    }
    mask |= 1 << x;
    ++x;
  }
  out[r] = mask;
}

__global__ void k_ninv(int ns, const long long *binom, int *ninv) {
  long long mask = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (mask >= (1ll << ns)) return;
  int k = __popc((unsigned)mask);
  long long r = 0;
  int x = 0, i = 0;
  for (int p = 0; p < ns; ++p) {
    if (!((mask >> p) & 1)) continue;
    for (int y = x; y < p; ++y) r += binom_at(binom, ns - 1 - y, k - 1 - i);
    x = p + 1;
    ++i;
  }
  ninv[((long long)k << ns) | mask] = (int)r;
}

void build_tables(const DevModel &m, long long *basis_off_host, int *basis, int *ninv, cudaStream_t st) {
  for (int k = 0; k <= m.ns; ++k) {
    long long cnt = binom_at_host(m.ns, k);
    if (cnt == 0) continue;
    k_unrank<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(m.ns, k, cnt, m.binom, basis + basis_off_host[k]); note_launch();
  }
  long long nm = 1ll << m.ns;
  cudaMemsetAsync(ninv, 0, sizeof(int) * (size_t)(m.ns + 1) * nm, st);
  k_ninv<<<(unsigned)((nm + 255) / 256), 256, 0, st>>>(m.ns, m.binom, ninv); note_launch();
}

// ------------------------------------------------------------------ exclusive scan (int64)
__global__ void k_scan_block(const long long *in, long long *out, long long n, long long *block_sums) {
  __shared__ long long s[1024];
  long long i = blockIdx.x * 1024ll + threadIdx.x;
  long long v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = s[1023];
}

__global__ void k_scan_add(long long *out, long long n, const long long *block_prefix) {
  long long i = blockIdx.x * 1024ll + threadIdx.x;
  if (i < n) out[i] += block_prefix[blockIdx.x];
}

__global__ void k_scan_total(const long long *in, long long *out, long long n) { out[n] = out[n - 1] + in[n - 1]; }

// out[0..n] = exclusive scan of in[0..n), out[n] = total.  tmp must hold 2*ceil(n/1024)+2 values.
void exclusive_scan(const long long *in, long long *out, long long n, long long *tmp, cudaStream_t st) {
  long long nb = (n + 1023) / 1024;
  if (nb <= 0) {
    cudaMemsetAsync(out, 0, sizeof(long long), st);
    return;
  }
  k_scan_block<<<(unsigned)nb, 1024, 0, st>>>(in, out, n, tmp); note_launch();
  if (nb > 1) {
    exclusive_scan(tmp, tmp + nb + 1, nb, tmp + 2 * nb + 2, st);  // recursion on block sums
    k_scan_add<<<(unsigned)nb, 1024, 0, st>>>(out, n, tmp + nb + 1); note_launch();
  }
  // total = out[n-1] + in[n-1]
  k_scan_total<<<1, 1, 0, st>>>(in, out, n); note_launch();
}

long long scan_tmp_size(long long n) {
  long long s = 0;
  while (n > 1) {
    long long nb = (n + 1023) / 1024;
    s += 2 * nb + 2;
    n = nb;
  }
  return s + 4;
}

// ------------------------------------------------------------------ per-spin hopping CSR
constexpr int kRowMax = 256;

// Builds row r of the spin-s hopping matrix for k particles; count_only -> write count.
__device__ int spin_row(const DevModel &m, int spin, int k, int mask, int *cols, double *vals, int *err) {
  const int shift = spin == 0 ? m.ns : 0;
  const state_t nst = (state_t)mask << shift;
  int len = 0;
  for (int q = 0; q < m.nT; ++q) {
    const Transition &tr = m.T[q];
    if (!trans_valid(tr, nst, m.ip)) continue;
    int sign;
    state_t kk = trans_apply(tr, nst, m.ip, sign);
    int col = m.ninv[((long long)k << m.ns) | (int)(kk >> shift)];
    double t = tr.value;
    if (fabs(t) == 0) continue;
    int found = -1;
    for (int e = 0; e < len; ++e)
      if (cols[e] == col) found = e;
    if (found >= 0) {
      vals[found] += sign * t;
    } else {
      if (len >= kRowMax) { atomicExch(err, 1); return len; }
      cols[len] = col;
      vals[len] = sign * t;
      ++len;
    }
  }
  // CRSMatrix::compress: drop |v| < 1e-15; the element shifted into a removed slot is not re-tested
  for (int e = 0; e < len; ++e) {
    if (fabs(vals[e]) < 1e-15) {
      for (int r = e; r < len - 1; ++r) { vals[r] = vals[r + 1]; cols[r] = cols[r + 1]; }
      --len;
    }
  }
  return len;
}

__global__ void k_spin_count(DevModel m, int spin, int k, long long rows, const int *basis_k, long long *count, int *err) {
  long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int cols[kRowMax];
  double vals[kRowMax];
  count[r] = spin_row(m, spin, k, basis_k[r], cols, vals, err);
}

__global__ void k_spin_fill(DevModel m, int spin, int k, long long rows, const int *basis_k, const long long *rp,
                            int *rp32, int *col, double *val64, float *val32, int *err) {
  long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int cols[kRowMax];
  double vals[kRowMax];
  int len = spin_row(m, spin, k, basis_k[r], cols, vals, err);
  long long o = rp[r];
  rp32[r] = (int)o;
  if (r == rows - 1) rp32[rows] = (int)(o + len);
  for (int e = 0; e < len; ++e) {
    col[o + e] = cols[e];
    val64[o + e] = vals[e];
    val32[o + e] = (float)vals[e];
  }
}

// ------------------------------------------------------------------ full CSR of a sector
__device__ int crs_row(const DevModel &m, const SectorOp<double> &op, long long i, int *cols, double *vals, int *err) {
  state_t nst = sector_state(op, i);
  int len = 1;
  cols[0] = (int)i;
  vals[0] = model_diagonal(m, nst);
  for (int pass = 0; pass < 2; ++pass) {
    const Transition *L = pass == 0 ? m.T : m.V;
    int nL = pass == 0 ? m.nT : m.nV;
    for (int q = 0; q < nL; ++q) {
      const Transition &tr = L[q];
      if (!trans_valid(tr, nst, m.ip)) continue;
      int sign;
      state_t kk = trans_apply(tr, nst, m.ip, sign);
      int col = (int)sector_index(op, kk);
      int found = -1;
      for (int e = 0; e < len; ++e)
        if (cols[e] == col) found = e;
      if (found >= 0) {
        vals[found] += sign * tr.value;
      } else {
        if (len >= kRowMax) { atomicExch(err, 1); return len; }
        cols[len] = col;
        vals[len] = sign * tr.value;
        ++len;
      }
    }
  }
  return len;
}

__global__ void k_crs_count(DevModel m, SectorOp<double> op, long long *count, int *err) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= op.dim) return;
  int cols[kRowMax];
  double vals[kRowMax];
  count[i] = crs_row(m, op, i, cols, vals, err);
}

__global__ void k_crs_fill(DevModel m, SectorOp<double> op, const long long *rp, int *col, double *val64,
                           float *val32, int *err) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= op.dim) return;
  int cols[kRowMax];
  double vals[kRowMax];
  int len = crs_row(m, op, i, cols, vals, err);
  long long o = rp[i];
  for (int e = 0; e < len; ++e) {
    col[o + e] = cols[e];
    val64[o + e] = vals[e];
    val32[o + e] = (float)vals[e];
  }
}

// ------------------------------------------------------------------ diagonal, collisions
__global__ void k_diag(DevModel m, SectorOp<double> op, double *d64, float *d32) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= op.dim) return;
  double v = model_diagonal(m, sector_state(op, i));
  d64[i] = v;
  d32[i] = (float)v;
}

// SOCRS refuses a transition that lands on the diagonal or twice on the same column
__global__ void k_socrs_check(DevModel m, SectorOp<double> op, int *err) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= op.dim) return;
  state_t nst = sector_state(op, i);
  long long cols[kRowMax];
  int len = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const Transition *L = pass == 0 ? m.T : m.V;
    int nL = pass == 0 ? m.nT : m.nV;
    for (int q = 0; q < nL; ++q) {
      if (!trans_valid(L[q], nst, m.ip)) continue;
      int sign;
      long long c = sector_index(op, trans_apply(L[q], nst, m.ip, sign));
      if (c == i) { atomicExch(err, 2); return; }
      for (int e = 0; e < len; ++e)
        if (cols[e] == c) { atomicExch(err, 3); return; }
      if (len < kRowMax) cols[len++] = c;
    }
  }
}

__global__ void k_spin_ell(const int *rp, const int *col, const double *v64, const float *v32, int rows, int ld,
                           int *len, int *ell_col, double *ell_v64, float *ell_v32) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < rows; d += gridDim.x * blockDim.x) {
    const int j0 = rp[d], j1 = rp[d + 1];
    len[d] = j1 - j0;
    for (int j = j0; j < j1; ++j) {
      const long long e = (long long)(j - j0) * ld + d;
      ell_col[e] = col[j];
      ell_v64[e] = v64[j];
      ell_v32[e] = v32[j];
    }
  }
}

void launch_spin_ell(const int *rp, const int *col, const double *v64, const float *v32, int rows, int ld, int *len,
                     int *ell_col, double *ell_v64, float *ell_v32, cudaStream_t st) {
  const int blocks = std::max(1, std::min(1024, (rows + 255) / 256));
  k_spin_ell<<<blocks, 256, 0, st>>>(rp, col, v64, v32, rows, ld, len, ell_col, ell_v64, ell_v32); note_launch();
}

void launch_spin_csr(const DevModel &m, int spin, int k, long long rows, const int *basis_k, long long *count,
                     long long *rp, long long *scan_tmp, int *rp32, int **col, double **val64, float **val32,
                     long long *nnz_out, int *err, DeviceAllocator &alloc, cudaStream_t st) {
  unsigned g = (unsigned)((rows + 127) / 128);
  k_spin_count<<<g, 128, 0, st>>>(m, spin, k, rows, basis_k, count, err); note_launch();
  exclusive_scan(count, rp, rows, scan_tmp, st);
  long long nnz = 0;
  cudaMemcpyAsync(&nnz, rp + rows, sizeof(long long), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *nnz_out = nnz;
  *col = (int *)alloc.alloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  *val64 = (double *)alloc.alloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  *val32 = (float *)alloc.alloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  k_spin_fill<<<g, 128, 0, st>>>(m, spin, k, rows, basis_k, rp, rp32, *col, *val64, *val32, err); note_launch();
}

void launch_crs(const DevModel &m, const SectorOp<double> &op, long long *count, long long *rp, long long *scan_tmp,
                int **col, double **val64, float **val32, long long *nnz_out, int *err, DeviceAllocator &alloc,
                cudaStream_t st) {
  unsigned g = (unsigned)((op.dim + 127) / 128);
  k_crs_count<<<g, 128, 0, st>>>(m, op, count, err); note_launch();
  exclusive_scan(count, rp, op.dim, scan_tmp, st);
  long long nnz = 0;
  cudaMemcpyAsync(&nnz, rp + op.dim, sizeof(long long), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *nnz_out = nnz;
  *col = (int *)alloc.alloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  *val64 = (double *)alloc.alloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  *val32 = (float *)alloc.alloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  k_crs_fill<<<g, 128, 0, st>>>(m, op, rp, *col, *val64, *val32, err); note_launch();
}

void launch_diag(const DevModel &m, const SectorOp<double> &op, double *d64, float *d32, cudaStream_t st) {
  if (op.dim == 0) return;
  k_diag<<<(unsigned)((op.dim + 255) / 256), 256, 0, st>>>(m, op, d64, d32); note_launch();
}

void launch_socrs_check(const DevModel &m, const SectorOp<double> &op, int *err, cudaStream_t st) {
  if (op.dim == 0) return;
  k_socrs_check<<<(unsigned)((op.dim + 127) / 128), 128, 0, st>>>(m, op, err); note_launch();
}

}  // namespace edgpu
