// Hamiltonian-times-vector kernels for the three storages, batched over work items.
//
// * SRS   -- SpinResolvedStorage::av (include/edlib/SpinResolvedStorage.h:58-115): the sector vector is the
//            row-major N_up x N_dn matrix X (d fastest) and
//            Y = D o X + X H_dn^T + H_up X + H_loc X,
//            accumulated per element in the reference order (diagonal, down hops, up hops, interaction).
//            A work item is a group of up-rows; its rows of X are staged in shared memory so the H_dn
//            gather reads shared memory, and the H_up term reads whole rows of X (coalesced in d).  Tiles:
//            4 rows x 16 bytes per thread for rows of a multiple of 16 bytes (srs_unit_full), lane-strided
//            (a warp on 32 consecutive columns, srs_unit_lanes) for rows starting off 16-byte boundaries,
//            one row at a time for rows of thousands of states (srs_longrow); short rows are spread flat
//            over the block (srs_flat) so rows shorter than the block keep every thread busy.
//            The off-diagonal interaction (H_loc) is applied matrix-free from the transition list.
//            Element types: FP32, FP64, and float-float pairs (the mixed mode's recurrences).
// * CRS   -- CRSStorage::av (include/edlib/CRSStorage.h:57-64): one thread per row, diagonal first.
// * SOCRS -- SOCRSStorage::av (include/edlib/SOCRSStorage.h:46-87): matrix-free; each row re-derives its
//            state from the combinadic tables, tests every transition, ranks the target with ninv and
//            takes the fermion sign from one popc; nothing but the tables is stored.
// Every kernel is instantiated per storage (a launch covers one storage) and optionally emits <x, y>
// per item (FP64 / float-float accumulation, fixed order).

#include "edgpu_kernels.h"

namespace edgpu {

constexpr int kMvBlock = 256;
#ifndef EDGPU_SRS_LONGROW
// 1: items of fewer than four rows of >= 2048 states take the one-row-at-a-time path (srs_longrow)
#define EDGPU_SRS_LONGROW 1
#endif
#ifndef EDGPU_SRS_LANES_ALL
// 1: the lane-strided tile for every staged row group, 16-byte aligned rows included
#define EDGPU_SRS_LANES_ALL 0
#endif
// up-spin rows per SRS tile
#ifndef EDGPU_SRS_R
#define EDGPU_SRS_R 4
#endif
// resident blocks per SM the register allocation is held to: two for launches with a z term or dot
// products (the Lanczos recurrence), three for plain H*v launches; the eigen step comes in both variants,
// chosen by the operator tuner
#ifndef EDGPU_MV_MIN_BLOCKS
#define EDGPU_MV_MIN_BLOCKS 2
#endif
template <typename T>
constexpr int kMvMinBlocks = EDGPU_MV_MIN_BLOCKS;
#ifndef EDGPU_MV_MIN_BLOCKS_FF
#define EDGPU_MV_MIN_BLOCKS_FF 2
#endif
// the float-float recurrence operator (resident blocks per SM its registers are held to)
template <>
constexpr int kMvMinBlocks<ffloat> = EDGPU_MV_MIN_BLOCKS_FF;
static_assert(kSrsLongRow >= kMvBlock / 2, "tiled SRS rows must fill most of a block");

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

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

// The block's bulk-copy barrier and its failure flag, in shared memory.  `dead` is set when both bounded
// waits on a stage gave up: that barrier phase never completed, so the barrier is never armed again and
// every later item of the block takes a path without bulk copies.
struct MvBar {
  unsigned long long bar;
  int dead;
};

// Shared memory of an operator block: the staged x rows of the current item.
template <typename T>
struct MvSmem {
  T *xs;
  int xs_cap;
  unsigned bar;    // shared-memory address of the block's transaction barrier (bulk copies)
  unsigned phase;  // parity of the barrier phase the next bulk stage completes
  int *dead;       // MvBar::dead of the block
};

// Set when a bounded wait on a bulk copy gave up (the copy never completed); read by the host.
__device__ int g_mv_stall = 0;
constexpr int kBulkSpin = 1 << 22;  // try_wait rounds before a bulk stage is declared stalled

// The block's transaction barrier: one arrival per phase (thread 0, with the byte count it expects).
__device__ __forceinline__ unsigned init_bulk_barrier(unsigned long long *b) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(b);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  return a;
}

// Bounded wait for the barrier phase of parity `phase`; false when it did not complete.
__device__ __forceinline__ bool wait_bulk(unsigned bar, unsigned phase, int rounds = kBulkSpin) {
  for (int it = 0; it < rounds; ++it) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One bulk (TMA) copy of `bytes` (a multiple of 16, both ends 16-byte aligned) global -> shared, completing on
// the barrier's transaction count.
__device__ __forceinline__ void bulk_copy(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Off-diagonal interaction of one SRS element (matrix-free, Kanamori-type V_states).
template <typename T>
__device__ __forceinline__ T srs_vloc(const SectorOp<T> &op, int u, int d, const T *__restrict__ x, T v) {
  state_t s = ((state_t)op.up_basis[u] << op.ns) | (state_t)op.dn_basis[d];
  return transitions_term(op, s, op.V_, op.V_val, op.nV, x, v);
}

// C consecutive vector elements (16 bytes: 4 FP32 or 2 FP64) in one load when `vec` is set (the caller
// guarantees the alignment); a ragged end (n < C) is read element by element.
template <typename T>
__device__ __forceinline__ Lanes<T> load_lanes(const T *p, bool vec, int n) {
  Lanes<T> q;
  if (vec && n == Lanes<T>::C) {
    if constexpr (std::is_same<T, ffloat>::value) {
      const float4 f = ldg_t(reinterpret_cast<const float4 *>(p));
      q.v[0] = ffloat(f.x, f.y), q.v[1] = ffloat(f.z, f.w);
    } else if constexpr (sizeof(T) == 4) {
      const float4 f = ldg_t(reinterpret_cast<const float4 *>(p));
      q.v[0] = f.x, q.v[1] = f.y, q.v[2] = f.z, q.v[3] = f.w;
    } else {
      const double2 f = ldg_t(reinterpret_cast<const double2 *>(p));
      q.v[0] = f.x, q.v[1] = f.y;
    }
  } else {
#pragma unroll
    for (int cc = 0; cc < Lanes<T>::C; ++cc) q.v[cc] = cc < n ? p[cc] : (T)0;
  }
  return q;
}

// C consecutive ints of a k-major table (16 bytes for C = 4, 8 for C = 2; always aligned: the table's
// leading dimension is a multiple of 4 and column tiles start at multiples of C).
template <int C>
__device__ __forceinline__ Lanes<int> load_ints(const int *p) {
  Lanes<int> q;
  if constexpr (C == 4) {
    const int4 f = ldg_t(reinterpret_cast<const int4 *>(p));
    q.v[0] = f.x, q.v[1] = f.y, q.v[2] = f.z, q.v[3] = f.w;
  } else {
    const int2 f = ldg_t(reinterpret_cast<const int2 *>(p));
    q.v[0] = f.x, q.v[1] = f.y;
  }
  return q;
}

// C consecutive elements at p: one 16-byte load when AL (p 16-byte aligned), else C element loads (rows whose
// length is not a multiple of C start at every alignment); global memory through the read-only path.
template <typename T, bool AL>
__device__ __forceinline__ Lanes<T> ldg_lanes(const T *p) {
  if constexpr (AL) return load_lanes(p, true, Lanes<T>::C);
  Lanes<T> q;
#pragma unroll
  for (int cc = 0; cc < Lanes<T>::C; ++cc) q.v[cc] = ldg_t(p + cc);
  return q;
}
template <typename T, bool AL>
__device__ __forceinline__ Lanes<T> lds_lanes(const T *p) {
  if constexpr (AL) return *reinterpret_cast<const Lanes<T> *>(p);
  Lanes<T> q;
#pragma unroll
  for (int cc = 0; cc < Lanes<T>::C; ++cc) q.v[cc] = p[cc];
  return q;
}
template <typename T, bool AL>
__device__ __forceinline__ void st_lanes(T *p, const T *v) {
  if constexpr (AL) {
    store_lanes(p, v);
  } else {
#pragma unroll
    for (int cc = 0; cc < Lanes<T>::C; ++cc) p[cc] = v[cc];
  }
}

// Full tile of the SRS sweep (4 rows x C columns, rows staged in shared memory): the common case, written
// without per-element predicates, for rows of a multiple of C elements on 16-byte aligned bases, so every
// access of the tile is one 16-byte load or store.  Entries past a down-spin row's end in the
// k-major copy hold value 0 and column 0, so the tile runs every column to the longest of its C rows and
// the padding adds exact zeros after the row's own entries (same sum).
template <typename T, bool HZ, bool DOT>
__device__ __forceinline__ void srs_unit_full(const SectorOp<T> &op, int u, int d0, int Nd, const T *__restrict__ xs,
                                              const T *__restrict__ x, const T *__restrict__ dg, T *__restrict__ yr,
                                              const T *__restrict__ zr, T c, DotAcc &acc) {
  constexpr int R = EDGPU_SRS_R, C = Lanes<T>::C;
  T a[R][C];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const Lanes<T> dq = ldg_lanes<T, true>(dg + r * Nd + d0);
    const Lanes<T> xq = lds_lanes<T, true>(xs + r * Nd + d0);
#pragma unroll
    for (int cc = 0; cc < C; ++cc) a[r][cc] = dq.v[cc] * xq.v[cc];
    if (HZ) {
      const Lanes<T> zq = ldg_lanes<T, true>(zr + r * Nd + d0);
#pragma unroll
      for (int cc = 0; cc < C; ++cc) a[r][cc] = a[r][cc] + c * zq.v[cc];
    }
  }
  {
    const int *__restrict__ ecol = op.dn_ell_col;
    const T *__restrict__ eval = op.dn_ell_val;
    const int eld = op.dn_ld;
    const Lanes<int> lq = load_ints<C>(op.dn_len + d0);
    int kk = lq.v[0];
#pragma unroll
    for (int cc = 1; cc < C; ++cc) kk = max(kk, lq.v[cc]);
#pragma unroll 2
    for (int k = 0; k < kk; ++k) {
      const Lanes<int> cq = load_ints<C>(ecol + k * eld + d0);
      const Lanes<T> vq = load_lanes(eval + k * eld + d0, true, C);
#pragma unroll
      for (int cc = 0; cc < C; ++cc)
#pragma unroll
        for (int r = 0; r < R; ++r) a[r][cc] += vq.v[cc] * xs[r * Nd + cq.v[cc]];
    }
  }
  // up hops: the R rows advance together, HB entries per row per round, so that R * HB row loads are in
  // flight at once (each row still adds its entries in order); one per row with a z term or dot products,
  // for registers
  {
    constexpr int HB = (HZ || DOT) ? 1 : 2;
    const int *__restrict__ urp = op.up_rp;
    const int *__restrict__ ucol = op.up_col;
    const T *__restrict__ uval = op.up_val;
    int kc[R], ke[R], nmax = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      kc[r] = ldg_t(urp + u + r);
      ke[r] = ldg_t(urp + u + r + 1);
      nmax = max(nmax, ke[r] - kc[r]);
    }
    for (int h = 0; h < nmax; h += HB) {
      T vk[R][HB];
      Lanes<T> xq[R][HB];
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int q = 0; q < HB; ++q) {
          const int k = kc[r] + h + q;
          const bool ok = k < ke[r];
          vk[r][q] = ok ? ldg_t(uval + k) : T(0);
          xq[r][q] = ok ? ldg_lanes<T, true>(x + ldg_t(ucol + k) * Nd + d0) : Lanes<T>{};
        }
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int q = 0; q < HB; ++q)
          if (kc[r] + h + q < ke[r]) {
#pragma unroll
            for (int cc = 0; cc < C; ++cc) a[r][cc] += vk[r][q] * xq[r][q].v[cc];
          }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (op.nV) {
#pragma unroll
      for (int cc = 0; cc < C; ++cc) a[r][cc] = srs_vloc(op, u + r, d0 + cc, x, a[r][cc]);
    }
    st_lanes<T, true>(yr + r * Nd + d0, a[r]);
    if (DOT) {
      const Lanes<T> xq = lds_lanes<T, true>(xs + r * Nd + d0);
#pragma unroll
      for (int cc = 0; cc < C; ++cc) dot_add(acc, xq.v[cc], a[r][cc]);
    }
  }
}

// Tile of rows whose length is not a multiple of C (e.g. 495-state rows: no 16-byte access of a row is
// aligned): the warp's 32 lanes take 32 consecutive columns, and each lane C columns 32 apart (c0 + 32 cc), so
// every load and store of the warp is one contiguous 128-byte (FP32) or 256-byte (FP64) piece instead of C
// pieces 16 bytes apart per lane.  nr <= R rows are real; FULL: all R rows and all C columns of every lane lie
// inside the item (no predicates).  Per element the sum runs in the same order as the other tiles: diagonal,
// (c z), down hops in CSR order (the k-major copy's zero padding adds exact zeros), up hops in order, interaction.
template <typename T, bool HZ, bool DOT, bool FULL>
__device__ __forceinline__ void srs_unit_lanes(const SectorOp<T> &op, int u, int c0, int Nd, int nr,
                                               const T *__restrict__ xs, const T *__restrict__ x,
                                               const T *__restrict__ dg, T *__restrict__ yr, const T *__restrict__ zr,
                                               T c, DotAcc &acc) {
  constexpr int R = EDGPU_SRS_R, C = Lanes<T>::C;
  bool okc[C];
#pragma unroll
  for (int cc = 0; cc < C; ++cc) okc[cc] = FULL || c0 + 32 * cc < Nd;
  T a[R][C];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int cc = 0; cc < C; ++cc) {
      const int o = r * Nd + c0 + 32 * cc;
      if (FULL || (r < nr && okc[cc])) {
        a[r][cc] = ldg_t(dg + o) * xs[o];
        if (HZ) a[r][cc] = a[r][cc] + c * ldg_t(zr + o);
      } else {
        a[r][cc] = T(0);
      }
    }
  {
    const int *__restrict__ ecol = op.dn_ell_col;
    const T *__restrict__ eval = op.dn_ell_val;
    const int eld = op.dn_ld;
    int kk = 0;
#pragma unroll
    for (int cc = 0; cc < C; ++cc)
      if (okc[cc]) kk = max(kk, ldg_t(op.dn_len + c0 + 32 * cc));
#pragma unroll 2
    for (int k = 0; k < kk; ++k) {
      int col[C];
      T val[C];
#pragma unroll
      for (int cc = 0; cc < C; ++cc) {
        col[cc] = okc[cc] ? ldg_t(ecol + k * eld + c0 + 32 * cc) : 0;
        val[cc] = okc[cc] ? ldg_t(eval + k * eld + c0 + 32 * cc) : T(0);
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (FULL || r < nr) {
#pragma unroll
          for (int cc = 0; cc < C; ++cc) a[r][cc] += val[cc] * xs[r * Nd + col[cc]];
        }
    }
  }
  {
    const int *__restrict__ urp = op.up_rp;
    const int *__restrict__ ucol = op.up_col;
    const T *__restrict__ uval = op.up_val;
    int kc[R], ke[R], nmax = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const bool live = FULL || r < nr;
      kc[r] = live ? ldg_t(urp + u + r) : 0;
      ke[r] = live ? ldg_t(urp + u + r + 1) : 0;
      nmax = max(nmax, ke[r] - kc[r]);
    }
    for (int h = 0; h < nmax; ++h) {
      T vk[R], xq[R][C];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = kc[r] + h;
        const bool ok = k < ke[r];
        vk[r] = ok ? ldg_t(uval + k) : T(0);
        const T *src = x + (long long)(ok ? ldg_t(ucol + k) : 0) * Nd + c0;
#pragma unroll
        for (int cc = 0; cc < C; ++cc) xq[r][cc] = ok && okc[cc] ? ldg_t(src + 32 * cc) : T(0);
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (kc[r] + h < ke[r]) {
#pragma unroll
          for (int cc = 0; cc < C; ++cc) a[r][cc] += vk[r] * xq[r][cc];
        }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int cc = 0; cc < C; ++cc)
      if (FULL || (r < nr && okc[cc])) {
        const int o = r * Nd + c0 + 32 * cc;
        T v = a[r][cc];
        if (op.nV) v = srs_vloc(op, u + r, c0 + 32 * cc, x, v);
        yr[o] = renorm(v);
        if (DOT) dot_add(acc, xs[o], v);
      }
}

// Tile of an SRS item whose up-spin source rows are staged in shared memory too (srcs: row h = the x row of
// hop entry kb + h): every gather of the tile reads shared memory.  nr <= 4 rows of the tile are real.
template <typename T, bool HZ, bool DOT>
__device__ __forceinline__ void srs_unit_staged(const SectorOp<T> &op, int u, int d0, int Nd, int nr,
                                                const T *__restrict__ xs, const T *__restrict__ srcs, int kb,
                                                const T *__restrict__ x, const T *__restrict__ dg, T *__restrict__ yr,
                                                const T *__restrict__ zr, T c, DotAcc &acc) {
  constexpr int R = EDGPU_SRS_R, C = Lanes<T>::C;
  T a[R][C];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (r < nr) {
      const Lanes<T> dq = load_lanes(dg + r * Nd + d0, true, C);
      const Lanes<T> xq = *reinterpret_cast<const Lanes<T> *>(xs + r * Nd + d0);
#pragma unroll
      for (int cc = 0; cc < C; ++cc) a[r][cc] = dq.v[cc] * xq.v[cc];
      if (HZ) {
        const Lanes<T> zq = load_lanes(zr + r * Nd + d0, true, C);
#pragma unroll
        for (int cc = 0; cc < C; ++cc) a[r][cc] = a[r][cc] + c * zq.v[cc];
      }
    }
  }
  {
    const int *__restrict__ ecol = op.dn_ell_col;
    const T *__restrict__ eval = op.dn_ell_val;
    const int eld = op.dn_ld;
    const Lanes<int> lq = load_ints<C>(op.dn_len + d0);
    int kk = lq.v[0];
#pragma unroll
    for (int cc = 1; cc < C; ++cc) kk = max(kk, lq.v[cc]);
#pragma unroll 2
    for (int k = 0; k < kk; ++k) {
      const Lanes<int> cq = load_ints<C>(ecol + k * eld + d0);
      const Lanes<T> vq = load_lanes(eval + k * eld + d0, true, C);
#pragma unroll
      for (int cc = 0; cc < C; ++cc)
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r < nr) a[r][cc] += vq.v[cc] * xs[r * Nd + cq.v[cc]];
    }
  }
  const int *__restrict__ urp = op.up_rp;
  const T *__restrict__ uval = op.up_val;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (r < nr) {
      const int k0 = ldg_t(urp + u + r), k1 = ldg_t(urp + u + r + 1);
#pragma unroll 4
      for (int k = k0; k < k1; ++k) {
        const T vk = ldg_t(uval + k);
        const Lanes<T> sq = *reinterpret_cast<const Lanes<T> *>(srcs + (k - kb) * Nd + d0);
#pragma unroll
        for (int cc = 0; cc < C; ++cc) a[r][cc] += vk * sq.v[cc];
      }
      if (op.nV) {
#pragma unroll
        for (int cc = 0; cc < C; ++cc) a[r][cc] = srs_vloc(op, u + r, d0 + cc, x, a[r][cc]);
      }
      store_lanes(yr + r * Nd + d0, a[r]);
      if (DOT) {
        const Lanes<T> xq = *reinterpret_cast<const Lanes<T> *>(xs + r * Nd + d0);
#pragma unroll
        for (int cc = 0; cc < C; ++cc) dot_add(acc, xq.v[cc], a[r][cc]);
      }
    }
  }
}

template <typename T, bool MZ, bool MD>
__device__ __forceinline__ void srs_staged(const SectorOp<T> &op, long long lo, int u0, int nrows, int kb, const T *__restrict__ x,
                                           const T *__restrict__ xs, const T *__restrict__ srcs, T *__restrict__ y,
                                           const T *__restrict__ z, T c, bool want_dot, DotAcc &acc) {
  constexpr int R = EDGPU_SRS_R, C = Lanes<T>::C;
  const int Nd = op.dn_rows;
  const int ncq = Nd / C;
  const int ngr = (nrows + R - 1) / R;
  // (row group, column quad) of the thread's units, advanced without a division per unit
  int gn = threadIdx.x / ncq, qn = threadIdx.x - gn * ncq;
  for (int unit = threadIdx.x; unit < ngr * ncq; unit += kMvBlock) {
    const int g = gn;
    const int d0 = qn * C;
    for (qn += kMvBlock; qn >= ncq; qn -= ncq) ++gn;
    const int rg = g * R;
    const int nr = min(R, nrows - rg);
    const int off = rg * Nd;
    const T *dg = op.diag + lo + off;
    T *yr = y + lo + off;
    if (MZ && z) {
      if (MD && want_dot) srs_unit_staged<T, MZ, MD>(op, u0 + rg, d0, Nd, nr, xs + off, srcs, kb, x, dg, yr, z + lo + off, c, acc);
      else srs_unit_staged<T, MZ, false>(op, u0 + rg, d0, Nd, nr, xs + off, srcs, kb, x, dg, yr, z + lo + off, c, acc);
    } else {
      if (MD && want_dot) srs_unit_staged<T, false, MD>(op, u0 + rg, d0, Nd, nr, xs + off, srcs, kb, x, dg, yr, nullptr, c, acc);
      else srs_unit_staged<T, false, false>(op, u0 + rg, d0, Nd, nr, xs + off, srcs, kb, x, dg, yr, nullptr, c, acc);
    }
  }
}

// SRS item, rows of at least kSrsLongRow elements, in tiles of 4 rows x C consecutive columns per thread
// (C = 4 in FP32, 2 in FP64: one 16-byte load): each down-spin CSR entry (column, value) of a column
// serves the 4 rows, each up-spin hop (row, value) of a row serves the C columns with one load of x.  Work units (row group, column quad) are
// spread over the block.  Per element the sum runs in the reference's order: diagonal, (c z), down hops,
// up hops, interaction.  All in-sector offsets are 32-bit.
template <typename T, bool MZ, bool MD>
__device__ __forceinline__ void srs_tiled(const SectorOp<T> &op, long long lo, int u0, int nrows, const T *__restrict__ x,
                                          const T *__restrict__ xr, bool staged, const T *__restrict__ xs,
                                          T *__restrict__ y, const T *__restrict__ z, T c, bool want_dot, DotAcc &acc) {
  constexpr int R = EDGPU_SRS_R, C = Lanes<T>::C;
  const int Nd = op.dn_rows;
  const T *__restrict__ dg = op.diag + lo;
  T *__restrict__ yb = y + lo;
  const T *__restrict__ zb = z ? z + lo : nullptr;
  const int *__restrict__ elen = op.dn_len;
  const int *__restrict__ ecol = op.dn_ell_col;
  const T *__restrict__ eval = op.dn_ell_val;
  const int eld = op.dn_ld;
  const int *__restrict__ urp = op.up_rp;
  const int *__restrict__ ucol = op.up_col;
  const T *__restrict__ uval = op.up_val;
  // 16-byte vector access needs rows of a multiple of C elements and aligned bases (uniform per item)
  const uintptr_t amask = (uintptr_t)15;
  const bool vec = (Nd % C) == 0 && ((uintptr_t)x & amask) == 0 && ((uintptr_t)dg & amask) == 0 &&
                   (!zb || ((uintptr_t)zb & amask) == 0);
  const int ncq = (Nd + C - 1) / C;
  const int ngr = (nrows + R - 1) / R;
  if (staged && (EDGPU_SRS_LANES_ALL || !(vec && (uintptr_t(yb) & amask) == 0))) {
    // rows without aligned 16-byte pieces: lane-strided tiles, a warp per (row group, 32 C columns)
    constexpr int W = 32 * C;
    const int ncb = (Nd + W - 1) / W;
    // (row group, column block) of the warp's units, advanced without a division per unit (uniform per warp)
    int gn = (threadIdx.x >> 5) / ncb, bn = (threadIdx.x >> 5) - gn * ncb;
    for (int unit = threadIdx.x; unit < ngr * ncb * 32; unit += kMvBlock) {
      const int g = gn, b = bn;
      for (bn += kMvBlock / 32; bn >= ncb; bn -= ncb) ++gn;
      const int rg = g * R, nr = min(R, nrows - rg), c0 = b * W + (unit & 31), off = rg * Nd;
      const bool hz = MZ && zb != nullptr, dot = MD && want_dot;
      const T *zo = hz ? zb + off : nullptr;
      if (nr == R && (b + 1) * W <= Nd) {
        if (hz && dot) srs_unit_lanes<T, MZ, MD, true>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else if (hz) srs_unit_lanes<T, MZ, false, true>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else if (dot) srs_unit_lanes<T, false, MD, true>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else srs_unit_lanes<T, false, false, true>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
      } else {
        if (hz && dot) srs_unit_lanes<T, MZ, MD, false>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else if (hz) srs_unit_lanes<T, MZ, false, false>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else if (dot) srs_unit_lanes<T, false, MD, false>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
        else srs_unit_lanes<T, false, false, false>(op, u0 + rg, c0, Nd, nr, xs + off, x, dg + off, yb + off, zo, c, acc);
      }
    }
    return;
  }
  // (row group, column quad) of the thread's units, advanced without a division per unit
  int gn = threadIdx.x / ncq, qn = threadIdx.x - gn * ncq;
  for (int unit = threadIdx.x; unit < ngr * ncq; unit += kMvBlock) {
    const int g = gn;
    const int d0 = qn * C;
    for (qn += kMvBlock; qn >= ncq; qn -= ncq) ++gn;
    const int rg = g * R;
    const int nr = min(R, nrows - rg);
    const int nc = min(C, Nd - d0);
    const T *xg = xr + rg * Nd;
    if (staged && vec && (uintptr_t(yb) & amask) == 0 && nr == R && nc == C) {
      const int off = rg * Nd;
      if (MZ && zb) {
        if (MD && want_dot) srs_unit_full<T, MZ, MD>(op, u0 + rg, d0, Nd, xs + off, x, dg + off, yb + off, zb + off, c, acc);
        else srs_unit_full<T, MZ, false>(op, u0 + rg, d0, Nd, xs + off, x, dg + off, yb + off, zb + off, c, acc);
      } else {
        if (MD && want_dot) srs_unit_full<T, false, MD>(op, u0 + rg, d0, Nd, xs + off, x, dg + off, yb + off, nullptr, c, acc);
        else srs_unit_full<T, false, false>(op, u0 + rg, d0, Nd, xs + off, x, dg + off, yb + off, nullptr, c, acc);
      }
      continue;
    }
    T a[R][C];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r < nr) {
        const Lanes<T> dq = load_lanes(dg + (rg + r) * Nd + d0, vec, nc);
#pragma unroll
        for (int cc = 0; cc < C; ++cc) a[r][cc] = cc < nc ? dq.v[cc] * xg[r * Nd + d0 + cc] : (T)0;
        if (zb) {
          const Lanes<T> zq = load_lanes(zb + (rg + r) * Nd + d0, vec, nc);
#pragma unroll
          for (int cc = 0; cc < C; ++cc) a[r][cc] = a[r][cc] + c * zq.v[cc];
        }
      }
    }
    // down hops from the k-major copy: entry k of the C columns in one 16-byte load of values and one of
    // columns; each element still adds its entries in CSR order
    {
      int len[C], kk = 0;
      const Lanes<int> lq = load_ints<C>(elen + d0);
#pragma unroll
      for (int cc = 0; cc < C; ++cc) {
        len[cc] = lq.v[cc];
        kk = max(kk, len[cc]);
      }
      for (int k = 0; k < kk; ++k) {
        const Lanes<int> cq = load_ints<C>(ecol + k * eld + d0);
        const Lanes<T> vq = load_lanes(eval + k * eld + d0, true, C);
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
          if (k < len[cc]) {
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (r < nr) a[r][cc] += vq.v[cc] * xg[r * Nd + cq.v[cc]];
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r < nr) {
        const int u = u0 + rg + r;
        const int k0 = ldg_t(urp + u), k1 = ldg_t(urp + u + 1);
        // hops in batches of 4 so that four row loads of x are in flight at once (entries past the row's
        // end are not added)
        for (int k = k0; k < k1; k += 4) {
          Lanes<T> xq[4];
          T vk[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int kq = k + q < k1 ? k + q : k0;
            vk[q] = ldg_t(uval + kq);
            xq[q] = load_lanes(x + ldg_t(ucol + kq) * Nd + d0, vec, nc);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (k + q < k1) {
#pragma unroll
              for (int cc = 0; cc < C; ++cc) a[r][cc] += vk[q] * xq[q].v[cc];
            }
          }
        }
        T *yr = yb + (rg + r) * Nd + d0;
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
          if (cc < nc) {
            T v = a[r][cc];
            if (op.nV) v = srs_vloc(op, u, d0 + cc, x, v);
            yr[cc] = renorm(v);
            if (want_dot) dot_add(acc, xg[r * Nd + d0 + cc], v);
          }
        }
      }
    }
  }
}

// SRS item of very long rows (one to three rows per item, each staged in shared memory): one row at a time,
// its up-spin hop list (source-row offsets and values) copied once to shared memory for the whole block, and
// each thread sweeping C-column quads of the row: diagonal (c z), the down hops from the staged row through
// the k-major copy, the up hops as gathers of the quad from each source row (8-byte pieces when rows have an
// even length), the interaction.  The same sums in the same order as the tiled paths.  For rows of 10^4
// states (the 4x4 cluster's 12,870) this replaces the four-row tile with three rows predicated off.
// Returns false (nothing done) when a row has more than kLongHops up hops.
constexpr int kLongHops = 128;
template <typename T, bool MZ, bool MD>
__device__ __forceinline__ bool srs_longrow(const SectorOp<T> &op, long long lo, int u0, int nrows, const T *__restrict__ x,
                                            const T *__restrict__ xs, T *__restrict__ y, const T *__restrict__ z, T c,
                                            bool want_dot, DotAcc &acc) {
  constexpr int C = Lanes<T>::C;
  __shared__ long long hop_off[kLongHops];
  __shared__ T hop_val[kLongHops];
  const int Nd = op.dn_rows;
  for (int r = 0; r < nrows; ++r)
    if (ldg_t(op.up_rp + u0 + r + 1) - ldg_t(op.up_rp + u0 + r) > kLongHops) return false;  // uniform
  const bool even = (Nd & 1) == 0 && ((uintptr_t)x & 7) == 0;
  const int *__restrict__ elen = op.dn_len;
  const int *__restrict__ ecol = op.dn_ell_col;
  const T *__restrict__ eval = op.dn_ell_val;
  const int eld = op.dn_ld;
  for (int r = 0; r < nrows; ++r) {
    const int u = u0 + r;
    const int k0 = ldg_t(op.up_rp + u), nh = ldg_t(op.up_rp + u + 1) - k0;
    __syncthreads();  // the previous row's hop list is no longer read
    for (int h = threadIdx.x; h < nh; h += blockDim.x) {
      hop_off[h] = (long long)ldg_t(op.up_col + k0 + h) * Nd;
      hop_val[h] = ldg_t(op.up_val + k0 + h);
    }
    __syncthreads();
    const T *__restrict__ xrow = xs + (long long)r * Nd;
    const long long rowbase = lo + (long long)r * Nd;
    for (int d0 = C * threadIdx.x; d0 < Nd; d0 += C * blockDim.x) {
      const int nc = min(C, Nd - d0);
      T a[C];
#pragma unroll
      for (int cc = 0; cc < C; ++cc) {
        const bool in = cc < nc;
        a[cc] = in ? ldg_t(op.diag + rowbase + d0 + cc) * xrow[d0 + cc] : (T)0;
        if (MZ && z && in) a[cc] = a[cc] + c * z[rowbase + d0 + cc];
      }
      {  // down hops: entry k of the quad's columns in one 16-byte load each of columns and values
        const Lanes<int> lq = load_ints<C>(elen + d0);
        int kk = lq.v[0];
#pragma unroll
        for (int cc = 1; cc < C; ++cc) kk = max(kk, lq.v[cc]);
        for (int k = 0; k < kk; ++k) {
          const Lanes<int> cq = load_ints<C>(ecol + k * eld + d0);
          const Lanes<T> vq = load_lanes(eval + k * eld + d0, true, C);
#pragma unroll
          for (int cc = 0; cc < C; ++cc)
            if (k < lq.v[cc]) a[cc] += vq.v[cc] * xrow[cq.v[cc]];
        }
      }
      // up hops: the quad of every source row, four hops' loads in flight
      if (nc == C && even) {
        for (int h = 0; h < nh; h += 4) {
          Lanes<T> xq[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int hq = h + q < nh ? h + q : h;
            const T *src = x + hop_off[hq] + d0;
            if constexpr (sizeof(T) == 4) {
              const float2 p0 = ldg_t(reinterpret_cast<const float2 *>(src));
              const float2 p1 = ldg_t(reinterpret_cast<const float2 *>(src + 2));
              xq[q].v[0] = p0.x, xq[q].v[1] = p0.y, xq[q].v[2] = p1.x, xq[q].v[3] = p1.y;
            } else {
              xq[q].v[0] = ldg_t(src);
              xq[q].v[1] = ldg_t(src + 1);
            }
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (h + q < nh) {
              const T v = hop_val[h + q];
#pragma unroll
              for (int cc = 0; cc < C; ++cc) a[cc] += v * xq[q].v[cc];
            }
        }
      } else {
        for (int h = 0; h < nh; ++h) {
          const T v = hop_val[h];
          const T *src = x + hop_off[h] + d0;
#pragma unroll
          for (int cc = 0; cc < C; ++cc)
            if (cc < nc) a[cc] += v * ldg_t(src + cc);
        }
      }
#pragma unroll
      for (int cc = 0; cc < C; ++cc) {
        if (cc < nc) {
          T v = a[cc];
          if (op.nV) v = srs_vloc(op, u, d0 + cc, x, v);
          y[rowbase + d0 + cc] = renorm(v);
          if (MD && want_dot) dot_add(acc, xrow[d0 + cc], v);
        }
      }
    }
  }
  return true;
}

// SRS item, short rows: elements spread flat over the block ((r, d) advanced incrementally), so rows
// shorter than the block keep every thread busy.
template <typename T>
__device__ __forceinline__ void srs_flat(const SectorOp<T> &op, long long lo, int u0, int nel, const T *__restrict__ x,
                                         const T *__restrict__ xr, T *__restrict__ y, const T *__restrict__ z, T c,
                                         bool want_dot, DotAcc &acc) {
  const int Nd = op.dn_rows;
  const T *__restrict__ dg = op.diag + lo;
  T *__restrict__ yb = y + lo;
  const T *__restrict__ zb = z ? z + lo : nullptr;
  const int *__restrict__ drp = op.dn_rp;
  const int *__restrict__ dcol = op.dn_col;
  const T *__restrict__ dval = op.dn_val;
  const int *__restrict__ urp = op.up_rp;
  const int *__restrict__ ucol = op.up_col;
  const T *__restrict__ uval = op.up_val;
  const int rstep = kMvBlock / Nd, dstep = kMvBlock - rstep * Nd;
  int r = threadIdx.x / Nd, d = threadIdx.x - r * Nd;
  for (int e = threadIdx.x; e < nel; e += kMvBlock) {
    const int u = u0 + r;
    const T *xrow = xr + r * Nd;
    const T xv = xrow[d];
    T v = ldg_t(dg + e) * xv;
    if (zb) v = v + c * zb[e];
    const int j0 = ldg_t(drp + d), j1 = ldg_t(drp + d + 1);
    for (int j = j0; j < j1; ++j) v += ldg_t(dval + j) * xrow[ldg_t(dcol + j)];
    const int k0 = ldg_t(urp + u), k1 = ldg_t(urp + u + 1);
#pragma unroll 4
    for (int k = k0; k < k1; ++k) v += ldg_t(uval + k) * x[ldg_t(ucol + k) * Nd + d];
    if (op.nV) v = srs_vloc(op, u, d, x, v);
    yb[e] = renorm(v);
    if (want_dot) dot_add(acc, xv, v);
    r += rstep;
    d += dstep;
    if (d >= Nd) {
      d -= Nd;
      ++r;
    }
  }
}

// One item of a sector: y[lo:hi) = (H x)[lo:hi) + c z[lo:hi); accumulates <x, y> into acc.  MZ / MD: the
// launch may carry a z term / may want dot products (false removes those paths at compile time).
template <typename T, int ST, bool MZ, bool MD>
__device__ __forceinline__ void mv_item(const SectorOp<T> *opp, int srs_rows, long long li, const T *__restrict__ x,
                                        T *__restrict__ y, const T *__restrict__ z, T c, bool want_dot, DotAcc &acc,
                                        MvSmem<T> &sm) {
  if constexpr (!MZ) z = nullptr;
  if constexpr (!MD) want_dot = false;
  const SectorOp<T> &op = *opp;
  long long lo, hi;
  item_range(op, srs_rows, li, lo, hi);
  const int tid = threadIdx.x;
  if constexpr (ST == kSRS) {
    // the item's rows of x are staged in shared memory for the down-spin gathers (when they fit); for
    // long 16-byte rows the x rows its up-spin hops read are staged beside them when there is room (112 KB), so
    // that every gather of the item is a shared-memory read and all its loads are in flight at once
    const int Nd = op.dn_rows;
    const int nel = (int)(hi - lo);
    // the item's first up-spin row and row count, from item_range's own arithmetic (no division)
    const int u0 = (int)li * srs_rows;
    const int nrows = min(srs_rows, op.up_rows - u0);
    const bool staged_x = nel <= sm.xs_cap;
    constexpr int C = Lanes<T>::C;
    const uintptr_t amask = (uintptr_t)15;
    int kb = 0, nh = 0;
    bool staged_src = false;
    if (!*sm.dead && Nd >= kSrsLongRow && (Nd % C) == 0 && ((uintptr_t)x & amask) == 0 &&
        ((uintptr_t)(op.diag + lo) & amask) == 0 &&
        ((uintptr_t)(y + lo) & amask) == 0 && (!z || ((uintptr_t)(z + lo) & amask) == 0)) {
      kb = ldg_t(op.up_rp + u0);
      nh = ldg_t(op.up_rp + u0 + nrows) - kb;
      staged_src = nel + nh * Nd <= sm.xs_cap;
    }
    __syncthreads();
    if (staged_src) {
      // bulk copies issued by one thread: the item's own rows, then the row of every up-spin hop
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        const unsigned row = (unsigned)(Nd * sizeof(T));
        unsigned long long state;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;\n"
                     : "=l"(state)
                     : "r"(sm.bar), "r"((unsigned)((nel + nh * Nd) * sizeof(T)))
                     : "memory");
        const unsigned base = (unsigned)__cvta_generic_to_shared(sm.xs);
        bulk_copy(base, x + lo, (unsigned)(nel * sizeof(T)), sm.bar);
        for (int h = 0; h < nh; ++h)
          bulk_copy(base + (unsigned)(nel * sizeof(T)) + (unsigned)h * row,
                    x + (long long)ldg_t(op.up_col + kb + h) * Nd, row, sm.bar);
      }
      bool ok = wait_bulk(sm.bar, sm.phase);
      if (!ok) {
        atomicExch(&g_mv_stall, 1);
        ok = wait_bulk(sm.bar, sm.phase);  // give copies still in flight a second bounded chance
        if (!ok) *sm.dead = 1;             // the phase never completed: the barrier is not armed again
      }
    } else if (staged_x) {
      stage_async(sm.xs, x + lo, nel);
      cp_async_wait_all();
    }
    __syncthreads();
    // every thread has seen the stage's outcome: the phase advances only when it completed (uniform)
    if (staged_src && !*sm.dead) sm.phase ^= 1u;
    const T *xr = staged_x ? sm.xs : x + lo;
    if (staged_src) srs_staged<T, MZ, MD>(op, lo, u0, nrows, kb, x, sm.xs, sm.xs + nel, y, z, c, want_dot, acc);
    else if (Nd >= kSrsLongRow) {
      // rows of several thousand states, fewer than four per item: one row at a time (uniform decision)
      if (!(EDGPU_SRS_LONGROW && staged_x && nrows < EDGPU_SRS_R && Nd >= 2048 &&
            srs_longrow<T, MZ, MD>(op, lo, u0, nrows, x, sm.xs, y, z, c, want_dot, acc)))
        srs_tiled<T, MZ, MD>(op, lo, u0, nrows, x, xr, staged_x, sm.xs, y, z, c, want_dot, acc);
    }
    else srs_flat<T>(op, lo, u0, nel, x, xr, y, z, c, want_dot, acc);
  } else if constexpr (ST == kCRS) {
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

template <typename T>
__device__ __forceinline__ MvSmem<T> make_smem(unsigned char *raw, int xs_cap, MvBar *b) {
  MvSmem<T> sm;
  sm.xs = reinterpret_cast<T *>(raw);
  sm.xs_cap = xs_cap;
  if (threadIdx.x == 0) b->dead = 0;
  sm.bar = init_bulk_barrier(&b->bar);  // its __syncthreads also publishes `dead`
  sm.phase = 0;
  sm.dead = &b->dead;
  return sm;
}

// ---------------------------------------------------------------- generic batch: y = H x (+ c z)
template <typename T, int ST, bool MZ, bool MD, int MB = 2>
__global__ void __launch_bounds__(kMvBlock, MB) k_mv(const MvTask<T> *tasks, const int *item_task, int nitems, int xs_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[kMvBlock / 32];
  __shared__ __align__(8) MvBar mv_bar;
  MvSmem<T> sm = make_smem<T>(smem_raw, xs_cap, &mv_bar);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const MvTask<T> &t = tasks[item_task[it]];
    const long long li = it - t.item_begin;
    DotAcc acc;
    dot_init(acc);
    const bool want = t.dot_partial != nullptr;
    mv_item<T, ST, MZ, MD>(t.op, t.srs_rows, li, t.x, t.y, t.z, (T)t.c, want, acc, sm);
    emit_dot<T>(want, acc, want ? t.dot_partial + li : nullptr, red);
  }
}

// ---------------------------------------------------------------- Lanczos recurrence, phase 1
// Iteration it (0-based) of Lanczos.h:44-68: v = buf[it%3], w = buf[(it+1)%3] <- H v - bet * buf[(it+2)%3].
template <typename T, int ST>
__global__ void __launch_bounds__(kMvBlock, kMvMinBlocks<T>) k_lz_mv(const LzTask<T> *tasks, const int *item_task, int nitems, int iter,
                                                    int xs_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[kMvBlock / 32];
  __shared__ __align__(8) MvBar mv_bar;
  MvSmem<T> sm = make_smem<T>(smem_raw, xs_cap, &mv_bar);
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
    mv_item<T, ST, true, true>(t.op, t.srs_rows, li, x, y, z, c, true, acc, sm);
    emit_dot<T>(true, acc, t.part_a + li, red);
  }
}

// ---------------------------------------------------------------- eigen-solver step, phase 1
// w = H V[j] for tasks in Lanczos mode that still grow their basis.
template <typename T, int ST, int MB = 2>
// probe_y (the operator tuner): every task, x = V[0], into probe_y (shared scratch: the values are not used).
__global__ void __launch_bounds__(kMvBlock, MB) k_eig_mv(const EigTask<T> *tasks, const int *item_task, int nitems, int xs_cap,
                                                        T *probe_y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) MvBar mv_bar;
  MvSmem<T> sm = make_smem<T>(smem_raw, xs_cap, &mv_bar);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const EigTask<T> &t = tasks[item_task[it]];
    if (!probe_y && (t.st[2] || t.st[1] != 0)) continue;  // full, or orthogonalising a random vector (uniform)
    const long long li = it - t.item_begin;
    const T *x = probe_y ? t.V : t.V + (long long)t.st[0] * t.ldv;
    DotAcc acc;
    mv_item<T, ST, false, false>(t.op, t.srs_rows, li, x, probe_y ? probe_y : t.w, nullptr, (T)0, false, acc, sm);
  }
}

static int grid_for(const void *fn, size_t smem, int nitems) { return occupancy_grid(fn, kMvBlock, smem, nitems); }

// Opt a kernel in to `bytes` of dynamic shared memory.  Without the opt-in static and dynamic shared memory
// together are held to 48 KB; the operator kernels carry a few KB of static arrays (the long-row hop list), so
// the attribute is set from 32 KB of dynamic memory on.
template <typename K>
static void set_smem(K kernel, size_t bytes) {
  if (bytes > 32 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T>
static int xs_of(const MvShape &sh) {
  return sh.staged && sh.xs_staged > sh.xs_elems ? sh.xs_staged : sh.xs_elems;
}
template <typename T>
static size_t smem_bytes(const MvShape &sh) {
  return align16(sizeof(T) * (size_t)xs_of<T>(sh));
}

#define EDGPU_DISPATCH_ST(ST_VAR, ...)                     \
  switch (ST_VAR) {                                        \
    case kSRS: { constexpr int S_ = kSRS; __VA_ARGS__ } break;   \
    case kCRS: { constexpr int S_ = kCRS; __VA_ARGS__ } break;   \
    default: { constexpr int S_ = kSOCRS; __VA_ARGS__ } break;   \
  }

template <typename T, int ST, int MB>
static void launch_plain(const MvTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, const MvShape &sh,
                         cudaStream_t st) {
  const size_t sm = smem_bytes<T>(sh);
  set_smem(k_mv<T, ST, false, false, MB>, sm);
  k_mv<T, ST, false, false, MB><<<grid_for((const void *)k_mv<T, ST, false, false, MB>, sm, nitems_total), kMvBlock, sm,
                                  st>>>(tasks_dev, item_task_dev, nitems_total, xs_of<T>(sh));
  note_launch();
}

template <typename T>
void launch_mv(const MvTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, cudaStream_t st) {
  const size_t sm = smem_bytes<T>(sh);
  if (sh.plain) {
    EDGPU_DISPATCH_ST(sh.storage, launch_plain<T, S_, 3>(tasks_dev, item_task_dev, nitems_total, sh, st);)
  } else {
    EDGPU_DISPATCH_ST(sh.storage,
      set_smem(k_mv<T, S_, true, true>, sm);
      k_mv<T, S_, true, true><<<grid_for((const void *)k_mv<T, S_, true, true>, sm, nitems_total), kMvBlock, sm, st>>>(tasks_dev, item_task_dev, nitems_total,
                                                                            xs_of<T>(sh));
      note_launch();
    )
  }
}

template <typename T>
void launch_lz_mv(const LzTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, int it, MvShape sh,
                  cudaStream_t st) {
  const size_t sm = smem_bytes<T>(sh);
  if constexpr (std::is_same<T, ffloat>::value) {  // float-float recurrences: spin-resolved storage only
    set_smem(k_lz_mv<T, kSRS>, sm);
    k_lz_mv<T, kSRS><<<grid_for((const void *)k_lz_mv<T, kSRS>, sm, nitems_total), kMvBlock, sm, st>>>(
        tasks_dev, item_task_dev, nitems_total, it, xs_of<T>(sh));
    note_launch();
  } else {
    EDGPU_DISPATCH_ST(sh.storage,
      set_smem(k_lz_mv<T, S_>, sm);
      k_lz_mv<T, S_><<<grid_for((const void *)k_lz_mv<T, S_>, sm, nitems_total), kMvBlock, sm, st>>>(tasks_dev, item_task_dev, nitems_total, it, xs_of<T>(sh));
      note_launch();
    )
  }
}

// Kernel attributes of k_eig_mv for a shape; called before a step is captured into a graph.
template <typename T>
void prepare_eig_mv(MvShape sh) {
  const size_t sm = smem_bytes<T>(sh);
  EDGPU_DISPATCH_ST(sh.storage,
    if (sh.mb >= 3) set_smem(k_eig_mv<T, S_, 3>, sm);
    else set_smem(k_eig_mv<T, S_, 2>, sm);
  )
}

template <typename T>
void launch_eig_mv(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, cudaStream_t st,
                   T *probe_y) {
  const size_t sm = smem_bytes<T>(sh);
  EDGPU_DISPATCH_ST(sh.storage,
    if (sh.mb >= 3)
      k_eig_mv<T, S_, 3><<<grid_for((const void *)k_eig_mv<T, S_, 3>, sm, nitems_total), kMvBlock, sm, st>>>(
          tasks_dev, item_task_dev, nitems_total, xs_of<T>(sh), probe_y);
    else
      k_eig_mv<T, S_, 2><<<grid_for((const void *)k_eig_mv<T, S_, 2>, sm, nitems_total), kMvBlock, sm, st>>>(
          tasks_dev, item_task_dev, nitems_total, xs_of<T>(sh), probe_y);
    note_launch();
  )
}

template <typename T>
OpTuning tune_eig_mv(const EigTask<T> *tasks_dev, const int *item_task_dev, int nitems_total, MvShape sh, T *probe_y,
                     cudaStream_t st) {
  OpTuning best;
  best.done = true;
  best.ms = 1e30;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return best;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return best;
  }
  const int nstaged = sh.storage == kSRS && sh.xs_staged > sh.xs_elems ? 2 : 1;
  for (int staged = 0; staged < nstaged; ++staged)
    for (int mb = 2; mb <= 3; ++mb) {
      MvShape v = sh;
      v.staged = staged;
      v.mb = mb;
      prepare_eig_mv<T>(v);
      launch_eig_mv<T>(tasks_dev, item_task_dev, nitems_total, v, st, probe_y);  // warm
      cudaEventRecord(e0, st);
      for (int r = 0; r < 3; ++r) launch_eig_mv<T>(tasks_dev, item_task_dev, nitems_total, v, st, probe_y);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms / 3.0 < best.ms) {
        best.ms = ms / 3.0;
        best.mb = mb;
        best.staged = staged;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

// Reads and clears the stalled-bulk-copy flag of the operator kernels (after the stream is synchronised).
bool take_mv_stall() {
  int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_mv_stall, sizeof(int)) != cudaSuccess) return false;
  if (v) cudaMemcpyToSymbol(g_mv_stall, &zero, sizeof(int));
  return v != 0;
}

// Self-test of the bounded wait: thread 0 arms an mbarrier for 16 bytes that no copy delivers, then takes
// the operator's path for a copy that does not complete -- a bounded wait of `rounds` try_wait rounds, the
// stall flag, a second bounded wait -- and records in *gave_up whether both waits gave up.
__global__ void k_wait_selftest(int rounds, int *gave_up) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const unsigned b = (unsigned)__cvta_generic_to_shared(&bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  unsigned long long state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;\n" : "=l"(state) : "r"(b), "r"(16u) : "memory");
  bool ok = wait_bulk(b, 0u, rounds);
  if (!ok) {
    atomicExch(&g_mv_stall, 1);
    ok = wait_bulk(b, 0u, rounds);
  }
  *gave_up = ok ? 0 : 1;
}

void launch_wait_selftest(int rounds, int *gave_up_dev, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(rounds, gave_up_dev);
  note_launch();
}

template void launch_mv<float>(const MvTask<float> *, const int *, int, MvShape, cudaStream_t);
template void launch_mv<double>(const MvTask<double> *, const int *, int, MvShape, cudaStream_t);
template void launch_lz_mv<float>(const LzTask<float> *, const int *, int, int, MvShape, cudaStream_t);
template void launch_lz_mv<double>(const LzTask<double> *, const int *, int, int, MvShape, cudaStream_t);
template void launch_lz_mv<ffloat>(const LzTask<ffloat> *, const int *, int, int, MvShape, cudaStream_t);
template void prepare_eig_mv<float>(MvShape);
template void prepare_eig_mv<double>(MvShape);
template void launch_eig_mv<float>(const EigTask<float> *, const int *, int, MvShape, cudaStream_t, float *);
template void launch_eig_mv<double>(const EigTask<double> *, const int *, int, MvShape, cudaStream_t, double *);
template OpTuning tune_eig_mv<float>(const EigTask<float> *, const int *, int, MvShape, float *, cudaStream_t);
template OpTuning tune_eig_mv<double>(const EigTask<double> *, const int *, int, MvShape, double *, cudaStream_t);

}  // namespace edgpu
