// Internal device-side definitions of the GB300 ED library (not part of the C ABI).
//
// Fock-state conventions (bit-exact with the reference, include/edlib/FermionicModel.h:35-68 and
// include/edlib/SzSymmetry.h:114-133):
//   spin-orbital im (spin-up orbital m -> im = m, spin-down -> im = m + Ns) is bit 2Ns-1-im;
//   the up occupations are the high Ns bits, the down occupations the low Ns bits;
//   the sign of c_im / c+_im is (-1)^(number of occupied spin-orbitals with index < im), i.e. the
//   parity of the bits ABOVE position 2Ns-1-im, which is one popc.
//   The index of state (up, dn) in sector (N_up, N_dn) is ninv[N_up][up] * C(Ns, N_dn) + ninv[N_dn][dn].
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cfloat>
#include <type_traits>

namespace edgpu {

typedef long long state_t;

constexpr int kMaxNs = 20;  // orbitals per spin: states use 2*Ns <= 40 bits, ninv has 2^Ns entries per row

// A hopping c+_b c_a (quad == 0) or a Coulomb term c+_i c+_j c_l c_k (quad == 1), indices are
// spin-orbitals.  value/sign_factor follow the reference transition objects:
// HubbardModel.h:99-108 (value t, sign -isign1*isign2) and SingleImpurityAndersonModel.h:77-84,
// 153-168 (value V or U/2, sign +product of the operator signs).
struct Transition {
  int quad;
  int a, b;        // hop: annihilate a, create b
  int k, l, j, i;  // quad: annihilate k, annihilate l, create j, create i
  double value;
  int sign_factor;
  int spin;        // hop: spin of both operators (0 up, 1 down); quad: -1
};

__host__ __device__ inline int occ(state_t s, int im, int ip) { return (int)((s >> (ip - 1 - im)) & 1); }

__host__ __device__ inline int parity_sign(state_t s, int im, int ip) {
#ifdef __CUDA_ARCH__
  int c = __popcll((unsigned long long)s >> (ip - im));
#else
  int c = __builtin_popcountll((unsigned long long)s >> (ip - im));
#endif
  return (c & 1) ? -1 : 1;
}

// validity of a transition on state nst (HubbardModel.h:86-88; SingleImpurityAndersonModel.h:74-76, 129-142)
__host__ __device__ inline int trans_valid(const Transition &tr, state_t nst, int ip) {
  if (!tr.quad) return occ(nst, tr.a, ip) & (1 - occ(nst, tr.b, ip));
  if (occ(nst, tr.k, ip)) {
    state_t k3 = nst - (1ll << (ip - 1 - tr.k));
    if (occ(k3, tr.l, ip)) {
      state_t k4 = k3 - (1ll << (ip - 1 - tr.l));
      if (!occ(k4, tr.j, ip)) {
        state_t k2 = k4 | (1ll << (ip - 1 - tr.j));
        return 1 - occ(k2, tr.i, ip);
      }
    }
  }
  return 0;
}

// target state and sign of a valid transition
__host__ __device__ inline state_t trans_apply(const Transition &tr, state_t nst, int ip, int &sign) {
  if (!tr.quad) {
    int s1 = parity_sign(nst, tr.a, ip);
    state_t k1 = nst - (1ll << (ip - 1 - tr.a));
    int s2 = parity_sign(k1, tr.b, ip);
    sign = tr.sign_factor * s1 * s2;
    return k1 + (1ll << (ip - 1 - tr.b));
  }
  int s1 = parity_sign(nst, tr.k, ip);
  state_t k3 = nst - (1ll << (ip - 1 - tr.k));
  int s2 = parity_sign(k3, tr.l, ip);
  state_t k4 = k3 - (1ll << (ip - 1 - tr.l));
  int s3 = parity_sign(k4, tr.j, ip);
  state_t k2 = k4 + (1ll << (ip - 1 - tr.j));
  int s4 = parity_sign(k2, tr.i, ip);
  sign = s1 * s2 * s3 * s4;
  return k2 + (1ll << (ip - 1 - tr.i));
}

// Model data needed on the device for diagonal elements and matrix-free transitions.
struct DevModel {
  int kind;  // 0 Hubbard, 1 single-impurity Anderson
  int ns, ip, ml;
  int nT, nV;
  const Transition *T;
  const Transition *V;
  // Hubbard (HubbardModel.h:116-132)
  const double *U, *xmu, *hmag, *J;
  // Anderson (SingleImpurityAndersonModel.h:282-306)
  const double *epsk, *h0, *Ut;
  double mu;
  // tables
  const long long *binom;  // binom[n * (kMaxNs + 2) + k]
  const int *basis;        // concatenated per particle number
  const long long *basis_off;
  const int *ninv;         // ninv[k << ns | mask]
};

__host__ __device__ inline long long binom_at(const long long *b, int n, int k) {
  if (n < 0 || k < 0 || k > n) return 0;
  return b[n * (kMaxNs + 2) + k];
}

// <s|H|s> in the loop order of the reference models
__device__ inline double model_diagonal(const DevModel &m, state_t st) {
  double x = 0.0;
  const int ns = m.ns, ip = m.ip;
  if (m.kind == 0) {
    for (int im = 0; im < ns; ++im) {
      for (int is = 0; is < 2; ++is) x += (0.0 - m.xmu[is]) * occ(st, im + is * ns, ip);
      x += m.U[im] * occ(st, im, ip) * occ(st, im + ns, ip);
      x += m.hmag[im] * (occ(st, im + ns, ip) - occ(st, im, ip));
      if (m.J)
        for (int im2 = 0; im2 < ns; ++im2)
          x += m.J[im * ns + im2] * (occ(st, im, ip) - occ(st, im + ns, ip)) * (occ(st, im2, ip) - occ(st, im2 + ns, ip));
    }
  } else {
    const int ml = m.ml, nk = ns - ml;
    auto Ut = [&](int s1, int s2, int i, int j, int k, int l) {
      return m.Ut[((((s1 * 2 + s2) * ml + i) * ml + j) * ml + k) * ml + l];
    };
    for (int is = 0; is < 2; ++is)
      for (int ik = 0; ik < nk; ++ik) x += (m.epsk[ik * 2 + is] * occ(st, ik + ml + is * ns, ip));
    for (int im = 0; im < ml; ++im) {
      for (int is = 0; is < 2; ++is) x += (m.h0[(im * ml + im) * 2 + is] - m.mu) * occ(st, im + is * ns, ip);
      for (int is = 0; is < 2; ++is) x += 0.5 * Ut(is, is, im, im, im, im) * occ(st, im, ip) * occ(st, im + ns, ip);
      for (int jm = 0; jm < ml; ++jm)
        for (int is = 0; is < 2; ++is)
          if (im != jm) {
            x += 0.5 * (Ut(is, is, im, jm, im, jm) - Ut(is, is, im, jm, jm, im)) * occ(st, im + is * ns, ip) *
                 occ(st, jm + is * ns, ip);
            x += 0.5 * (Ut(is, 1 - is, im, jm, im, jm)) * occ(st, im + is * ns, ip) * occ(st, jm + (1 - is) * ns, ip);
          }
    }
  }
  return x;
}

enum StorageKind { kCRS = 0, kSRS = 1, kSOCRS = 2 };

// Everything a Hamiltonian-times-vector kernel needs for one symmetry sector (N_up, N_dn).
template <typename T>
struct SectorOp {
  int storage;
  int ns, ip, nup, ndn;
  long long dim;      // C(Ns,N_up) * C(Ns,N_dn)
  int up_rows, dn_rows;  // C(Ns,N_up), C(Ns,N_dn)
  const T *diag;      // [dim]
  // spin-resolved Kronecker pieces (SpinResolvedStorage.h:622-638)
  const int *up_rp, *up_col;
  const T *up_val;
  const int *dn_rp, *dn_col;
  const T *dn_val;
  int dn_nnz;         // non-zeros of the down-spin CSR
  // the same down-spin matrix k-major ("ELL"): entry k of row d at [k * dn_ld + d], row lengths dn_len[d];
  // dn_ld = dn_rows rounded up to 4, so 4 consecutive rows load as one 16-byte vector
  const int *dn_len, *dn_ell_col;
  const T *dn_ell_val;
  int dn_ld;
  // plain CSR (CRSStorage.h:66-83), diagonal first in each row
  const long long *crs_rp;
  const int *crs_col;
  const T *crs_val;
  // tables for state <-> index and matrix-free transitions
  const int *up_basis, *dn_basis;    // masks of the C(Ns,N) states
  const int *ninv_up, *ninv_dn;      // ninv rows for N_up, N_dn
  int nT, nV;
  const Transition *T_;
  const Transition *V_;
  const T *T_val;                    // transition values in vector precision
  const T *V_val;
};

template <typename T>
__device__ inline state_t sector_state(const SectorOp<T> &op, long long i) {
  long long u = i / op.dn_rows, d = i - u * op.dn_rows;
  return ((state_t)op.up_basis[u] << op.ns) | (state_t)op.dn_basis[d];
}

template <typename T>
__device__ inline long long sector_index(const SectorOp<T> &op, state_t s) {
  int up = (int)(s >> op.ns), dn = (int)(s & ((1ll << op.ns) - 1));
  return (long long)op.ninv_up[up] * op.dn_rows + op.ninv_dn[dn];
}

// ---------------------------------------------------------------- reductions
// Dot products of FP32 vectors are accumulated per thread in float-float (exact products via
// fma, Knuth two-sum), then combined in FP64 across threads.  FP64 vectors accumulate in FP64.
// A value held to about 2^-48 relative as the unevaluated sum hi + lo of two FP32 numbers ("float-float",
// Dekker's double-length arithmetic restated with fused multiply-adds): the vectors of the mixed mode's
// Green's-function and susceptibility recurrences.  GB300 issues FP64 at 1/64 of its FP32 rate, so FP64-accurate
// sums built from FP32 operations (about 15 per multiply-add) run several times faster than FP64 itself.  A
// value occupies 8 bytes (hi, lo), like an FP64 element.
struct __align__(8) ffloat {
  float hi, lo;
  ffloat() = default;
  __host__ __device__ constexpr ffloat(float h, float l) : hi(h), lo(l) {}
  // nearest float-float of an FP64 value (hi = x rounded to FP32, lo = the rest rounded to FP32)
  __host__ __device__ explicit ffloat(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
};
__host__ __device__ inline double ff_value(ffloat a) { return (double)a.hi + (double)a.lo; }
// a + b: exact sum of the high parts (two-sum), the low parts added to its error.  Not renormalised: sums of a
// few terms keep |lo| within a few ulp of hi; every value is renormalised once when it is stored (renorm, the
// stores of the recurrence kernels), which also restores hi after a cancellation.
// (Device code uses the _rn intrinsics, which the compiler never contracts into fused multiply-adds: the
// error-free transformations need every product and sum rounded on its own.)
__host__ __device__ __forceinline__ float ff_add_rn(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(x, y);
#else
  return x + y;
#endif
}
__host__ __device__ __forceinline__ float ff_sub_rn(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(x, y);
#else
  return x - y;
#endif
}
__host__ __device__ __forceinline__ ffloat operator+(ffloat a, ffloat b) {
  const float s = ff_add_rn(a.hi, b.hi);
  const float bb = ff_sub_rn(s, a.hi);
  float e = ff_add_rn(ff_sub_rn(a.hi, ff_sub_rn(s, bb)), ff_sub_rn(b.hi, bb));
  e = ff_add_rn(ff_add_rn(e, a.lo), b.lo);
  return ffloat(s, e);
}
__host__ __device__ __forceinline__ ffloat operator-(ffloat a) { return ffloat(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ ffloat operator-(ffloat a, ffloat b) { return a + (-b); }
// a * b: exact product of the high parts (its rounding error by a fused multiply-add) plus the cross terms;
// the result is left unnormalised (|lo| a few ulp of hi), which the next addition absorbs
__host__ __device__ __forceinline__ ffloat operator*(ffloat a, ffloat b) {
#ifdef __CUDA_ARCH__
  const float p = __fmul_rn(a.hi, b.hi);
#else
  const float p = a.hi * b.hi;
#endif
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return ffloat(p, e);
}
__host__ __device__ __forceinline__ ffloat &operator+=(ffloat &a, ffloat b) {
  a = a + b;
  return a;
}

// A float-float value with |lo| <= ulp(hi) / 2 again (after a product); FP32 and FP64 values unchanged.
template <typename T>
__host__ __device__ __forceinline__ T renorm(T x) {
  return x;
}
template <>
__host__ __device__ __forceinline__ ffloat renorm<ffloat>(ffloat x) {
  const float h = ff_add_rn(x.hi, x.lo);
  return ffloat(h, ff_sub_rn(x.lo, ff_sub_rn(h, x.hi)));
}

// Read-only-path load of one element (FP32, FP64, int or float-float).
template <typename T>
__device__ __forceinline__ T ldg_t(const T *p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ ffloat ldg_t<ffloat>(const ffloat *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return ffloat(v.x, v.y);
}

struct DotAcc {
  float hi, lo;
  double d;
};

__device__ inline void dot_init(DotAcc &a) { a.hi = 0.f; a.lo = 0.f; a.d = 0.0; }
__device__ inline void dot_add(DotAcc &a, float x, float y) {
  float p = x * y;
  float pe = fmaf(x, y, -p);
  float s = a.hi + p;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (p - bb);
  a.hi = s;
  a.lo += e + pe;
}
__device__ inline void dot_add(DotAcc &a, double x, double y) { a.d = fma(x, y, a.d); }
// float-float data: the product in float-float, summed into the float-float accumulator (hi, lo)
__device__ inline void dot_add(DotAcc &a, ffloat x, ffloat y) {
  const ffloat p = x * y;
  const float s = __fadd_rn(a.hi, p.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(p.hi, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, __fadd_rn(e, p.lo));
}
__device__ inline double dot_value(const DotAcc &a) { return (double)a.hi + (double)a.lo + a.d; }

// Merging accumulators without FP64 arithmetic (GB300 issues FP64 at a small fraction of the FP32 rate):
// float-float sums for FP32 data, plain double for FP64 data.
__device__ inline void ff_add(float &hi, float &lo, float bh, float bl) {
  const float s = hi + bh;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (bh - bb);
  hi = s;
  lo = lo + bl + e;
}
template <typename T>
__device__ inline void dot_merge(DotAcc &a, const DotAcc &b) {
  if constexpr (sizeof(T) == 4 || std::is_same<T, ffloat>::value) ff_add(a.hi, a.lo, b.hi, b.lo);
  else a.d += b.d;
}
// warp-wide sum of an accumulator of T data (fixed shuffle tree), valid in lane 0
template <typename T>
__device__ inline void dot_warp_sum(DotAcc &a) {
  for (int o = 16; o > 0; o >>= 1) {
    if constexpr (sizeof(T) == 4) {
      const float bh = __shfl_down_sync(0xffffffffu, a.hi, o);
      const float bl = __shfl_down_sync(0xffffffffu, a.lo, o);
      ff_add(a.hi, a.lo, bh, bl);
    } else {
      a.d += __shfl_down_sync(0xffffffffu, a.d, o);
    }
  }
}

// One bulk (TMA) copy, issued by one thread, of `bytes` (a multiple of 16, both ends 16-byte aligned) into the stage at
// shared address dst, completing on the stage's full barrier.
__device__ __forceinline__ void stage_copy(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
  // the block's generic-proxy reads of the stage (ordered by its empty barrier) precede the copy's writes
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  unsigned long long state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;\n" : "=l"(state) : "r"(bar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// 16 bytes of vector elements (4 FP32 or 2 FP64) in registers
template <typename T>
struct alignas(16) Lanes {
  static constexpr int C = 16 / sizeof(T);
  T v[C];
};
template <typename T>
__device__ __forceinline__ void store_lanes(T *p, const T *v) {
  if constexpr (std::is_same<T, ffloat>::value) {
    const ffloat a = renorm(v[0]), b = renorm(v[1]);
    *reinterpret_cast<float4 *>(p) = make_float4(a.hi, a.lo, b.hi, b.lo);
  }
  else if constexpr (sizeof(T) == 4) *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  else *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}
template <typename T>
__device__ __forceinline__ Lanes<T> load16(const T *p) {
  Lanes<T> q;
  if constexpr (std::is_same<T, ffloat>::value) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    q.v[0] = ffloat(f.x, f.y), q.v[1] = ffloat(f.z, f.w);
  } else if constexpr (sizeof(T) == 4) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    q.v[0] = f.x, q.v[1] = f.y, q.v[2] = f.z, q.v[3] = f.w;
  } else {
    const double2 f = *reinterpret_cast<const double2 *>(p);
    q.v[0] = f.x, q.v[1] = f.y;
  }
  return q;
}

// Block-wide asynchronous copy of n contiguous elements global -> shared (cp.async: every load is in
// flight at once instead of one round trip per loop iteration).  16-byte copies when both ends are
// 16-byte aligned and the length is a whole number of 16-byte pieces, else element copies.  Completes at
// cp_async_wait_all() + __syncthreads().
template <typename T>
__device__ __forceinline__ void stage_async(T *smem, const T *g, int n) {
  const unsigned s0 = (unsigned)__cvta_generic_to_shared(smem);
  if (((uintptr_t)g & 15) == 0 && (s0 & 15) == 0 && ((size_t)n * sizeof(T)) % 16 == 0) {
    const int nv = (int)(((size_t)n * sizeof(T)) / 16);
    for (int q = threadIdx.x; q < nv; q += blockDim.x)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s0 + 16u * q), "l"(g + q * (16 / sizeof(T))));
  } else {
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s0 + 8u * q), "l"(g + q));
      else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s0 + 4u * q), "l"(g + q));
    }
  }
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// block-wide sum of a double, result valid in thread 0
template <int BLOCK>
__device__ inline double block_sum(double v, double *smem) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double r = 0.0;
  const int nwarps = (blockDim.x + 31) >> 5;  // <= BLOCK / 32
  if (threadIdx.x == 0)
    for (int w = 0; w < nwarps; ++w) r += smem[w];
  return r;
}

// ---------------------------------------------------------------- continued fraction
__device__ inline double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ inline double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

__device__ inline double2 frac_point(const double *alpha, const double *beta, int nlanc, int isign, double scale, double2 z) {
  if (nlanc <= 0) return make_double2(0.0, 0.0);
  auto dl = [&](int i) { return make_double2(z.x - alpha[i] * isign, z.y); };
  if (nlanc == 1) return cdiv(make_double2(scale, 0.0), dl(0));
  double2 d2 = dl(nlanc - 1);                                  // det_{i+2}
  double2 d1 = cmul(dl(nlanc - 2), dl(nlanc - 1));             // det_{i+1}
  double b = beta[nlanc - 1];
  d1.x -= b * b;
  const double big = (double)FLT_MAX / 2.0;
  const double shift = 1.0 / ((double)FLT_MAX / 1000.0);
  // |d0| > big decided from |d0|^2 away from the threshold (a relative margin of 2^-20, far above the
  // roundings of the square), by hypot only within it: the same decisions as hypot alone, without its cost
  const double big2_hi = big * big * (1.0 + 0x1p-20), big2_lo = big * big * (1.0 - 0x1p-20);
  for (int i = nlanc - 3; i >= 0; --i) {
    double bb = beta[i + 1] * beta[i + 1];
    double2 d0 = cmul(dl(i), d1);
    d0.x -= bb * d2.x;
    d0.y -= bb * d2.y;
    const double n2 = d0.x * d0.x + d0.y * d0.y;
    const bool over = n2 > big2_hi ? true : (n2 < big2_lo ? false : hypot(d0.x, d0.y) > big);
    if (over && i != 0) {
      d0.x *= shift; d0.y *= shift;
      d1.x *= shift; d1.y *= shift;
    }
    d2 = d1;
    d1 = d0;
  }
  // d1 = det_0, d2 = det_1
  return cdiv(make_double2(scale * d2.x, scale * d2.y), d1);
}

}  // namespace edgpu
