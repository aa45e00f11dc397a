// Self-energy from the Dyson equation on the device.
//
// GreensFunction::compute_selfenergy (include/edlib/GreensFunction.h:202-222) builds the model's bare
// Green's function on the mesh of G_ij and solves Sigma = G0^-1 - G^-1 per frequency and spin
// (FermionicModel::solve_dyson, include/edlib/FermionicModel.h:83-108).  The bare inverse is known in
// closed form, so the device builds G0^-1 directly and inverts two n x n complex matrices per (w, spin):
//
// * Hubbard (HubbardModel.h:180-201): G0^-1_IJ = (z + xmu_I) delta_IJ + t_IJ (the site shift _Eps is
//   never read from the input, so it is zero).
// * Anderson impurity (SingleImpurityAndersonModel.h:377-391): G0^-1 is diagonal over the impurity
//   orbitals, G0^-1_mm = z - H0_mm - sum_k V_mk^2 / (z - eps_k); the reference drops H0's off-diagonal
//   and any off-diagonal hybridisation, and so does this.
//
// z is i w_n on the Matsubara mesh and w + i pi / beta on the real one (CommonUtils.h:14-20).  One warp
// owns one matrix, lane j one column; the inversion is in-place Gauss-Jordan with partial (row) pivoting
// in FP64, the matrix in shared memory.  A zero pivot marks the (w, spin) singular instead of writing
// infinities; the host turns that into an error.
#include "model_internal.h"

namespace edgpu {

namespace {

constexpr int kDysonWarps = 4;

struct Cplx {
  double re, im;
};

__device__ __forceinline__ Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Cplx csub(Cplx a, Cplx b) { return {a.re - b.re, a.im - b.im}; }

// a / b by Smith's algorithm (R. L. Smith, "Algorithm 116: Complex division", CACM 5(8), 1962), which
// scales by the larger component of b so neither |b|^2 nor the products overflow.
__device__ __forceinline__ Cplx cdiv(Cplx a, Cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  const double r = b.re / b.im, d = b.re * r + b.im;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

// In-place inverse of the n x n matrix a (row-major, leading dimension n) by the warp; lane j < n owns
// column j.  perm and col are n-entry scratch.  Returns false (all lanes) on a zero pivot.
__device__ bool warp_invert(Cplx *a, int n, int *perm, Cplx *col) {
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < n; ++k) {
    // pivot: the largest |a_ik| for i >= k, the lowest row on ties
    double best = -1.0;
    int arg = k;
    if (lane >= k && lane < n) {
      const Cplx x = a[lane * n + k];
      best = x.re * x.re + x.im * x.im;
      arg = lane;
    }
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
      if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
    }
    if (!(best > 0.0)) return false;
    if (lane == 0) perm[k] = arg;
    if (arg != k && lane < n) {
      const Cplx t = a[k * n + lane];
      a[k * n + lane] = a[arg * n + lane];
      a[arg * n + lane] = t;
    }
    __syncwarp();
    const Cplx piv = a[k * n + k];
    if (lane < n) col[lane] = a[lane * n + k];
    __syncwarp();
    // row k: a_kj / piv, with a_kk taking 1 / piv
    if (lane < n) a[k * n + lane] = cdiv(lane == k ? Cplx{1.0, 0.0} : a[k * n + lane], piv);
    __syncwarp();
    // every other row: a_ij - a_ik a_kj, with a_ik taking -a_ik / piv
    if (lane < n) {
      const Cplx rk = a[k * n + lane];
      for (int i = 0; i < n; ++i) {
        if (i == k) continue;
        const Cplx f = col[i];
        a[i * n + lane] = lane == k ? Cplx{-(f.re * rk.re - f.im * rk.im), -(f.re * rk.im + f.im * rk.re)}
                                    : csub(a[i * n + lane], cmul(f, rk));
      }
    }
    __syncwarp();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = n - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k && lane < n) {
      const Cplx t = a[lane * n + k];
      a[lane * n + k] = a[lane * n + p];
      a[lane * n + p] = t;
    }
    __syncwarp();
  }
  return true;
}

// One warp per (w, spin).  G, G0 and Sigma are [nw][n*n][2 spins] complex (re, im interleaved), the
// layout of GreensFunction::G_ij.  kind 0 = Hubbard (D[n*n] = xmu_I delta_IJ + t_IJ), kind 1 = Anderson
// impurity (h0d[n][2] = H0_mm per spin, epsk[nk][2], vk[n][nk][2]).
__global__ void __launch_bounds__(32 * kDysonWarps)
k_dyson(const double *__restrict__ G, const double2 *__restrict__ z, int nw, int n, int kind,
        const double *__restrict__ D, const double *__restrict__ h0d, const double *__restrict__ epsk,
        const double *__restrict__ vk, int nk, double *__restrict__ G0, double *__restrict__ Sig,
        int *__restrict__ singular) {
  extern __shared__ __align__(16) unsigned char dyson_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int job = blockIdx.x * kDysonWarps + warp;
  if (job >= 2 * nw) return;  // whole warps leave together
  const int w = job >> 1, s = job & 1;
  const int nn = n * n;
  Cplx *g0i = reinterpret_cast<Cplx *>(dyson_smem) + (size_t)warp * (2 * nn + n);
  Cplx *a = g0i + nn, *col = a + nn;
  int *perm = reinterpret_cast<int *>(reinterpret_cast<Cplx *>(dyson_smem) + (size_t)kDysonWarps * (2 * nn + n)) +
              warp * n;
  const Cplx zz{z[w].x, z[w].y};
  // G0^-1, kept for Sigma, and a copy to invert into G0
  for (int e = lane; e < nn; e += 32) {
    const int I = e / n, J = e - I * n;
    Cplx x{0.0, 0.0};
    if (kind == 0) {
      x.re = D[e];
      if (I == J) { x.re += zz.re; x.im += zz.im; }
    } else if (I == J) {
      Cplx delta{0.0, 0.0};
      for (int k = 0; k < nk; ++k) {
        const double v = vk[((size_t)I * nk + k) * 2 + s];
        const Cplx t = cdiv(Cplx{v * v, 0.0}, Cplx{zz.re - epsk[2 * k + s], zz.im});
        delta.re += t.re;
        delta.im += t.im;
      }
      x = Cplx{zz.re - h0d[2 * I + s] - delta.re, zz.im - delta.im};
    }
    g0i[e] = x;
    a[e] = x;
  }
  __syncwarp();
  const size_t base = (size_t)w * nn * 2;
  bool ok = warp_invert(a, n, perm, col);
  if (ok && G0) {
    for (int e = lane; e < nn; e += 32) {
      const size_t o = ((base + (size_t)e * 2) + s) * 2;
      G0[o] = a[e].re;
      G0[o + 1] = a[e].im;
    }
  }
  __syncwarp();
  for (int e = lane; e < nn; e += 32) {
    const size_t o = ((base + (size_t)e * 2) + s) * 2;
    a[e] = Cplx{G[o], G[o + 1]};
  }
  __syncwarp();
  ok = ok && warp_invert(a, n, perm, col);
  if (!ok) {
    if (lane == 0) singular[job] = 1;
    return;
  }
  if (Sig) {
    for (int e = lane; e < nn; e += 32) {
      const size_t o = ((base + (size_t)e * 2) + s) * 2;
      const Cplx x = csub(g0i[e], a[e]);
      Sig[o] = x.re;
      Sig[o + 1] = x.im;
    }
  }
}

}  // namespace

namespace host {

int self_energy_dispatch(edgpu_model *m, const edgpu_gf_params *p, const double *Gij, double *G0, double *Sigma) {
  edgpu_ctx *c = m->ctx;
  const int n = m->interacting();
  const int nw = p->nomega;
  if (nw < 1) throw ApiError(EDGPU_ERR_ARG, "NOMEGA must be positive");
  if (!(p->beta > 0)) throw ApiError(EDGPU_ERR_ARG, "BETA must be positive");
  if (n > 32) throw ApiError(EDGPU_ERR_ARG, "the Dyson solve takes at most 32 interacting orbitals");
  std::vector<double2> z(nw);
  if (p->mesh == EDGPU_MESH_REAL) {
    // RealFreqMeshFactory (MeshFactory.h:27-34), evaluated at w + i pi / beta (CommonUtils.h:18-20)
    if (nw < 2 || !(p->emax > p->emin)) throw ApiError(EDGPU_ERR_ARG, "the real mesh needs NOMEGA >= 2 and EMAX > EMIN");
    for (int w = 0; w < nw; ++w) z[w] = make_double2(p->emin + (p->emax - p->emin) * w / double(nw - 1), M_PI / p->beta);
  } else {
    for (int w = 0; w < nw; ++w) z[w] = make_double2(0.0, (2.0 * w + 1) * M_PI / p->beta);
  }
  std::vector<double> D, h0d, epsk, vk;
  int nk = 0;
  if (m->kind == 0) {
    D.assign(m->t.begin(), m->t.end());
    for (int i = 0; i < n; ++i) D[(size_t)i * n + i] += m->xmu[i];
  } else {
    nk = m->ns - m->ml;
    h0d.resize(2 * n);
    for (int i = 0; i < n; ++i)
      for (int s = 0; s < 2; ++s) h0d[2 * i + s] = m->h0[((size_t)i * n + i) * 2 + s];
    epsk = m->epsk;
    vk = m->vk;
  }
  const size_t nel = (size_t)nw * n * n * 2 * 2;
  DBuf dG = DBuf(c->alloc, sizeof(double) * nel);
  CK(cudaMemcpyAsync(dG.p, Gij, sizeof(double) * nel, cudaMemcpyHostToDevice, c->stream));
  DBuf dz = upload(c, z), dD = upload(c, D), dh0 = upload(c, h0d), de = upload(c, epsk), dv = upload(c, vk);
  DBuf dG0, dS;
  if (G0) dG0 = DBuf(c->alloc, sizeof(double) * nel);
  if (Sigma) dS = DBuf(c->alloc, sizeof(double) * nel);
  DBuf dsing(c->alloc, sizeof(int) * 2 * nw);
  CK(cudaMemsetAsync(dsing.p, 0, dsing.bytes, c->stream));
  const size_t smem = (size_t)kDysonWarps * ((2 * n * n + n) * sizeof(Cplx) + n * sizeof(int));
  const int blocks = (2 * nw + kDysonWarps - 1) / kDysonWarps;
  if (smem > 48 * 1024) CK(cudaFuncSetAttribute(k_dyson, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_dyson<<<blocks, 32 * kDysonWarps, smem, c->stream>>>(
      (const double *)dG.p, (const double2 *)dz.p, nw, n, m->kind, (const double *)dD.p, (const double *)dh0.p,
      (const double *)de.p, (const double *)dv.p, nk, G0 ? (double *)dG0.p : nullptr,
      Sigma ? (double *)dS.p : nullptr, (int *)dsing.p);
  CK(cudaGetLastError());
  std::vector<int> sing(2 * nw);
  CK(cudaMemcpyAsync(sing.data(), dsing.p, sizeof(int) * 2 * nw, cudaMemcpyDeviceToHost, c->stream));
  if (G0) CK(cudaMemcpyAsync(G0, dG0.p, sizeof(double) * nel, cudaMemcpyDeviceToHost, c->stream));
  if (Sigma) CK(cudaMemcpyAsync(Sigma, dS.p, sizeof(double) * nel, cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  for (int j = 0; j < 2 * nw; ++j)
    if (sing[j])
      throw ApiError(EDGPU_ERR_ARG, "G_ij is singular at frequency " + std::to_string(j / 2) + ", spin " +
                                        std::to_string(j % 2) +
                                        " (an orbital missing from GreensFunction_orbitals leaves a zero row)");
  return EDGPU_OK;
}

}  // namespace host
}  // namespace edgpu
