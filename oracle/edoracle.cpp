// edoracle — CPU restatement of EDLib's exact-diagonalisation hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is checked against
// (tests, the smoke check and the CPU baseline of the benchmark).  Nothing in the product
// links, loads or calls it.  It restates, function by function and in the same arithmetic
// order, the reference algorithms cited beside each routine (paths are relative to the
// reference project root).  Its results are pinned against the reference's own golden files
// and against the reference headers compiled unmodified (oracle/refshim).
//
// Conventions restated from the reference:
//  * spin-orbital im (spin-up orbital m: im = m, spin-down: im = m + Ns) is bit 2Ns-1-im of
//    the Fock state (include/edlib/FermionicModel.h:35-37); up occupations are the high Ns
//    bits, down the low Ns bits (include/edlib/SzSymmetry.h:114-121);
//  * fermion sign of c_i / c+_i = (-1)^(number of occupied spin-orbitals with index < i)
//    (include/edlib/FermionicModel.h:45-68).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef long long state_t;

// ---------------------------------------------------------------- combinatorics
// include/edlib/Combination.h:13-78
struct Binomial {
  std::vector<std::vector<int64_t>> c;
  explicit Binomial(int n) : c(n + 2, std::vector<int64_t>(n + 2, 0)) {
    for (int i = 0; i <= n + 1; ++i) {
      c[i][0] = 1;
      for (int j = 1; j <= i; ++j) c[i][j] = c[i - 1][j - 1] + (j <= i - 1 ? c[i - 1][j] : 0);
    }
  }
  int64_t operator()(int n, int k) const {
    if (n < 0 || k < 0 || k > n || n >= (int)c.size()) return 0;
    return c[n][k];
  }
};

// Per-particle-number basis in the order of Combination::next_combination (lexicographic on
// the sorted position tuple, starting from {0..k-1}) and the dense inverse table.
// include/edlib/SzSymmetry.h:191-216
struct SpinBasis {
  int ns = 0;
  std::vector<std::vector<int>> basis;  // basis[k][r] = bit mask
  std::vector<std::vector<int>> ninv;   // ninv[k][mask] = r
  void build(int n) {
    ns = n;
    basis.assign(n + 1, {});
    ninv.assign(n + 1, std::vector<int>(size_t(1) << n, 0));
    for (int k = 0; k <= n; ++k) {
      std::vector<int> pos(k);
      for (int i = 0; i < k; ++i) pos[i] = i;
      while (true) {
        int m = 0;
        for (int i = 0; i < k; ++i) m += 1 << pos[i];
        ninv[k][m] = (int)basis[k].size();
        basis[k].push_back(m);
        // advance: rightmost position that can move right
        int i = k - 1;
        while (i >= 0 && pos[i] >= n - k + i) --i;
        if (i < 0) break;
        pos[i] += 1;
        for (int j = i + 1; j < k; ++j) pos[j] = pos[j - 1] + 1;
      }
    }
  }
};

// NSymmetry rank used by SpinResolvedStorage::fill_spin: index = C(N,k) - num(b,N,k) - 1, with
// num the recursion of include/edlib/NSymmetry.h:155-162 written as a loop.
int nsym_index(const Binomial &C, int N, int k, state_t b) {
  int res = 0, n = N, m = k;
  while ((n - 1) > 0 && m > 0 && m < n) {
    if ((b & (1ll << (N - n))) == 0) {
      n -= 1;
    } else {
      res += (int)C(n - 1, m);
      n -= 1;
      m -= 1;
    }
  }
  return (int)C(N, k) - res - 1;
}

inline int occ(state_t s, int im, int ip) { return (int)((s >> (ip - 1 - im)) & 1); }
// number of occupied spin-orbitals with index < im, i.e. bits above position ip-1-im
inline int parity_above(state_t s, int im, int ip) {
  int cnt = __builtin_popcountll((unsigned long long)s >> (ip - im));
  return (cnt & 1) ? -1 : 1;
}

// ---------------------------------------------------------------- transitions
// A hopping transition c+_b c_a (valid if a occupied and b empty in the ORIGINAL state,
// include/edlib/HubbardModel.h:86-88, SingleImpurityAndersonModel.h:74-76) or a Coulomb
// transition c+_i s c+_j s' c_l s' c_k s (sequential validity, SingleImpurityAndersonModel.h:129-142).
struct Transition {
  int quad = 0;
  int a = 0, b = 0;            // hop: annihilate a, create b (spin-orbital indices)
  int k = 0, l = 0, j = 0, i = 0;  // quad: annihilate k, annihilate l, create j, create i
  double value = 0;            // value() of the reference transition object
  int sign_factor = 1;         // Hubbard hop: -1 ("-t c+ c"), SIAM hop and quad: +1
};

struct Model {
  int kind = 0;  // 0 = Hubbard, 1 = single-impurity Anderson
  int ns = 0, ip = 0, ml = 0;
  // Hubbard data (include/edlib/HubbardModel.h:48-77)
  std::vector<double> t, U, xmu, hmag, J;
  // SIAM data (include/edlib/SingleImpurityAndersonModel.h:195-275)
  std::vector<double> epsk, vk, h0, Utens;
  double mu = 0;
  std::vector<Transition> T, V;
  Binomial C{1};
  SpinBasis sb;

  double Ut(int s1, int s2, int i, int j, int k, int l) const {
    size_t m = ml;
    return Utens[((((size_t(s1) * 2 + s2) * m + i) * m + j) * m + k) * m + l];
  }

  int valid(const Transition &tr, state_t nst) const {
    if (!tr.quad) return occ(nst, tr.a, ip) * (1 - occ(nst, tr.b, ip));
    if (occ(nst, tr.k, ip) != 0) {
      state_t k3 = nst - (1ll << (ip - 1 - tr.k));
      if (occ(k3, tr.l, ip) != 0) {
        state_t k4 = k3 - (1ll << (ip - 1 - tr.l));
        if (occ(k4, tr.j, ip) == 0) {
          state_t k2 = k4 | (1ll << (ip - 1 - tr.j));
          return 1 - occ(k2, tr.i, ip);
        }
      }
    }
    return 0;
  }

  // new state and sign (HubbardModel.h:99-108, SingleImpurityAndersonModel.h:77-84, 153-162)
  void apply(const Transition &tr, state_t nst, state_t &out, int &sign) const {
    if (!tr.quad) {
      int s1 = parity_above(nst, tr.a, ip);
      state_t k1 = nst - (1ll << (ip - 1 - tr.a));
      int s2 = parity_above(k1, tr.b, ip);
      out = k1 + (1ll << (ip - 1 - tr.b));
      sign = tr.sign_factor * s1 * s2;
    } else {
      int s1 = parity_above(nst, tr.k, ip);
      state_t k3 = nst - (1ll << (ip - 1 - tr.k));
      int s2 = parity_above(k3, tr.l, ip);
      state_t k4 = k3 - (1ll << (ip - 1 - tr.l));
      int s3 = parity_above(k4, tr.j, ip);
      state_t k2 = k4 + (1ll << (ip - 1 - tr.j));
      int s4 = parity_above(k2, tr.i, ip);
      out = k2 + (1ll << (ip - 1 - tr.i));
      sign = s1 * s2 * s3 * s4;
    }
  }

  // <s|H|s>: HubbardModel.h:116-132 and SingleImpurityAndersonModel.h:282-306, same loop order
  double diagonal(state_t st) const {
    double x = 0.0;
    if (kind == 0) {
      for (int im = 0; im < ns; ++im) {
        for (int is = 0; is < 2; ++is) x += (0.0 - xmu[is]) * occ(st, im + is * ns, ip);
        x += U[im] * occ(st, im, ip) * occ(st, im + ns, ip);
        x += hmag[im] * (occ(st, im + ns, ip) - occ(st, im, ip));
        for (int im2 = 0; im2 < ns; ++im2)
          x += J[size_t(im) * ns + im2] * (occ(st, im, ip) - occ(st, im + ns, ip)) *
               (occ(st, im2, ip) - occ(st, im2 + ns, ip));
      }
    } else {
      int nk = ns - ml;
      for (int is = 0; is < 2; ++is)
        for (int ik = 0; ik < nk; ++ik) x += (epsk[size_t(ik) * 2 + is] * occ(st, ik + ml + is * ns, ip));
      for (int im = 0; im < ml; ++im) {
        for (int is = 0; is < 2; ++is) x += (h0[(size_t(im) * ml + im) * 2 + is] - mu) * occ(st, im + is * ns, ip);
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

  int interacting_orbitals() const { return kind == 0 ? ns : ml; }

  // SzSymmetry::state_by_index / index (SzSymmetry.h:114-133)
  state_t state_by_index(int nup, int ndn, long long ind) const {
    long long cd = C(ns, ndn);
    long long u = ind / cd, d = ind % cd;
    state_t r = sb.basis[nup][u];
    r <<= ns;
    r += sb.basis[ndn][d];
    return r;
  }
  long long index(state_t st, int nup, int ndn) const {
    state_t up = st >> ns, dn = st & ((1ll << ns) - 1);
    return (long long)sb.ninv[nup][(int)up] * C(ns, ndn) + sb.ninv[ndn][(int)dn];
  }
};

// ---------------------------------------------------------------- growable CSR used by SRS
// include/edlib/CRSMatrix.h:30-98 (including the element-skipping behaviour of compress)
struct GrowCSR {
  std::vector<double> val;
  std::vector<int> col, rp;
  int vind = 0;
  void init(size_t n) { val.clear(); col.clear(); rp.assign(n + 1, 0); vind = 0; }
  void add(int i, int j, double t, int sign) {
    if (std::abs(t) == 0) return;
    bool has = false;
    size_t found = 0;
    for (int q = rp[i]; q < vind; ++q)
      if (col[q] == j) { has = true; found = q; }
    if (has) {
      val[found] += sign * t;
    } else {
      col.push_back(j);
      val.push_back(sign * t);
      ++vind;
    }
  }
  void end_line(int i) {
    for (int q = rp[i]; q < vind; ++q) {
      if (std::abs(val[q]) < 1e-15) {
        for (int r = q; r < vind - 1; ++r) { val[r] = val[r + 1]; col[r] = col[r + 1]; }
        --vind;
        val.pop_back();
        col.pop_back();
      }
    }
    rp[i + 1] = vind;
  }
};

enum { ST_CRS = 0, ST_SRS = 1, ST_SOCRS = 2 };

struct Oracle {
  Model m;
  int storage = ST_CRS;
  int nup = 0, ndn = 0;
  long long dim = 0;
  // CRS (include/edlib/CRSStorage.h:66-83, 169-205)
  std::vector<double> crs_val;
  std::vector<int> crs_col, crs_rp;
  // SRS (include/edlib/SpinResolvedStorage.h:120-155, 622-638)
  GrowCSR hup, hdn, hloc;
  std::vector<double> sdiag;
  long long int_start = 0;
  int up_size = 0, dn_size = 0;
  // SOCRS (include/edlib/SOCRSStorage.h:114-160, 295-326)
  std::vector<double> dvalues;
  std::vector<int> so_col;
  std::vector<int8_t> so_sign;
  std::vector<long long> so_rowstart;
  std::string err;
};

void fill_crs(Oracle &o) {
  Model &m = o.m;
  long long n = o.dim;
  o.crs_rp.assign(n + 1, 0);
  o.crs_val.clear();
  o.crs_col.clear();
  size_t vind = 0;
  auto add = [&](long long i, long long j, double t, int sign) {
    bool has = false;
    size_t found = 0;
    for (size_t q = o.crs_rp[i]; q < vind; ++q)
      if (o.crs_col[q] == j) { has = true; found = q; }
    if (has) {
      o.crs_val[found] += sign * t;
    } else {
      o.crs_col.push_back((int)j);
      o.crs_val.push_back(sign * t);
      ++vind;
    }
  };
  for (long long i = 0; i < n; ++i) {
    state_t nst = m.state_by_index(o.nup, o.ndn, i);
    o.crs_rp[i] = (int)vind;
    o.crs_col.push_back((int)i);
    o.crs_val.push_back(m.diagonal(nst));
    ++vind;
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<Transition> &L = pass == 0 ? m.T : m.V;
      for (const Transition &tr : L) {
        if (m.valid(tr, nst)) {
          state_t k;
          int sign;
          m.apply(tr, nst, k, sign);
          add(i, m.index(k, o.nup, o.ndn), tr.value, sign);
        }
      }
    }
  }
  o.crs_rp[n] = (int)vind;
}

void fill_spin(Oracle &o, int nspin, int shift, GrowCSR &mat) {
  Model &m = o.m;
  const std::vector<int> &B = m.sb.basis[nspin];
  mat.init(B.size());
  for (size_t i = 0; i < B.size(); ++i) {
    state_t nst = B[i];
    for (const Transition &tr : m.T) {
      if (m.valid(tr, nst << shift)) {
        state_t k;
        int sign;
        m.apply(tr, nst << shift, k, sign);
        int j = nsym_index(m.C, m.ns, nspin, k >> shift);
        mat.add((int)i, j, tr.value, sign);
      }
    }
    mat.end_line((int)i);
  }
}

void fill_srs(Oracle &o) {
  Model &m = o.m;
  o.up_size = (int)m.C(m.ns, o.nup);
  o.dn_size = (int)m.C(m.ns, o.ndn);
  fill_spin(o, o.nup, m.ns, o.hup);
  fill_spin(o, o.ndn, 0, o.hdn);
  o.sdiag.assign(o.dim, 0.0);
  o.int_start = o.dim;
  if (!m.V.empty()) o.hloc.init(o.dim);
  for (long long i = 0; i < o.dim; ++i) {
    state_t nst = m.state_by_index(o.nup, o.ndn, i);
    o.sdiag[i] = m.diagonal(nst);
    if (!m.V.empty()) {
      for (const Transition &tr : m.V) {
        if (m.valid(tr, nst)) {
          o.int_start = std::min(i, o.int_start);
          state_t k;
          int sign;
          m.apply(tr, nst, k, sign);
          o.hloc.add((int)i, (int)m.index(k, o.nup, o.ndn), tr.value, sign);
        }
      }
      o.hloc.end_line((int)i);
    }
  }
}

void fill_socrs(Oracle &o) {
  Model &m = o.m;
  long long n = o.dim;
  o.dvalues.assign(n, 0.0);
  o.so_col.clear();
  o.so_sign.clear();
  o.so_rowstart.assign(n + 1, 0);
  for (long long i = 0; i < n; ++i) {
    state_t nst = m.state_by_index(o.nup, o.ndn, i);
    o.dvalues[i] = m.diagonal(nst);
    o.so_rowstart[i] = (long long)o.so_col.size();
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<Transition> &L = pass == 0 ? m.T : m.V;
      for (const Transition &tr : L) {
        if (m.valid(tr, nst)) {
          state_t k;
          int sign;
          m.apply(tr, nst, k, sign);
          long long j = m.index(k, o.nup, o.ndn);
          if (j == i) throw std::logic_error("Attempt to use addElement() to add diagonal element.");
          for (long long q = o.so_rowstart[i]; q < (long long)o.so_col.size(); ++q)
            if (o.so_col[q] == j) throw std::logic_error("Collision. Check a, adag, numState, ninv_value!");
          o.so_col.push_back((int)j);
          o.so_sign.push_back(sign < 0 ? 1 : 0);
        }
      }
    }
  }
  o.so_rowstart[n] = (long long)o.so_col.size();
}

// w = H v (clear) or w += H v, in the reference's accumulation order.
void av(Oracle &o, const double *v, double *w, bool clear) {
  long long n = o.dim;
  if (o.storage == ST_CRS) {  // CRSStorage.h:57-64
    for (long long i = 0; i < n; ++i) {
      w[i] = clear ? 0.0 : w[i];
      for (int j = o.crs_rp[i]; j < o.crs_rp[i + 1]; ++j) w[i] = w[i] + o.crs_val[j] * v[o.crs_col[j]];
    }
  } else if (o.storage == ST_SRS) {  // SpinResolvedStorage.h:58-115
    for (long long i = 0; i < n; ++i) w[i] = o.sdiag[i] * v[i] + (clear ? 0.0 : w[i]);
    const long long D = o.dn_size;
    for (long long k = 0; k < o.up_size; ++k)
      for (int i = 0; i < o.dn_size; ++i)
        for (int j = o.hdn.rp[i]; j < o.hdn.rp[i + 1]; ++j) w[i + k * D] += o.hdn.val[j] * v[o.hdn.col[j] + k * D];
    for (int i = 0; i < o.up_size; ++i)
      for (int j = o.hup.rp[i]; j < o.hup.rp[i + 1]; ++j)
        for (long long k = 0; k < D; ++k) w[i * D + k] += o.hup.val[j] * v[o.hup.col[j] * D + k];
    if (!o.m.V.empty())
      for (long long i = o.int_start; i < n; ++i)
        for (int j = o.hloc.rp[i]; j < o.hloc.rp[i + 1]; ++j) w[i] += o.hloc.val[j] * v[o.hloc.col[j]];
  } else {  // SOCRSStorage.h:46-87: every transition re-tested per row; OpenMP over rows
    const Model &m = o.m;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      state_t nst = m.state_by_index(o.nup, o.ndn, i);
      double acc = o.dvalues[i] * v[i] + (clear ? 0.0 : w[i]);
      long long q = o.so_rowstart[i];
      for (int pass = 0; pass < 2; ++pass) {
        const std::vector<Transition> &L = pass == 0 ? m.T : m.V;
        for (const Transition &tr : L) {
          int test = m.valid(tr, nst);
          if (test) {
            acc += test * tr.value * (1 - 2 * (o.so_sign[q] & 1)) * v[o.so_col[q]];
            ++q;
          }
        }
      }
      w[i] = acc;
    }
  }
}

}  // namespace

// ====================================================================== C API
extern "C" {

void *eo_create_hubbard(int ns, const double *t, const double *U, const double *xmu, const double *hmag,
                        const double *J) {
  Oracle *o = new Oracle();
  Model &m = o->m;
  m.kind = 0;
  m.ns = ns;
  m.ip = 2 * ns;
  m.t.assign(t, t + size_t(ns) * ns);
  m.U.assign(U, U + ns);
  m.xmu.assign(xmu, xmu + ns);
  m.hmag.assign(hmag, hmag + ns);
  m.J.assign(J, J + size_t(ns) * ns);
  // HubbardModel.h:68-76
  for (int ii = 0; ii < ns; ++ii)
    for (int jj = 0; jj < ns; ++jj)
      if (std::abs(m.t[size_t(ii) * ns + jj]) > 1e-10)
        for (int is = 0; is < 2; ++is) {
          Transition tr;
          tr.a = ii + is * ns;
          tr.b = jj + is * ns;
          tr.value = m.t[size_t(ii) * ns + jj];
          tr.sign_factor = -1;
          m.T.push_back(tr);
        }
  m.C = Binomial(ns);
  m.sb.build(ns);
  return o;
}

// epsk[(ns-ml)][2], vk[ml][ns-ml][2], h0[ml][ml][2], U[2][2][ml][ml][ml][ml]
void *eo_create_siam(int ns, int ml, const double *epsk, const double *vk, const double *h0, double mu,
                     const double *U) {
  Oracle *o = new Oracle();
  Model &m = o->m;
  m.kind = 1;
  m.ns = ns;
  m.ml = ml;
  m.ip = 2 * ns;
  int nk = ns - ml;
  m.epsk.assign(epsk, epsk + size_t(nk) * 2);
  m.vk.assign(vk, vk + size_t(ml) * nk * 2);
  m.h0.assign(h0, h0 + size_t(ml) * ml * 2);
  m.mu = mu;
  size_t m4 = size_t(ml) * ml * ml * ml;
  m.Utens.assign(U, U + 4 * m4);
  auto hop = [&](int i, int j, int s, double v) {
    Transition tr;
    tr.a = i + s * ns;
    tr.b = j + s * ns;
    tr.value = v;
    tr.sign_factor = 1;
    m.T.push_back(tr);
  };
  // SingleImpurityAndersonModel.h:232-254
  for (int im = 0; im < ml; ++im)
    for (int jm = 0; jm < im; ++jm)
      for (int is = 0; is < 2; ++is) {
        double h = m.h0[(size_t(im) * ml + jm) * 2 + is];
        if (std::abs(h) > 1e-10) { hop(im, jm, is, h); hop(jm, im, is, h); }
      }
  for (int im = 0; im < ml; ++im)
    for (int ik = 0; ik < nk; ++ik)
      for (int is = 0; is < 2; ++is) {
        double v = m.vk[(size_t(im) * nk + ik) * 2 + is];
        if (std::abs(v) > 1e-10) { hop(im, ik + ml, is, v); hop(ik + ml, im, is, v); }
      }
  // SingleImpurityAndersonModel.h:256-274
  for (int s1 = 0; s1 < 2; ++s1)
    for (int s2 = 0; s2 < 2; ++s2)
      for (int i = 0; i < ml; ++i)
        for (int j = 0; j < ml; ++j)
          for (int k = 0; k < ml; ++k)
            for (int l = 0; l < ml; ++l) {
              if (((i == l) && (j == k) && (s1 == s2)) || ((i == k) && (j == l))) continue;
              double u = m.Ut(s1, s2, i, j, k, l);
              if (std::abs(u) != 0.0) {
                Transition tr;
                tr.quad = 1;
                tr.k = k + s1 * ns;
                tr.l = l + s2 * ns;
                tr.j = j + s2 * ns;
                tr.i = i + s1 * ns;
                tr.value = 0.5 * u;
                m.V.push_back(tr);
              }
            }
  m.C = Binomial(ns);
  m.sb.build(ns);
  return o;
}

void eo_destroy(void *h) { delete (Oracle *)h; }

int eo_num_transitions(void *h, int which) {
  Oracle *o = (Oracle *)h;
  return which == 0 ? (int)o->m.T.size() : (int)o->m.V.size();
}

long long eo_binom(void *h, int n, int k) { return ((Oracle *)h)->m.C(n, k); }

// Sector list in the reference's iteration order: the same comparator and std::sort as
// include/edlib/SzSymmetry.h:51-54, 72-98.  in_list == nullptr means all (N_up, N_dn).
int eo_sector_order(void *h, const int *in_list, int n_in, int *out) {
  Oracle *o = (Oracle *)h;
  int ns = o->m.ns;
  struct Sec { int up, dn; size_t size; };
  std::vector<Sec> s;
  if (in_list) {
    for (int i = 0; i < n_in; ++i)
      s.push_back({in_list[2 * i], in_list[2 * i + 1], size_t(o->m.C(ns, in_list[2 * i]) * o->m.C(ns, in_list[2 * i + 1]))});
  } else {
    for (int i = 0; i <= ns; ++i)
      for (int j = 0; j <= ns; ++j) s.push_back({i, j, size_t(o->m.C(ns, i) * o->m.C(ns, j))});
  }
  std::sort(s.begin(), s.end(), [](const Sec &a, const Sec &b) {
    return a.size < b.size || (a.size == b.size && a.up < b.up && a.dn < b.dn) ||
           (a.size == b.size && a.up == b.up && a.dn < b.dn);
  });
  for (size_t i = 0; i < s.size(); ++i) { out[2 * i] = s[i].up; out[2 * i + 1] = s[i].dn; }
  return (int)s.size();
}

int eo_basis(void *h, int k, int *out) {
  Oracle *o = (Oracle *)h;
  const std::vector<int> &B = o->m.sb.basis[k];
  std::copy(B.begin(), B.end(), out);
  return (int)B.size();
}

int eo_nsym_index(void *h, int k, long long st) { Oracle *o = (Oracle *)h; return nsym_index(o->m.C, o->m.ns, k, st); }

long long eo_state_by_index(void *h, int nup, int ndn, long long i) { return ((Oracle *)h)->m.state_by_index(nup, ndn, i); }

double eo_diagonal(void *h, long long st) { return ((Oracle *)h)->m.diagonal(st); }

// Fills the storage for sector (nup, ndn); returns the dimension, or -1 with eo_error() set.
long long eo_fill(void *h, int storage, int nup, int ndn) {
  Oracle *o = (Oracle *)h;
  o->storage = storage;
  o->nup = nup;
  o->ndn = ndn;
  o->dim = o->m.C(o->m.ns, nup) * o->m.C(o->m.ns, ndn);
  try {
    if (storage == ST_CRS) fill_crs(*o);
    else if (storage == ST_SRS) fill_srs(*o);
    else fill_socrs(*o);
  } catch (std::exception &e) {
    o->err = e.what();
    return -1;
  }
  return o->dim;
}

const char *eo_error(void *h) { return ((Oracle *)h)->err.c_str(); }

void eo_av(void *h, const double *v, double *w, int clear) { av(*(Oracle *)h, v, w, clear != 0); }

// Per-spin CSR of the current SRS fill (which = 0: H_up, 1: H_dn, 2: H_loc).  Returns nnz;
// with null outputs only the sizes are reported.
long long eo_srs_csr(void *h, int which, int *rp, int *col, double *val, int *nrows) {
  Oracle *o = (Oracle *)h;
  GrowCSR &g = which == 0 ? o->hup : which == 1 ? o->hdn : o->hloc;
  *nrows = (int)g.rp.size() - 1;
  if (rp) {
    std::copy(g.rp.begin(), g.rp.end(), rp);
    std::copy(g.col.begin(), g.col.begin() + g.vind, col);
    std::copy(g.val.begin(), g.val.begin() + g.vind, val);
  }
  return g.vind;
}

double eo_zero_eigenpair(void *h) {
  Oracle *o = (Oracle *)h;
  if (o->storage == ST_CRS) return o->crs_val[0];
  if (o->storage == ST_SRS) return o->sdiag[0];
  return o->dvalues[0];
}

// a_adag for a vector of sector (nup, ndn) into the target sector: out[index(k)] = sign*in[i]
// (CRSStorage.h:131-145, SpinResolvedStorage.h:293-381, SOCRSStorage.h:228-242).
// out must be zero on entry and sized for the target sector.
void eo_a_adag(void *h, int im, int nup, int ndn, int tnup, int tndn, const double *in, double *out, int annihilate) {
  Oracle *o = (Oracle *)h;
  const Model &m = o->m;
  long long n = m.C(m.ns, nup) * m.C(m.ns, ndn);
  for (long long i = 0; i < n; ++i) {
    state_t nst = m.state_by_index(nup, ndn, i);
    if (occ(nst, im, m.ip) == (annihilate ? 1 : 0)) {
      int sign = parity_above(nst, im, m.ip);
      state_t k = annihilate ? nst - (1ll << (m.ip - im - 1)) : nst + (1ll << (m.ip - im - 1));
      long long i1 = m.index(k, tnup, tndn);
      out[i1] = sign * in[i];
    }
  }
}

// ChiLoc operation (ChiLoc.h:474-530): out[i] = (O_mu [+ O_nu])(state_i) * in[i]; op 0 = Sz, 1 = N.
void eo_diag_op(void *h, int op, int mu, int nu, int nup, int ndn, const double *in, double *out) {
  Oracle *o = (Oracle *)h;
  const Model &m = o->m;
  long long n = m.C(m.ns, nup) * m.C(m.ns, ndn);
  auto act = [&](state_t s, int iii) -> double {
    if (op == 0) return 0.5 * (occ(s, iii, m.ip) - occ(s, iii + m.ns, m.ip));
    return (occ(s, iii, m.ip) + occ(s, iii + m.ns, m.ip));
  };
  for (long long i = 0; i < n; ++i) {
    state_t s = m.state_by_index(nup, ndn, i);
    out[i] = (nu < 0 ? act(s, mu) : act(s, mu) + act(s, nu)) * in[i];
  }
}

// Lanczos recurrence of include/edlib/Lanczos.h:36-77 on the current fill.  v is the
// normalised start vector (overwritten).  alpha[nlanc_max], beta[nlanc_max+1] (beta[0]
// untouched).  Returns the number of iterations.
int eo_lanczos(void *h, double *v, int nlanc_max, double *alpha, double *beta) {
  Oracle *o = (Oracle *)h;
  long long size = o->dim;
  std::vector<double> w(size, 0.0);
  double alf = 0, bet = 0;
  int nlanc = 0;
  if (size == 0) return 0;
  for (int iter = 1; iter <= nlanc_max; ++iter) {
    ++nlanc;
    if (iter != 1) {
      for (long long j = 0; j < size; ++j) {
        double dummy = v[j];
        v[j] = w[j] / bet;
        w[j] = -bet * dummy;
      }
    }
    av(*o, v, w.data(), false);
    alf = 0.0;
    for (long long k = 0; k < size; ++k) alf += w[k] * v[k];
    alpha[iter - 1] = alf;
    for (long long j = 0; j < size; ++j) w[j] -= alf * v[j];
    bet = 0.0;
    for (long long k = 0; k < size; ++k) bet += w[k] * w[k];
    bet = std::sqrt(bet);
    if (iter != nlanc_max) beta[iter] = bet;
    if (std::abs(bet) < 1e-10) break;
  }
  return nlanc;
}

// get_frac_point (Lanczos.h:201-224) for nz complex energies `ener` (re, im pairs).
void eo_frac_points(const double *alpha, const double *beta, int nlanc, int isign, double expectation, double expb,
                    const double *ener, int nz, double *out) {
  std::vector<std::complex<double>> det(nlanc), dl(nlanc);
  for (int p = 0; p < nz; ++p) {
    std::complex<double> e(ener[2 * p], ener[2 * p + 1]);
    std::complex<double> swp = 0.0;
    std::fill(det.begin(), det.end(), std::complex<double>(0.0));
    for (int i = 0; i < nlanc; ++i) dl[i] = e - ((double)(alpha[i]) * isign);
    if (nlanc == 1) {
      det[0] = dl[0];
      swp += expectation * expb / det[0];
    } else {
      det[nlanc - 1] = dl[nlanc - 1];
      det[nlanc - 2] = dl[nlanc - 2] * dl[nlanc - 1] - std::pow(beta[nlanc - 1], 2);
      for (int i = nlanc - 3; i >= 0; --i) {
        det[i] = (dl[i] * det[i + 1] - std::pow(beta[i + 1], 2) * det[i + 2]);
        if (std::abs(det[i]) > (std::numeric_limits<float>::max() / 2.0) && i != 0) {
          double shift = 1.0 / (std::numeric_limits<float>::max() / 1000.0);
          det[i] *= shift;
          det[i + 1] *= shift;
        }
      }
      swp += expectation * expb * det[1] / det[0];
    }
    out[2 * p] = swp.real();
    out[2 * p + 1] = swp.imag();
  }
}

}  // extern "C"
