// FP64 stand-in for ARPACK's dsaupd_/dseupd_ reverse-communication pair, used only by the
// oracle harness that compiles the reference EDLib headers (ARPACK-ng is not installed here).
//
// Protocol followed (as EDLib's Storage::diag drives it, include/edlib/Storage.h:77-95):
//   dsaupd_ is called with ido = 0 first; it answers ido = 1 with x = workd[ipntr[0]-1 ...]
//   and expects y = OP x in workd[ipntr[1]-1 ...] on the next call.  The stand-in asks for
//   y = H e_j for every unit vector e_j, assembles the dense sector matrix, diagonalises it
//   with LAPACK dsyev (scipy's bundled OpenBLAS) and returns ido = 99.  dseupd_ then hands
//   back the nev smallest-algebraic eigenpairs in ascending order, as ARPACK's "SA" mode does.
// Exact multiplicities are kept, which is what ARPACK yields when ncv == n.
#include <cstring>
#include <stdexcept>
#include <vector>
#include <cstdio>

extern "C" void scipy_dsyev_(const char *jobz, const char *uplo, const int *n, double *a, const int *lda,
                             double *w, double *work, const int *lwork, int *info, size_t, size_t);

namespace {
struct DenseState {
  int n = 0;
  int col = 0;
  std::vector<double> h;      // column-major n x n
  std::vector<double> evals;  // ascending
};
DenseState g_state;
const int kDenseMax = 12000;
}  // namespace

extern "C" void dsaupd_(int *ido, char *, int *n, char *, int *nev, double *, double *, int *, double *,
                        int *, int *iparam, int *ipntr, double *workd, double *, int *, int *info) {
  const int N = *n;
  if (*ido == 0) {
    if (N > kDenseMax) { *info = -9999; *ido = 99; return; }
    g_state.n = N;
    g_state.col = 0;
    g_state.h.assign(size_t(N) * N, 0.0);
  } else {
    // y = H e_col has been written to workd[N .. 2N)
    std::memcpy(&g_state.h[size_t(g_state.col) * N], workd + N, sizeof(double) * N);
    g_state.col++;
  }
  if (g_state.col < N) {
    std::fill(workd, workd + N, 0.0);
    workd[g_state.col] = 1.0;
    ipntr[0] = 1;
    ipntr[1] = N + 1;
    *ido = 1;
    return;
  }
  // diagonalise
  g_state.evals.assign(N, 0.0);
  int lwork = -1, linfo = 0;
  double wq = 0;
  scipy_dsyev_("V", "L", &N, g_state.h.data(), &N, g_state.evals.data(), &wq, &lwork, &linfo, 1, 1);
  lwork = int(wq) + 1;
  std::vector<double> work(lwork);
  scipy_dsyev_("V", "L", &N, g_state.h.data(), &N, g_state.evals.data(), work.data(), &lwork, &linfo, 1, 1);
  if (linfo != 0) { *info = -9998; *ido = 99; return; }
  iparam[2] = 1;
  iparam[4] = *nev;
  iparam[8] = N;
  *info = 0;
  *ido = 99;
}

extern "C" void dseupd_(int *rvec, char *, int *, double *d, double *z, int *ldz, double *, char *, int *n,
                        char *, int *nev, double *, double *, int *, double *, int *, int *, int *, double *,
                        double *, int *, int *ierr) {
  const int N = *n;
  for (int k = 0; k < *nev; ++k) {
    d[k] = g_state.evals[k];
    if (*rvec) std::memcpy(z + size_t(k) * (*ldz), &g_state.h[size_t(k) * N], sizeof(double) * N);
  }
  *ierr = 0;
}

// single-precision entry points exist only so the reference's Storage<float> specialisations link
extern "C" void ssaupd_(int *ido, char *, int *, char *, int *, float *, float *, int *, float *, int *, int *,
                        int *, float *, float *, int *, int *info) { *info = -9999; *ido = 99; }
extern "C" void sseupd_(int *, char *, int *, float *, float *, int *, float *, char *, int *, char *, int *,
                        float *, float *, int *, float *, int *, int *, int *, float *, float *, int *,
                        int *ierr) { *ierr = -9999; }
