/* Plain C client of the C ABI (C99, include/edgpu.h, libedgpu.so): the reference's Lanczos test workflow
 * (test/Lanczos_Test.cpp of the reference) driven from C -- read a Hubbard cluster from a model input in the
 * text exchange format (lines "param KEY VALUE" and "data PATH NDIM DIMS... VALUES..."), Hamiltonian::diag
 * with CRSStorage in FP64, GreensFunction::compute and both ChiLoc susceptibilities, printed one value per line:
 *   E <index> <eigenvalue>           every eigen-pair, ascending
 *   G <w> <re> <im>                  G(i w_n) of orbital 0, spin up
 *   CHISZ <w> <re> / CHIN <w> <re>   chi_Sz and chi_N of orbital 0 (operator averages from StaticObservables)
 * Without a device it prints "no device" and exits 0. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "edgpu.h"

#define MAXN 16

static double t_[MAXN * MAXN], U_[MAXN], mu_[MAXN];
static int orbs_[2 * MAXN * MAXN], norbs_ = 0;

static int read_input(const char *path, int *ns, int *nev, double *beta, int *nomega) {
  FILE *f = fopen(path, "r");
  char tok[256], key[256];
  if (!f) return -1;
  while (fscanf(f, "%255s", tok) == 1) {
    if (strcmp(tok, "param") == 0) {
      char val[256];
      if (fscanf(f, "%255s %255s", key, val) != 2) break;
      if (strcmp(key, "NSITES") == 0) *ns = atoi(val);
      else if (strcmp(key, "arpack.NEV") == 0) *nev = atoi(val);
      else if (strcmp(key, "lanc.BETA") == 0) *beta = atof(val);
      else if (strcmp(key, "lanc.NOMEGA") == 0) *nomega = atoi(val);
    } else if (strcmp(tok, "data") == 0) {
      int nd = 0, n = 1, d, i;
      if (fscanf(f, "%255s %d", key, &nd) != 2) break;
      for (i = 0; i < nd; ++i) {
        if (fscanf(f, "%d", &d) != 1) return -1;
        n *= d;
      }
      for (i = 0; i < n; ++i) {
        double x;
        if (fscanf(f, "%lf", &x) != 1) return -1;
        if (strcmp(key, "hopping/values") == 0 && i < MAXN * MAXN) t_[i] = x;
        else if (strcmp(key, "interaction/values") == 0 && i < MAXN) U_[i] = x;
        else if (strcmp(key, "chemical_potential/values") == 0 && i < MAXN) mu_[i] = x;
        else if (strcmp(key, "GreensFunction_orbitals/values") == 0 && i < 2 * MAXN * MAXN) {
          orbs_[i] = (int)x;
          norbs_ = (i + 1) / 2;
        }
      }
    }
  }
  fclose(f);
  return 0;
}

int main(int argc, char **argv) {
  int ns = 0, nev = 2, nomega = 32, npairs = 0, i, rc;
  double beta = 10.0, Z = 0.0;
  edgpu_ctx *ctx = NULL;
  edgpu_model *m = NULL;
  if (argc < 2 || read_input(argv[1], &ns, &nev, &beta, &nomega) != 0 || ns < 1 || ns > MAXN) {
    fprintf(stderr, "usage: abi_c_client <model input>\n");
    return 2;
  }
  rc = edgpu_ctx_create(&ctx, 0, 0);
  if (rc != EDGPU_OK) {
    printf("no device\n");
    return 0;
  }
  rc = edgpu_model_hubbard(ctx, ns, t_, U_, mu_, NULL, NULL, &m);
  if (rc != EDGPU_OK) {
    fprintf(stderr, "model: %s\n", edgpu_last_error(ctx));
    return 1;
  }
  {
    edgpu_diag_params p;
    memset(&p, 0, sizeof(p));
    p.storage = EDGPU_CRS;
    p.precision = EDGPU_FP64;
    p.nev = nev;
    rc = edgpu_diag(m, &p, &npairs);
    if (rc < 0) {
      fprintf(stderr, "diag: %s\n", edgpu_last_error(ctx));
      return 1;
    }
  }
  {
    double *e = (double *)malloc(sizeof(double) * (npairs > 0 ? npairs : 1));
    edgpu_eigenpairs(m, e, NULL, NULL, npairs);
    for (i = 0; i < npairs; ++i) printf("E %d %.17g\n", i, e[i]);
    free(e);
  }
  {
    edgpu_gf_params g;
    const int nint = ns;
    double *G = (double *)calloc((size_t)nomega * nint * 2 * 2, sizeof(double));
    double *chi = (double *)calloc((size_t)nomega * nint * 2, sizeof(double));
    memset(&g, 0, sizeof(g));
    g.beta = beta;
    g.nomega = nomega;
    g.nlanc = 100;
    g.cutoff = 1e-12;
    g.precision = EDGPU_FP64;
    g.orbitals = norbs_ ? orbs_ : NULL;
    g.n_orbitals = norbs_;
    g.mesh = EDGPU_MESH_MATSUBARA;
    rc = edgpu_greens_function(m, &g, G, NULL, &Z);
    if (rc < 0) {
      fprintf(stderr, "gf: %s\n", edgpu_last_error(ctx));
      return 1;
    }
    for (i = 0; i < nomega; ++i) printf("G %d %.17g %.17g\n", i, G[((size_t)i * nint) * 4], G[((size_t)i * nint) * 4 + 1]);
    /* ChiLoc with the operator averages from StaticObservables, as the reference's drivers take them:
     * sum_i M_i / (2 n) and sum_i N_i / n */
    double nn[MAXN], mm[MAXN], avg_m = 0.0, avg_n = 0.0;
    rc = edgpu_static_observables(m, beta, 1e-12, nn, NULL, NULL, mm, NULL, NULL, NULL, NULL);
    if (rc < 0) {
      fprintf(stderr, "observables: %s\n", edgpu_last_error(ctx));
      return 1;
    }
    for (i = 0; i < nint; ++i) {
      avg_m += mm[i] / (2.0 * nint);
      avg_n += nn[i] / nint;
    }
    rc = edgpu_chiloc(m, &g, EDGPU_OP_SZ, avg_m, chi, NULL, &Z);
    if (rc < 0) {
      fprintf(stderr, "chi: %s\n", edgpu_last_error(ctx));
      return 1;
    }
    for (i = 0; i < nomega; ++i) printf("CHISZ %d %.17g\n", i, chi[((size_t)i * nint) * 2]);
    rc = edgpu_chiloc(m, &g, EDGPU_OP_N, avg_n, chi, NULL, &Z);
    if (rc < 0) {
      fprintf(stderr, "chi: %s\n", edgpu_last_error(ctx));
      return 1;
    }
    for (i = 0; i < nomega; ++i) printf("CHIN %d %.17g\n", i, chi[((size_t)i * nint) * 2]);
    free(G);
    free(chi);
  }
  edgpu_model_destroy(m);
  edgpu_ctx_destroy(ctx);
  return 0;
}
