/* Plain C client of the C ABI: compiles as C99 against include/edgpu.h and links libedgpu.so. */
#include <stdio.h>
#include "edgpu.h"

int main(void) {
  edgpu_ctx *ctx = NULL;
  int rc = edgpu_ctx_create(&ctx, 0, 0);
  if (rc != EDGPU_OK) {
    printf("no device: %d\n", rc);
    return 0;
  }
  double t[4] = {0, 1, 1, 0}, U[2] = {4, 4}, mu[2] = {2, 2};
  edgpu_model *m = NULL;
  rc = edgpu_model_hubbard(ctx, 2, t, U, mu, NULL, NULL, &m);
  if (rc != EDGPU_OK) return 1;
  edgpu_diag_params p = {EDGPU_CRS, EDGPU_FP64, 2, 0, 0, 0.0, 0, NULL, 0};
  int npairs = 0;
  rc = edgpu_diag(m, &p, &npairs);
  double e[32];
  edgpu_eigenpairs(m, e, NULL, NULL, npairs < 32 ? npairs : 32);
  printf("pairs %d E0 %.12f\n", npairs, e[0]);
  edgpu_model_destroy(m);
  edgpu_ctx_destroy(ctx);
  return rc < 0;
}
