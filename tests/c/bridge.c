/* The drop-in sequence a C driver runs through include/ffv.h, as the reference's loop would
 * after the bridge is added (INTEGRATION.md sections 1-2): leaves -> ffv_mesh_build ->
 * ffv_create -> ffv_set_mesh, then per time step the state copied from the leaves (AoS, as
 * LEAF.S holds it) into the SoA staging buffer, ffv_upload_state, ffv_step(dt, 1),
 * ffv_download_state and the copy back.
 *
 * Usage: bridge <case.bin> <out.bin>
 *   case.bin: int32 ntrees[3], bc[6], steps, order, rk_steps; int64 n; double tree_edge, dt,
 *             gamma, pinf; int32 tree[3n], level[n], ijk[3n]; double S[n][5]
 *   out.bin:  double S[n][5] after `steps` steps
 * Exit status 0, or the ffv error code of the call that failed. */
#include <stdio.h>
#include <stdlib.h>

#include "ffv.h"

#define NEQ 5

static int rd(void *p, size_t sz, size_t cnt, FILE *f) { return fread(p, sz, cnt, f) == cnt; }

int main(int argc, char **argv) {
  if (argc != 3) return 100;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 101;
  int32_t head[12];
  int64_t n;
  double dd[4];
  if (!rd(head, 4, 12, f) || !rd(&n, 8, 1, f) || !rd(dd, 8, 4, f)) return 102;
  int32_t *tree = malloc(12 * n), *lev = malloc(4 * n), *ijk = malloc(12 * n);
  double *S = malloc(sizeof(double) * NEQ * n), *soa = malloc(sizeof(double) * NEQ * n);
  if (!tree || !lev || !ijk || !S || !soa) return 103;
  if (!rd(tree, 4, 3 * n, f) || !rd(lev, 4, n, f) || !rd(ijk, 4, 3 * n, f) ||
      !rd(S, 8, NEQ * n, f))
    return 104;
  fclose(f);

  ffv_forest_desc d;
  for (int a = 0; a < 3; a++) d.ntrees[a] = head[a];
  for (int s = 0; s < 6; s++) d.bc[s] = head[3 + s];
  d.tree_edge = dd[0];
  ffv_mesh *mesh = NULL;
  int64_t *order = malloc(sizeof(int64_t) * n);
  int rc = ffv_mesh_build(&d, n, tree, lev, ijk, &mesh, order);
  if (rc) return rc;
  for (int64_t i = 0; i < n; i++)
    if (order[i] != i) return 105; /* the reference's leaf order comes back unchanged */
  if (ffv_mesh_ncells(mesh) != n) return 106;

  ffv_params p = {0};
  p.model = 0;
  p.nmaterials = 1;
  p.order = head[10];
  p.rk_steps = head[11];
  p.precision = FFV_FP64;
  p.gamma[0] = dd[2];
  p.pinf[0] = dd[3];
  ffv_ctx *ctx = NULL;
  if ((rc = ffv_create(&ctx, &p, 0))) return rc;
  if ((rc = ffv_set_mesh(ctx, mesh))) return rc;
  for (int step = 0; step < head[9]; step++) {
    for (int64_t i = 0; i < n; i++)
      for (int v = 0; v < NEQ; v++) soa[v * n + i] = S[NEQ * i + v];
    if ((rc = ffv_upload_state(ctx, soa, n, NEQ))) return rc;
    if ((rc = ffv_step(ctx, dd[1], 1))) return rc;
    if ((rc = ffv_download_state(ctx, soa, n, NEQ))) return rc;
    for (int64_t i = 0; i < n; i++)
      for (int v = 0; v < NEQ; v++) S[NEQ * i + v] = soa[v * n + i];
  }
  ffv_destroy(ctx);
  ffv_mesh_free(mesh);

  f = fopen(argv[2], "wb");
  if (!f || fwrite(S, 8, NEQ * n, f) != (size_t)(NEQ * n)) return 107;
  fclose(f);
  free(tree);
  free(lev);
  free(ijk);
  free(S);
  free(soa);
  free(order);
  return 0;
}
