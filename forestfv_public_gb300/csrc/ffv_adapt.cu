// Mesh adaptation: one refineh pass of the reference (refineh.c:3-57) on the owner-sorted
// tables, with the state carried over on the device.
//
// Given each leaf's target level (ffv_tags), eight sibling leaves that all want a coarser
// level merge into their parent, whose state is sum_k S_k / 8 in child order
// (merge.c:35-45) followed, for model 5, by the pressure relaxation of the merged state
// (merge.c:52-57); a leaf that wants a finer level splits into its eight children, which
// copy its state (split.c:424-427); every other leaf is kept.  Merges and splits exclude
// each other (all eight below their level vs. above it), so one sweep in leaf order does
// both of the reference's loops.  The new leaves and tables come from ffv_mesh_adapt (the
// host rebuild around the changed leaves); the context then holds the new tables and the
// carried-over state.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ffv_device.cuh"
#include "ffv_m5.cuh"

namespace {

// new cell i takes old cell map[i] (>= 0) or the mean of old cells j..j+7 (map[i] = -1 - j)
__global__ void adapt_remap(int64_t n_new, int64_t n_old, int neq, const int64_t *__restrict__ map,
                            const double *__restrict__ Sold, double *__restrict__ Snew) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_new;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = map[i];
    for (int v = 0; v < neq; v++) {
      double x;
      if (src >= 0) {
        x = Sold[(int64_t)v * n_old + src];
      } else {
        const int64_t j = -1 - src;
        x = 0.0;
        for (int q = 0; q < 8; q++) x += Sold[(int64_t)v * n_old + j + q] / ((double)8);
      }
      Snew[(int64_t)v * n_new + i] = x;
    }
  }
}

}  // namespace

// defined in ffv_api.cu
int ffv_ctx_adapt_view(ffv_ctx *ctx, int *device, cudaStream_t *st, int64_t *n, int *neq,
                       double **d_S, int *model, const M5Consts **k);
extern "C" int ffv_set_mesh(ffv_ctx *c, const ffv_mesh *m);
extern "C" int ffv_mesh_adapt(const ffv_mesh *m, const int32_t *split, ffv_mesh **out,
                              int64_t *src);
extern "C" int ffv_adapt_changes(const ffv_mesh *m, const int32_t *split, int64_t *nsplit,
                                 int64_t *nmerge);
extern "C" void ffv_mesh_free(ffv_mesh *m);
int ffv_ctx_mark_state(ffv_ctx *ctx);
int ffv_ctx_scratch(ffv_ctx *c, double **d_SN, double **d_SF, int64_t *cap, int64_t *cap_nsub);

extern "C" int ffv_adapt_map(ffv_ctx *ctx, const ffv_mesh *m, const int32_t *split,
                             ffv_mesh **out, int64_t *src) {
  if (!ctx || !m || !split || !out) return FFV_ERR_ARG;
  *out = nullptr;
  int device, neq, model;
  cudaStream_t st;
  int64_t n;
  double *d_S;
  const M5Consts *k;
  int rc = ffv_ctx_adapt_view(ctx, &device, &st, &n, &neq, &d_S, &model, &k);
  if (rc != FFV_OK) return rc;
  if (n != m->n) return FFV_ERR_ARG;
  // the new leaves and their tables (host; rows of leaves the pass leaves alone are the old
  // ones renumbered), then the state carried over on the device
  ffv_mesh *nm = nullptr;
  std::vector<int64_t> own_map;
  int64_t *cmap = src;  // every new leaf's source: the caller's array, else one of our own
  int64_t nsplit = 0, nmerged = 0;  // leaves that split, merged parents
  rc = ffv_adapt_changes(m, split, &nsplit, &nmerged);
  if (rc != FFV_OK) return rc;
  if (!cmap) {
    own_map.resize(m->n + 7 * (nsplit - nmerged));
    cmap = own_map.data();
  }
  rc = ffv_mesh_adapt(m, split, &nm, cmap);
  if (rc != FFV_OK) return rc;
  const int64_t n_new = nm->n;
  // carry the state over on the device, then swap the tables.  When the new mesh fits the
  // context's buffers (ffv_set_mesh then keeps them), the new state is assembled in the RK
  // copy and the map in the face-state buffer, both idle between steps: the regrid allocates
  // nothing on the device.  Otherwise ffv_set_mesh reallocates every buffer, and the remap
  // uses buffers of its own.
  cudaError_t e = cudaSetDevice(device);
  double *d_SN = nullptr, *d_SF = nullptr;
  int64_t cap = 0, cap_nsub = 0;
  rc = ffv_ctx_scratch(ctx, &d_SN, &d_SF, &cap, &cap_nsub);
  if (rc != FFV_OK) {
    ffv_mesh_free(nm);
    return rc;
  }
  const bool fits = n_new <= cap && (nm->nsub > 0 ? nm->nsub : 1) <= cap_nsub;
  int64_t *d_map = fits ? reinterpret_cast<int64_t *>(d_SF) : nullptr;
  double *d_T = fits ? d_SN : nullptr;
  if (!fits && e == cudaSuccess) e = cudaMalloc(&d_map, sizeof(int64_t) * n_new);
  if (!fits && e == cudaSuccess) e = cudaMalloc(&d_T, sizeof(double) * neq * n_new);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_map, cmap, sizeof(int64_t) * n_new, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    adapt_remap<<<152 * 4, 256, 0, st>>>(n_new, n, neq, d_map, d_S, d_T);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && model == 5 && nmerged > 0) {
    ffv_m5_relax_merged(n_new, *k, d_map, d_T, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  rc = e == cudaSuccess ? FFV_OK : FFV_ERR_CUDA;
  if (rc == FFV_OK) rc = ffv_set_mesh(ctx, nm);  // new tables and buffers; state unset
  if (rc == FFV_OK) {
    ffv_ctx_mark_state(ctx);
    double *d_Snew = nullptr;
    int64_t n2 = 0;
    rc = ffv_ctx_adapt_view(ctx, &device, &st, &n2, &neq, &d_Snew, &model, &k);
    if (rc == FFV_OK && (n2 != n_new || !d_Snew)) rc = FFV_ERR_STATE;
    if (rc == FFV_OK) {
      e = cudaMemcpyAsync(d_Snew, d_T, sizeof(double) * neq * n_new, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = FFV_ERR_CUDA;
    }
  }
  if (!fits) {
    cudaFree(d_map);
    cudaFree(d_T);
  }
  if (rc != FFV_OK) {
    ffv_mesh_free(nm);
    return rc;
  }
  *out = nm;
  return FFV_OK;
}

extern "C" int ffv_adapt(ffv_ctx *ctx, const ffv_mesh *m, const int32_t *split, ffv_mesh **out) {
  return ffv_adapt_map(ctx, m, split, out, nullptr);
}

// the leaves of a mesh in its cell order (the inverse of ffv_mesh_build's input); any of the
// three outputs may be null
extern "C" int ffv_mesh_leaves(const ffv_mesh *m, int32_t *tree_ijk, int32_t *level,
                               int32_t *cell_ijk) {
  if (!m || (!tree_ijk && !level && !cell_ijk)) return FFV_ERR_ARG;
  if (tree_ijk) memcpy(tree_ijk, m->tree_ijk, sizeof(int32_t) * 3 * m->n);
  if (cell_ijk) memcpy(cell_ijk, m->cell_ijk, sizeof(int32_t) * 3 * m->n);
  if (level)
    parallel_chunks(m->n, host_threads(), [&](int, int64_t a, int64_t b) {
      for (int64_t c = a; c < b; c++) level[c] = ffv_info_level(m->info[c]);
    });
  return FFV_OK;
}
