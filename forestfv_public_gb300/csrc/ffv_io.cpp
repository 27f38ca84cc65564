// Checkpoint/restart and field export (host side).
//
// Binary checkpoint: a Morton-keyed leaf list and the SoA FP64 state, bit-exact.  Layout
// (little-endian):
//   "FFVCKPT1"                                   8 bytes
//   int32 version (1), int32 neq, int64 n, int64 istep, double time,
//   int32 ntrees[3], int32 bc[6], double tree_edge                      80 bytes
//   uint32 tree[n]   rank of the leaf's tree in Morton order of the tree coordinates
//   uint8  level[n]
//   uint64 key[n]    the leaf's child indices from level 2 down, 3 bits each, the
//                    deepest in the lowest bits (corner k at (bit1 k, bit0 k, bit2 k))
//   double S[neq][n]
//   uint64 FNV-1a hash of every byte after the magic
//
// The reference's text restart (restart_save.c:13-50, restart_load.c:13-45): a header line
// "istep time nleaves ntrees neq", then per leaf "root tag" and the neq state values with
// "%15.10e" (eleven significant digits); root is the tree's index in Morton order of the
// tree coordinates, tag the base-10 number whose digit j (from the lowest, j = 0) is one
// plus the child index at level j + 2 (tagaddress.c:3-11).
//
// Tecplot ASCII (headless): one FEBRICK zone, nodes shared between leaves on the lattice of
// the finest level, the cell fields in BLOCK form with VARLOCATION cell-centred.
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "ffv_internal.h"

extern "C" int ffv_mesh_build(const ffv_forest_desc *desc, int64_t nleaves, const int32_t *tree_ijk,
                              const int32_t *level, const int32_t *cell_ijk, ffv_mesh **out,
                              int64_t *order_out);
extern "C" void ffv_mesh_free(ffv_mesh *m);

namespace {

const char kMagic[8] = {'F', 'F', 'V', 'C', 'K', 'P', 'T', '1'};

struct Header {
  int32_t version, neq;
  int64_t n, istep;
  double time;
  int32_t ntrees[3], bc[6];
  double tree_edge;
};
static_assert(sizeof(Header) == 80, "checkpoint header layout");

uint64_t fnv1a(uint64_t h, const void *p, size_t len) {
  const uint8_t *b = (const uint8_t *)p;
  for (size_t i = 0; i < len; i++) {
    h ^= b[i];
    h *= 0x100000001B3ull;
  }
  return h;
}
const uint64_t kFnvBasis = 0xCBF29CE484222325ull;

// trees in Morton order of their coordinates: rank -> (i, j, k) and (i, j, k) -> rank
struct TreeOrder {
  std::vector<int32_t> ijk;   // [3 T] by rank
  std::vector<uint32_t> rank;  // by (i * ny + j) * nz + k
  int32_t nt[3];
  explicit TreeOrder(const int32_t ntrees[3]) {
    for (int d = 0; d < 3; d++) nt[d] = ntrees[d];
    const int64_t T = (int64_t)nt[0] * nt[1] * nt[2];
    std::vector<std::pair<uint64_t, int64_t>> k(T);
    for (int64_t t = 0; t < T; t++) {
      const int32_t i = (int32_t)(t / ((int64_t)nt[1] * nt[2]));
      const int32_t j = (int32_t)((t / nt[2]) % nt[1]);
      const int32_t l = (int32_t)(t % nt[2]);
      k[t] = {ffv_morton(i, j, l), t};
    }
    std::sort(k.begin(), k.end());
    ijk.resize(3 * T);
    rank.resize(T);
    for (int64_t r = 0; r < T; r++) {
      const int64_t t = k[r].second;
      ijk[3 * r] = (int32_t)(t / ((int64_t)nt[1] * nt[2]));
      ijk[3 * r + 1] = (int32_t)((t / nt[2]) % nt[1]);
      ijk[3 * r + 2] = (int32_t)(t % nt[2]);
      rank[t] = (uint32_t)r;
    }
  }
  uint32_t of(const int32_t *t) const {
    return rank[((int64_t)t[0] * nt[1] + t[1]) * nt[2] + t[2]];
  }
};

// child index of a leaf at level j (2 <= j <= l) from its coordinates at level l
inline int child_at(const int32_t *c, int l, int j) {
  const int s = l - j;
  return (((c[0] >> s) & 1) << 1) | ((c[1] >> s) & 1) | (((c[2] >> s) & 1) << 2);
}

// rebuild a mesh from leaves in any order; S_in [neq][n] in that order goes to S_out in
// the mesh's cell order
int build_with_state(const ffv_forest_desc *desc, int64_t n, const std::vector<int32_t> &tij,
                     const std::vector<int32_t> &lev, const std::vector<int32_t> &cij,
                     const double *S_in, int32_t neq, ffv_mesh **out, double *S_out) {
  std::vector<int64_t> order(n);
  int rc = ffv_mesh_build(desc, n, tij.data(), lev.data(), cij.data(), out, order.data());
  if (rc != FFV_OK) return rc;
  if (S_out)
    for (int32_t v = 0; v < neq; v++)
      for (int64_t i = 0; i < n; i++) S_out[(int64_t)v * n + i] = S_in[(int64_t)v * n + order[i]];
  return FFV_OK;
}

struct File {
  FILE *f;
  explicit File(FILE *x) : f(x) {}
  ~File() {
    if (f) fclose(f);
  }
};

}  // namespace

extern "C" {

int ffv_checkpoint_write(const char *path, const ffv_mesh *m, const double *S, int32_t neq,
                         int64_t istep, double time) {
  if (!path || !m || !S || neq < 1) return FFV_ERR_ARG;
  const int64_t n = m->n;
  Header h{};
  h.version = 1;
  h.neq = neq;
  h.n = n;
  h.istep = istep;
  h.time = time;
  memcpy(h.ntrees, m->desc.ntrees, sizeof(h.ntrees));
  memcpy(h.bc, m->desc.bc, sizeof(h.bc));
  h.tree_edge = m->desc.tree_edge;
  TreeOrder to(m->desc.ntrees);
  std::vector<uint32_t> tree(n);
  std::vector<uint8_t> level(n);
  std::vector<uint64_t> key(n);
  for (int64_t c = 0; c < n; c++) {
    const int l = ffv_info_level(m->info[c]);
    tree[c] = to.of(m->tree_ijk + 3 * c);
    level[c] = (uint8_t)l;
    uint64_t k = 0;
    for (int j = 2; j <= l; j++) k = (k << 3) | (uint64_t)child_at(m->cell_ijk + 3 * c, l, j);
    key[c] = k;
  }
  File f(fopen(path, "wb"));
  if (!f.f) return FFV_ERR_IO;
  uint64_t hash = kFnvBasis;
  auto put = [&](const void *p, size_t len) {
    hash = fnv1a(hash, p, len);
    return fwrite(p, 1, len, f.f) == len;
  };
  bool ok = fwrite(kMagic, 1, 8, f.f) == 8 && put(&h, sizeof(h)) &&
            put(tree.data(), sizeof(uint32_t) * n) && put(level.data(), n) &&
            put(key.data(), sizeof(uint64_t) * n) && put(S, sizeof(double) * neq * n);
  ok = ok && fwrite(&hash, 1, 8, f.f) == 8;
  ok = (fflush(f.f) == 0) && ok;
  return ok ? FFV_OK : FFV_ERR_IO;
}

int ffv_checkpoint_info(const char *path, ffv_forest_desc *desc, int64_t *n, int32_t *neq,
                        int64_t *istep, double *time) {
  if (!path) return FFV_ERR_ARG;
  File f(fopen(path, "rb"));
  if (!f.f) return FFV_ERR_IO;
  char mg[8];
  Header h;
  if (fread(mg, 1, 8, f.f) != 8 || memcmp(mg, kMagic, 8) != 0) return FFV_ERR_IO;
  if (fread(&h, 1, sizeof(h), f.f) != sizeof(h) || h.version != 1 || h.n < 0 || h.neq < 1)
    return FFV_ERR_IO;
  if (desc) {
    memcpy(desc->ntrees, h.ntrees, sizeof(h.ntrees));
    memcpy(desc->bc, h.bc, sizeof(h.bc));
    desc->tree_edge = h.tree_edge;
  }
  if (n) *n = h.n;
  if (neq) *neq = h.neq;
  if (istep) *istep = h.istep;
  if (time) *time = h.time;
  return FFV_OK;
}

int ffv_checkpoint_read(const char *path, ffv_mesh **out, double *S) {
  if (!path || !out) return FFV_ERR_ARG;
  *out = nullptr;
  File f(fopen(path, "rb"));
  if (!f.f) return FFV_ERR_IO;
  char mg[8];
  Header h;
  if (fread(mg, 1, 8, f.f) != 8 || memcmp(mg, kMagic, 8) != 0) return FFV_ERR_IO;
  if (fread(&h, 1, sizeof(h), f.f) != sizeof(h) || h.version != 1 || h.n < 0 || h.neq < 1)
    return FFV_ERR_IO;
  const int64_t n = h.n;
  uint64_t hash = fnv1a(kFnvBasis, &h, sizeof(h));
  std::vector<uint32_t> tree(n);
  std::vector<uint8_t> level(n);
  std::vector<uint64_t> key(n);
  std::vector<double> Sin((size_t)h.neq * n);
  auto get = [&](void *p, size_t len) {
    if (fread(p, 1, len, f.f) != len) return false;
    hash = fnv1a(hash, p, len);
    return true;
  };
  uint64_t stored;
  if (!get(tree.data(), sizeof(uint32_t) * n) || !get(level.data(), n) ||
      !get(key.data(), sizeof(uint64_t) * n) || !get(Sin.data(), sizeof(double) * Sin.size()) ||
      fread(&stored, 1, 8, f.f) != 8 || stored != hash)
    return FFV_ERR_IO;
  ffv_forest_desc d;
  memcpy(d.ntrees, h.ntrees, sizeof(h.ntrees));
  memcpy(d.bc, h.bc, sizeof(h.bc));
  d.tree_edge = h.tree_edge;
  TreeOrder to(d.ntrees);
  const uint64_t T = (uint64_t)to.rank.size();
  std::vector<int32_t> tij(3 * n), lev(n), cij(3 * n);
  for (int64_t c = 0; c < n; c++) {
    const int l = level[c];
    if (tree[c] >= T || l < 1 || l > FFV_MAX_LEVEL) return FFV_ERR_IO;
    for (int d3 = 0; d3 < 3; d3++) tij[3 * c + d3] = to.ijk[3 * tree[c] + d3];
    lev[c] = l;
    int32_t x = 0, y = 0, z = 0;
    for (int j = 2; j <= l; j++) {
      const int k = (int)((key[c] >> (3 * (l - j))) & 7);
      x = 2 * x + ((k >> 1) & 1);
      y = 2 * y + (k & 1);
      z = 2 * z + ((k >> 2) & 1);
    }
    cij[3 * c] = x;
    cij[3 * c + 1] = y;
    cij[3 * c + 2] = z;
  }
  return build_with_state(&d, n, tij, lev, cij, Sin.data(), h.neq, out, S);
}

int ffv_restart_text_write(const char *path, const ffv_mesh *m, const double *S, int32_t neq,
                           int64_t istep, double time) {
  if (!path || !m || !S || neq < 1) return FFV_ERR_ARG;
  if (m->max_level > 10) return FFV_ERR_UNSUPPORTED;  // tags are 32-bit base-10 numbers
  TreeOrder to(m->desc.ntrees);
  File f(fopen(path, "w"));
  if (!f.f) return FFV_ERR_IO;
  const int64_t n = m->n;
  bool ok = fprintf(f.f, "%d %15.10e %d %d %d \n", (int)istep, time, (int)n,
                    (int)to.rank.size(), (int)neq) > 0;
  for (int64_t c = 0; c < n && ok; c++) {
    const int l = ffv_info_level(m->info[c]);
    int64_t tag = 0, p10 = 1;
    for (int j = 2; j <= l; j++, p10 *= 10) tag += p10 * (1 + child_at(m->cell_ijk + 3 * c, l, j));
    ok = fprintf(f.f, "%d %d ", (int)to.of(m->tree_ijk + 3 * c), (int)tag) > 0;
    for (int32_t v = 0; v < neq && ok; v++) ok = fprintf(f.f, " %15.10e ", S[(int64_t)v * n + c]) > 0;
    ok = ok && fputc('\n', f.f) != EOF;
  }
  ok = (fflush(f.f) == 0) && ok;
  return ok ? FFV_OK : FFV_ERR_IO;
}

int ffv_restart_text_info(const char *path, int64_t *n, int32_t *neq, int64_t *istep, double *time,
                          int32_t *ntrees_total) {
  if (!path) return FFV_ERR_ARG;
  File f(fopen(path, "r"));
  if (!f.f) return FFV_ERR_IO;
  int is, nl, nt, nv;
  double t;
  if (fscanf(f.f, "%d %lf %d %d %d", &is, &t, &nl, &nt, &nv) != 5 || nl < 0 || nv < 1)
    return FFV_ERR_IO;
  if (n) *n = nl;
  if (neq) *neq = nv;
  if (istep) *istep = is;
  if (time) *time = t;
  if (ntrees_total) *ntrees_total = nt;
  return FFV_OK;
}

int ffv_restart_text_read(const char *path, const ffv_forest_desc *desc, ffv_mesh **out,
                          double *S) {
  if (!path || !desc || !out) return FFV_ERR_ARG;
  *out = nullptr;
  File f(fopen(path, "r"));
  if (!f.f) return FFV_ERR_IO;
  int is, nl, nt, nv;
  double t;
  if (fscanf(f.f, "%d %lf %d %d %d", &is, &t, &nl, &nt, &nv) != 5 || nl < 0 || nv < 1)
    return FFV_ERR_IO;
  TreeOrder to(desc->ntrees);
  if ((int64_t)nt != (int64_t)to.rank.size()) return FFV_ERR_ARG;
  const int64_t n = nl;
  std::vector<int32_t> tij(3 * n), lev(n), cij(3 * n);
  std::vector<double> Sin((size_t)nv * n);
  for (int64_t c = 0; c < n; c++) {
    int root, tag;
    if (fscanf(f.f, "%d %d", &root, &tag) != 2 || root < 0 || root >= nt || tag < 0)
      return FFV_ERR_IO;
    // restart_load.c -> spawntree.c:21-33: the digits of tag, lowest first, are the child
    // indices plus one from level 2 down
    int digits[10], nd = 0;
    for (int tg = tag; tg > 0; tg /= 10) {
      if (nd == 10 || tg % 10 < 1 || tg % 10 > 8) return FFV_ERR_IO;
      digits[nd++] = tg % 10 - 1;
    }
    int32_t x = 0, y = 0, z = 0;
    for (int j = 0; j < nd; j++) {
      const int k = digits[j];
      x = 2 * x + ((k >> 1) & 1);
      y = 2 * y + (k & 1);
      z = 2 * z + ((k >> 2) & 1);
    }
    for (int d3 = 0; d3 < 3; d3++) tij[3 * c + d3] = to.ijk[3 * root + d3];
    lev[c] = 1 + nd;
    cij[3 * c] = x;
    cij[3 * c + 1] = y;
    cij[3 * c + 2] = z;
    for (int v = 0; v < nv; v++)
      if (fscanf(f.f, "%lf", &Sin[(size_t)v * n + c]) != 1) return FFV_ERR_IO;
  }
  return build_with_state(desc, n, tij, lev, cij, Sin.data(), nv, out, S);
}

int ffv_tecplot_write(const char *path, const ffv_mesh *m, int32_t nfields, const char *const *names,
                      const double *F, double time) {
  if (!path || !m || (nfields > 0 && (!names || !F)) || nfields < 0) return FFV_ERR_ARG;
  const int64_t n = m->n;
  const int L = m->max_level;
  // nodes on the lattice of the finest level, shared between the leaves that touch them
  const int64_t e = (int64_t)1 << (L - 1);  // lattice steps per tree edge
  const int64_t NX = (int64_t)m->desc.ntrees[0] * e + 1, NY = (int64_t)m->desc.ntrees[1] * e + 1;
  std::unordered_map<int64_t, int64_t> node_id;
  node_id.reserve((size_t)(2 * n + 16));
  std::vector<int64_t> nodes;  // lattice keys by node id
  std::vector<int64_t> conn(8 * n);
  // FEBRICK corner order: (0,0,0) (1,0,0) (1,1,0) (0,1,0) then the same at z + 1
  const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
            cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int64_t c = 0; c < n; c++) {
    const int l = ffv_info_level(m->info[c]);
    const int64_t s = (int64_t)1 << (L - l);  // leaf edge in lattice steps
    const int64_t gx = ((int64_t)m->tree_ijk[3 * c] << (l - 1)) + m->cell_ijk[3 * c];
    const int64_t gy = ((int64_t)m->tree_ijk[3 * c + 1] << (l - 1)) + m->cell_ijk[3 * c + 1];
    const int64_t gz = ((int64_t)m->tree_ijk[3 * c + 2] << (l - 1)) + m->cell_ijk[3 * c + 2];
    for (int q = 0; q < 8; q++) {
      const int64_t key = ((gz + cz[q]) * s * NY + (gy + cy[q]) * s) * NX + (gx + cx[q]) * s;
      auto it = node_id.find(key);
      if (it == node_id.end()) {
        it = node_id.emplace(key, (int64_t)nodes.size()).first;
        nodes.push_back(key);
      }
      conn[8 * c + q] = it->second;
    }
  }
  File f(fopen(path, "w"));
  if (!f.f) return FFV_ERR_IO;
  bool ok = fprintf(f.f, "TITLE = \"forestfv fields\"\nVARIABLES = \"X\" \"Y\" \"Z\"") > 0;
  for (int32_t v = 0; v < nfields && ok; v++) ok = fprintf(f.f, " \"%s\"", names[v]) > 0;
  ok = ok && fprintf(f.f, "\nZONE T=\"t=%.10e\", N=%lld, E=%lld, DATAPACKING=BLOCK, "
                          "ZONETYPE=FEBRICK, SOLUTIONTIME=%.10e",
                     time, (long long)nodes.size(), (long long)n, time) > 0;
  if (nfields > 0) ok = ok && fprintf(f.f, ", VARLOCATION=([4-%d]=CELLCENTERED)", 3 + nfields) > 0;
  ok = ok && fputc('\n', f.f) != EOF;
  const double h = m->desc.tree_edge / (double)e;
  for (int d3 = 0; d3 < 3 && ok; d3++) {
    for (size_t i = 0; i < nodes.size() && ok; i++) {
      const int64_t k = nodes[i];
      const int64_t q = d3 == 0 ? k % NX : (d3 == 1 ? (k / NX) % NY : k / (NX * NY));
      ok = fprintf(f.f, "%.10e%c", (double)q * h, (i % 6 == 5) ? '\n' : ' ') > 0;
    }
    ok = ok && fputc('\n', f.f) != EOF;
  }
  for (int32_t v = 0; v < nfields && ok; v++) {
    for (int64_t c = 0; c < n && ok; c++)
      ok = fprintf(f.f, "%.10e%c", F[(int64_t)v * n + c], (c % 6 == 5) ? '\n' : ' ') > 0;
    ok = ok && fputc('\n', f.f) != EOF;
  }
  for (int64_t c = 0; c < n && ok; c++)
    ok = fprintf(f.f, "%lld %lld %lld %lld %lld %lld %lld %lld\n",
                 (long long)conn[8 * c] + 1, (long long)conn[8 * c + 1] + 1,
                 (long long)conn[8 * c + 2] + 1, (long long)conn[8 * c + 3] + 1,
                 (long long)conn[8 * c + 4] + 1, (long long)conn[8 * c + 5] + 1,
                 (long long)conn[8 * c + 6] + 1, (long long)conn[8 * c + 7] + 1) > 0;
  ok = (fflush(f.f) == 0) && ok;
  return ok ? FFV_OK : FFV_ERR_IO;
}

}  // extern "C"
