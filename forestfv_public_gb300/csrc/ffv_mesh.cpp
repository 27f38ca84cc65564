// Host-side face-table builder for Cartesian forests of hex octrees.
//
// Replaces, for forests of axis-aligned cubic trees, the reference's neighbour search
// (elconn.c:3-145, elconnfin.c, brchconn.c) and geometry (meshproperties.c:3-126,
// normalvector.c:15-46, tagvector.c:60-87, distance.c:120-167).  Input is the set of
// leaves; output is the cell order of the reference's leaf list (rebuildlist.c:30-91)
// plus owner-sorted tables: one 32-bit info word per cell (6 x 4-bit face kinds and the
// level), one neighbour slot per cell face, and 4-entry subface groups for the coarse
// side of 2:1 faces.  Geometry is not stored per cell: on a Cartesian forest it is a
// function of level and face index, evaluated here once per level with the reference's
// own formulas so that the device reproduces the reference's values bit for bit.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "ffv_internal.h"

namespace {

struct V3 {
  double x, y, z;
};

V3 corner_pos(int k, double h) {
  return V3{ffv_corner_x(k) * h, ffv_corner_y(k) * h, ffv_corner_z(k) * h};
}

// normalvector.c:23-29: n = (P1-P0) x (P2-P0) / |.|, component formulas as written there.
V3 face_normal(const V3 *nd, int f) {
  const V3 &p0 = nd[ffv_face_nodes[f][0]], &p1 = nd[ffv_face_nodes[f][1]],
           &p2 = nd[ffv_face_nodes[f][2]];
  double a = (p1.y - p0.y) * (p2.z - p0.z) - (p2.y - p0.y) * (p1.z - p0.z);
  double b = (p1.x - p0.x) * (p2.z - p0.z) - (p2.x - p0.x) * (p1.z - p0.z);
  double c = (p1.x - p0.x) * (p2.y - p0.y) - (p2.x - p0.x) * (p1.y - p0.y);
  double norm = sqrt(a * a + b * b + c * c);
  return V3{a / norm, -b / norm, c / norm};
}

// tagvector.c:69-83: t1 along the first face edge, t2 = n x t1 normalised.
void face_tangents(const V3 *nd, int f, const V3 &n, V3 *t1, V3 *t2) {
  const V3 &p0 = nd[ffv_face_nodes[f][0]], &p1 = nd[ffv_face_nodes[f][1]];
  double norm = sqrt((p1.y - p0.y) * (p1.y - p0.y) + (p1.x - p0.x) * (p1.x - p0.x) +
                     (p1.z - p0.z) * (p1.z - p0.z));
  *t1 = V3{(p1.x - p0.x) / norm, (p1.y - p0.y) / norm, (p1.z - p0.z) / norm};
  double a = n.y * t1->z - t1->y * n.z, b = n.x * t1->z - t1->x * n.z,
         c = n.x * t1->y - t1->x * n.y;
  double norm1 = sqrt(a * a + b * b + c * c);
  *t2 = V3{a / norm1, -b / norm1, c / norm1};
}

// meshproperties.c:61-69: face area as a fan of triangles from node 0.
double face_area(const V3 *nd, int f) {
  double area = 0.0;
  for (int it = 0; it < 2; it++) {
    const V3 &p0 = nd[ffv_face_nodes[f][0]], &p1 = nd[ffv_face_nodes[f][1 + it]],
             &p2 = nd[ffv_face_nodes[f][2 + it]];
    double dx1 = p1.x - p0.x, dx2 = p2.x - p0.x, dy1 = p1.y - p0.y, dy2 = p2.y - p0.y,
           dz1 = p1.z - p0.z, dz2 = p2.z - p0.z;
    double cx = dy1 * dz2 - dz1 * dy2, cy = dz1 * dx2 - dx1 * dz2, cz = dx1 * dy2 - dy1 * dx2;
    area += fabs(0.5 * sqrt(cx * cx + cy * cy + cz * cz));
  }
  return area;
}

// meshproperties.c:83-123: signed volume of the hex as six tetrahedra on node 0.
double hex_volume(const V3 *nd) {
  static const int vn[6][3] = {{1, 3, 5}, {5, 3, 7}, {5, 7, 4}, {3, 2, 7}, {7, 2, 6}, {7, 6, 4}};
  double vol = 0.0;
  for (int it = 0; it < 6; it++) {
    double dx[3], dy[3], dz[3];
    for (int in = 0; in < 3; in++) {
      dx[in] = nd[vn[it][in]].x - nd[0].x;
      dy[in] = nd[vn[it][in]].y - nd[0].y;
      dz[in] = nd[vn[it][in]].z - nd[0].z;
    }
    double c0 = dy[0] * dz[1] - dz[0] * dy[1], c1 = dz[0] * dx[1] - dx[0] * dz[1],
           c2 = dx[0] * dy[1] - dy[0] * dx[1];
    vol += (c0 * dx[2] + c1 * dy[2] + c2 * dz[2]) / 6.0;
  }
  return vol;
}

int axis_of(const V3 &v, int8_t *axis, int8_t *sign) {
  const double c[3] = {v.x, v.y, v.z};
  int found = -1;
  for (int a = 0; a < 3; a++) {
    if (c[a] == 1.0 || c[a] == -1.0) {
      if (found >= 0) return -1;
      found = a;
    } else if (c[a] != 0.0) {
      return -1;
    }
  }
  if (found < 0) return -1;
  *axis = (int8_t)found;
  *sign = (int8_t)(c[found] > 0 ? 1 : -1);
  return 0;
}

uint64_t cell_key(int level, uint32_t gx, uint32_t gy, uint32_t gz) {
  return ((uint64_t)level << 60) | ffv_morton(gx, gy, gz);
}

// fn(t, c0, c1) over [0, n) in nthreads contiguous chunks, on nthreads host threads
// open-addressing map from cell keys to cell indices (linear probing, power-of-two size;
// filled once, then only read -- from several threads)
struct CellMap {
  // key and value side by side: a probe touches one cache line
  struct Slot {
    uint64_t key;
    int32_t val;  // -1: empty slot
    int32_t pad;
  };
  std::unique_ptr<Slot[]> slot;  // allocated without initialisation, filled in parallel
  uint64_t mask = 0;
  CellMap(int64_t n, int nthreads) {
    uint64_t cap = 16;
    while (cap < (uint64_t)(2 * n)) cap <<= 1;
    slot.reset(new Slot[cap]);
    mask = cap - 1;
    parallel_chunks((int64_t)cap, nthreads, [&](int, int64_t a, int64_t b) {
      for (int64_t i = a; i < b; i++) slot[i].val = -1;
    });
  }
  static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // insert a key known to be absent (keys are distinct: overlapping leaves are rejected
  // before); safe from several threads at once -- a slot is claimed by an atomic
  // compare-and-swap of its value, and the table is only read after all inserts
  void put_new(uint64_t k, int32_t v) {
    for (uint64_t i = mix(k) & mask;; i = (i + 1) & mask) {
      int32_t expect = -1;
      if (__atomic_compare_exchange_n(&slot[i].val, &expect, v, false, __ATOMIC_RELAXED,
                                      __ATOMIC_RELAXED)) {
        slot[i].key = k;
        return;
      }
    }
  }
  int32_t get(uint64_t k) const {
    for (uint64_t i = mix(k) & mask;; i = (i + 1) & mask) {
      const Slot &e = slot[i];
      if (e.val < 0) return -1;
      if (e.key == k) return e.val;
    }
  }
};

}  // namespace

// part: the leaves are a part of a forest (one rank's cells and halo): a face whose
// neighbour, or any of whose four finer neighbours, is not among them becomes a transmissive
// boundary face instead of an error
static int mesh_build(const ffv_forest_desc *desc, int64_t nleaves, const int32_t *tree_ijk,
                      const int32_t *level, const int32_t *cell_ijk, ffv_mesh **out,
                      int64_t *order_out, bool part) {
  if (!desc || !tree_ijk || !level || !cell_ijk || !out || nleaves <= 0) return FFV_ERR_ARG;
  if (nleaves > (int64_t)INT32_MAX / 8) return FFV_ERR_ARG;
  *out = nullptr;
  const int32_t *T = desc->ntrees;
  for (int a = 0; a < 3; a++)
    if (T[a] <= 0 || T[a] > (1 << 16)) return FFV_ERR_ARG;
  if (!(desc->tree_edge > 0.0)) return FFV_ERR_ARG;
  for (int s = 0; s < 6; s++)
    if (desc->bc[s] < 1 || desc->bc[s] > 5) return FFV_ERR_ARG;

  const int nthreads = host_threads();
  std::vector<int> tmin(nthreads, FFV_MAX_LEVEL), tmax(nthreads, 1), terr(nthreads, FFV_OK);
  // per-thread results in locals, stored once (the threads' slots share cache lines)
  parallel_chunks(nleaves, nthreads, [&](int t, int64_t c0, int64_t c1) {
    int err = FFV_OK, lo = FFV_MAX_LEVEL, hi = 1;
    for (int64_t i = c0; i < c1 && err == FFV_OK; i++) {
      int l = level[i];
      if (l < 1 || l > FFV_MAX_LEVEL) {
        err = FFV_ERR_TABLE;
        break;
      }
      lo = std::min(lo, l);
      hi = std::max(hi, l);
      const int32_t ext = 1 << (l - 1);
      for (int a = 0; a < 3; a++)
        if (tree_ijk[3 * i + a] < 0 || tree_ijk[3 * i + a] >= T[a] || cell_ijk[3 * i + a] < 0 ||
            cell_ijk[3 * i + a] >= ext)
          err = FFV_ERR_TABLE;
      // global coordinates at the leaf level must fit the 21-bit Morton lanes
      if (err == FFV_OK && ((int64_t)T[0] * ext > (1 << 21) || (int64_t)T[1] * ext > (1 << 21) ||
                            (int64_t)T[2] * ext > (1 << 21)))
        err = FFV_ERR_UNSUPPORTED;
    }
    terr[t] = err;
    tmin[t] = lo;
    tmax[t] = hi;
  });
  int lmin = FFV_MAX_LEVEL, lmax = 1;
  for (int t = 0; t < nthreads; t++) {
    if (terr[t] != FFV_OK) return terr[t];
    lmin = std::min(lmin, tmin[t]);
    lmax = std::max(lmax, tmax[t]);
  }
  const int D = lmax - 1;  // local depth of the finest leaves

  // canonical order: trees by Morton key of their indices, then depth-first by child index
  std::vector<int64_t> perm(nleaves);
  std::vector<uint64_t> tkey(nleaves), lkey(nleaves);
  parallel_chunks(nleaves, nthreads, [&](int, int64_t c0, int64_t c1) {
    for (int64_t i = c0; i < c1; i++) {
      perm[i] = i;
      tkey[i] = ffv_morton(tree_ijk[3 * i], tree_ijk[3 * i + 1], tree_ijk[3 * i + 2]);
      int sh = D - (level[i] - 1);
      lkey[i] = ffv_morton((uint32_t)cell_ijk[3 * i] << sh, (uint32_t)cell_ijk[3 * i + 1] << sh,
                       (uint32_t)cell_ijk[3 * i + 2] << sh);
    }
  });
  auto before = [&](int64_t a, int64_t b) {
    if (tkey[a] != tkey[b]) return tkey[a] < tkey[b];
    if (lkey[a] != lkey[b]) return lkey[a] < lkey[b];
    return level[a] < level[b];
  };
  // leaves given in canonical order (a regrid's output) need no sort
  std::vector<char> unsorted(nthreads, 0), overlap(nthreads, 0);
  parallel_chunks(nleaves > 0 ? nleaves - 1 : 0, nthreads, [&](int t, int64_t a, int64_t b) {
    bool u = false;
    for (int64_t i = a; i < b && !u; i++) u = before(i + 1, i);
    unsorted[t] = u;
  });
  if (std::any_of(unsorted.begin(), unsorted.end(), [](char x) { return x != 0; }))
    std::sort(perm.begin(), perm.end(), before);
  // overlap check: a leaf's key range must end before the next leaf of the same tree starts
  parallel_chunks(nleaves > 0 ? nleaves - 1 : 0, nthreads, [&](int t, int64_t c0, int64_t c1) {
    bool ov = false;
    for (int64_t k = c0; k < c1 && !ov; k++) {
      int64_t a = perm[k], b = perm[k + 1];
      if (tkey[a] != tkey[b]) continue;
      uint64_t span = 1ULL << (3 * (D - (level[a] - 1)));
      if (lkey[a] + span > lkey[b]) ov = true;
    }
    overlap[t] = ov;
  });
  if (std::any_of(overlap.begin(), overlap.end(), [](char x) { return x != 0; }))
    return FFV_ERR_TABLE;

  ffv_mesh *m = new (std::nothrow) ffv_mesh();
  if (!m) return FFV_ERR_NOMEM;
  memset(m, 0, sizeof(*m));
  m->desc = *desc;
  m->n = nleaves;
  m->min_level = lmin;
  m->max_level = lmax;
  m->info = (uint32_t *)calloc((size_t)nleaves, sizeof(uint32_t));
  m->nbr = (int32_t *)malloc((size_t)nleaves * 6 * sizeof(int32_t));
  m->tree_ijk = (int32_t *)malloc((size_t)nleaves * 3 * sizeof(int32_t));
  m->cell_ijk = (int32_t *)malloc((size_t)nleaves * 3 * sizeof(int32_t));
  if (!m->info || !m->nbr || !m->tree_ijk || !m->cell_ijk) {
    ffv_mesh_free(m);
    return FFV_ERR_NOMEM;
  }

  // face frames and per-level geometry from the reference's formulas on a canonical cell
  {
    V3 nd[8];
    for (int k = 0; k < 8; k++) nd[k] = corner_pos(k, 1.0);
    for (int f = 0; f < 6; f++) {
      V3 n = face_normal(nd, f), t1, t2;
      face_tangents(nd, f, n, &t1, &t2);
      ffv_face_frame &fr = m->frame[f];
      if (axis_of(n, &fr.n_axis, &fr.n_sign) || axis_of(t1, &fr.t1_axis, &fr.t1_sign) ||
          axis_of(t2, &fr.t2_axis, &fr.t2_sign)) {
        ffv_mesh_free(m);
        return FFV_ERR_TABLE;
      }
      // the face's nodes share one coordinate: that axis and its value give the side
      const int *q = ffv_face_nodes[f];
      int bits[3][4];
      for (int j = 0; j < 4; j++) {
        bits[0][j] = ffv_corner_x(q[j]);
        bits[1][j] = ffv_corner_y(q[j]);
        bits[2][j] = ffv_corner_z(q[j]);
      }
      for (int a = 0; a < 3; a++)
        if (bits[a][0] == bits[a][1] && bits[a][0] == bits[a][2] && bits[a][0] == bits[a][3]) {
          fr.side_axis = (int8_t)a;
          fr.side_dir = (int8_t)(bits[a][0] ? 1 : -1);
        }
    }
    for (int l = 1; l <= FFV_MAX_LEVEL + 1; l++) {
      double h = desc->tree_edge / (double)(1 << (l - 1));
      for (int k = 0; k < 8; k++) nd[k] = corner_pos(k, h);
      m->geom[l].h = h;
      m->geom[l].vol = hex_volume(nd);
      m->geom[l].area = face_area(nd, 0);
    }
  }

  CellMap where(nleaves, nthreads);
  std::vector<uint32_t> gx(3 * nleaves);
  const int64_t chunk = (nleaves + nthreads - 1) / nthreads;
  auto fill = [&](int t) {
    const int64_t c0 = t * chunk, c1 = std::min<int64_t>(nleaves, c0 + chunk);
    for (int64_t c = c0; c < c1; c++) {
      int64_t i = perm[c];
      if (order_out) order_out[c] = i;
      for (int a = 0; a < 3; a++) {
        m->tree_ijk[3 * c + a] = tree_ijk[3 * i + a];
        m->cell_ijk[3 * c + a] = cell_ijk[3 * i + a];
        gx[3 * c + a] = (uint32_t)tree_ijk[3 * i + a] * (1u << (level[i] - 1)) +
                        (uint32_t)cell_ijk[3 * i + a];
      }
      where.put_new(cell_key(level[i], gx[3 * c], gx[3 * c + 1], gx[3 * c + 2]), (int32_t)c);
    }
  };
  {
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; t++) pool.emplace_back(fill, t);
    fill(0);
    for (auto &th : pool) th.join();
  }

  // face tables, in the same chunks; subface groups are numbered per chunk and shifted
  // afterwards, which gives the numbering of one sweep in cell order
  std::vector<std::vector<int32_t>> csub(nthreads);
  std::vector<int> crc(nthreads, FFV_OK);
  // first cell of c's complete group of eight sibling leaves (consecutive in canonical
  // order, child indices 0..7, one parent), or -1: a face between two of them needs no
  // lookup, the neighbour is the sibling with that axis' bit flipped
  auto kid_of = [&](int64_t c) {
    return (int)(((gx[3 * c] & 1) << 1) | (gx[3 * c + 1] & 1) | ((gx[3 * c + 2] & 1) << 2));
  };
  auto group_start = [&](int64_t c, int l) -> int64_t {
    if (l <= 1) return -1;
    const int64_t s0 = c - kid_of(c);
    if (s0 < 0 || s0 + 8 > nleaves) return -1;
    for (int q = 0; q < 8; q++) {
      const int64_t o = s0 + q;
      if (level[perm[o]] != l || kid_of(o) != q) return -1;
      for (int b = 0; b < 3; b++)
        if ((gx[3 * o + b] >> 1) != (gx[3 * c + b] >> 1)) return -1;
    }
    return s0;
  };
  auto work = [&](int t) {
    const int64_t c0 = t * chunk, c1 = std::min<int64_t>(nleaves, c0 + chunk);
    std::vector<int32_t> &sub = csub[t];
    for (int64_t c = c0; c < c1; c++) {
      int l = level[perm[c]];
      uint32_t info = (uint32_t)l << 24;
      const int64_t gs = group_start(c, l);
      const int kid = kid_of(c);
      for (int f = 0; f < 6; f++) {
        const ffv_face_frame &fr = m->frame[f];
        int a = fr.side_axis;
        int64_t g[3] = {gx[3 * c], gx[3 * c + 1], gx[3 * c + 2]};
        const int bit = (int)(g[a] & 1);
        g[a] += fr.side_dir;
        int64_t ext = (int64_t)T[a] << (l - 1);
        uint32_t kind;
        int32_t slot = -1;
        if (gs >= 0 && bit == (fr.side_dir > 0 ? 0 : 1)) {
          kind = FFV_FK_SAME;  // the sibling across the parent's inner face
          slot = (int32_t)(gs + (kid ^ (a == 0 ? 2 : (a == 1 ? 1 : 4))));
        } else if (g[a] < 0 || g[a] >= ext) {
          int side = 2 * a + (fr.side_dir > 0 ? 1 : 0);
          kind = FFV_FK_BC | (uint32_t)desc->bc[side];
        } else {
          int32_t hit = where.get(cell_key(l, (uint32_t)g[0], (uint32_t)g[1], (uint32_t)g[2]));
          if (hit >= 0) {
            kind = FFV_FK_SAME;
            slot = hit;
          } else if (l > 1 && (hit = where.get(cell_key(l - 1, (uint32_t)(g[0] >> 1),
                                                        (uint32_t)(g[1] >> 1),
                                                        (uint32_t)(g[2] >> 1)))) >= 0) {
            kind = FFV_FK_COARSER;
            slot = hit;
          } else {
            // four finer neighbours; subface k touches node ffv_face_nodes[f][k] of this face
            int32_t ids[4];
            bool ok = l < FFV_MAX_LEVEL;
            for (int k = 0; k < 4 && ok; k++) {
              int q = ffv_face_nodes[f][k];
              int cb[3] = {ffv_corner_x(q), ffv_corner_y(q), ffv_corner_z(q)};
              uint32_t fg[3];
              for (int b = 0; b < 3; b++)
                fg[b] = (uint32_t)(2 * g[b] + (b == a ? (fr.side_dir > 0 ? 0 : 1) : cb[b]));
              ids[k] = where.get(cell_key(l + 1, fg[0], fg[1], fg[2]));
              ok = ids[k] >= 0;
            }
            if (!ok && part) {
              info |= (FFV_FK_BC | (uint32_t)FFV_BC_OUTLET) << (4 * f);
              m->nbr[6 * c + f] = -1;
              continue;
            }
            if (!ok) {
              // distinguish a 2:1 violation (deeper leaves behind the face) from a hole
              bool deeper = false;
              for (int d = 2; d + l <= FFV_MAX_LEVEL && !deeper; d++) {
                uint32_t fg[3];
                for (int b = 0; b < 3; b++)
                  fg[b] = (uint32_t)((g[b] << d) + (b == a ? (fr.side_dir > 0 ? 0 : (1 << d) - 1) : 0));
                deeper = where.get(cell_key(l + d, fg[0], fg[1], fg[2])) >= 0;
              }
              bool coarser = false;
              for (int d = 2; l - d >= 1 && !coarser; d++)
                coarser = where.get(cell_key(l - d, (uint32_t)(g[0] >> d), (uint32_t)(g[1] >> d),
                                             (uint32_t)(g[2] >> d))) >= 0;
              crc[t] = (deeper || coarser) ? FFV_ERR_BALANCE : FFV_ERR_TABLE;
              return;
            }
            kind = FFV_FK_FINER;
            slot = (int32_t)(sub.size() / 4);  // shifted by the chunk's offset below
            sub.insert(sub.end(), ids, ids + 4);
          }
        }
        info |= kind << (4 * f);
        m->nbr[6 * c + f] = slot;
      }
      m->info[c] = info;
    }
  };
  {
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; t++) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
  }
  int rc = FFV_OK;
  for (int t = 0; t < nthreads && rc == FFV_OK; t++) rc = crc[t];
  if (rc != FFV_OK) {
    ffv_mesh_free(m);
    return rc;
  }
  std::vector<int32_t> sub;
  {
    size_t total = 0;
    for (auto &v : csub) total += v.size();
    sub.reserve(total);
    for (int t = 0; t < nthreads; t++) {
      const int32_t off = (int32_t)(sub.size() / 4);
      if (off) {
        const int64_t c0 = t * chunk, c1 = std::min<int64_t>(nleaves, c0 + chunk);
        for (int64_t c = c0; c < c1; c++)
          for (int f = 0; f < 6; f++)
            if (ffv_face_kind(m->info[c], f) == FFV_FK_FINER) m->nbr[6 * c + f] += off;
      }
      sub.insert(sub.end(), csub[t].begin(), csub[t].end());
    }
  }
  m->nsub = (int32_t)(sub.size() / 4);
  m->sub = (int32_t *)malloc(sizeof(int32_t) * (sub.size() ? sub.size() : 4));
  if (!m->sub) {
    ffv_mesh_free(m);
    return FFV_ERR_NOMEM;
  }
  if (!sub.empty()) memcpy(m->sub, sub.data(), sizeof(int32_t) * sub.size());
  *out = m;
  return FFV_OK;
}

extern "C" int ffv_mesh_build(const ffv_forest_desc *desc, int64_t nleaves,
                              const int32_t *tree_ijk, const int32_t *level,
                              const int32_t *cell_ijk, ffv_mesh **out, int64_t *order_out) {
  return mesh_build(desc, nleaves, tree_ijk, level, cell_ijk, out, order_out, false);
}

extern "C" int ffv_mesh_build_part(const ffv_forest_desc *desc, int64_t nleaves,
                                   const int32_t *tree_ijk, const int32_t *level,
                                   const int32_t *cell_ijk, ffv_mesh **out, int64_t *order_out) {
  return mesh_build(desc, nleaves, tree_ijk, level, cell_ijk, out, order_out, true);
}

int64_t ffv_sibling_group(const ffv_mesh *m, int64_t c) {
  const int l = ffv_info_level(m->info[c]);
  if (l <= 1) return -1;
  const int32_t *x = m->cell_ijk + 3 * c, *t = m->tree_ijk + 3 * c;
  const int64_t k = ((x[0] & 1) << 1) | (x[1] & 1) | ((x[2] & 1) << 2);
  const int64_t s = c - k;
  if (s < 0 || s + 8 > m->n) return -1;
  for (int64_t q = 0; q < 8; q++) {
    const int32_t *y = m->cell_ijk + 3 * (s + q), *u = m->tree_ijk + 3 * (s + q);
    if (ffv_info_level(m->info[s + q]) != l || u[0] != t[0] || u[1] != t[1] || u[2] != t[2] ||
        (y[0] >> 1) != (x[0] >> 1) || (y[1] >> 1) != (x[1] >> 1) || (y[2] >> 1) != (x[2] >> 1) ||
        (((y[0] & 1) << 1) | (y[1] & 1) | ((y[2] & 1) << 2)) != q)
      return -1;
  }
  return s;
}

extern "C" int64_t ffv_mesh_ncells(const ffv_mesh *m) { return m ? m->n : 0; }

extern "C" void ffv_mesh_free(ffv_mesh *m) {
  if (!m) return;
  free(m->info);
  free(m->nbr);
  free(m->sub);
  free(m->tree_ijk);
  free(m->cell_ijk);
  delete m;
}

// distance.c:120-167 for the three neighbour relations of a Cartesian forest; the centre
// distance d is exact (dyadic coordinates), so these are the reference's values.
static void face_dist(const ffv_mesh *m, int l, uint32_t kind, double *dcf, double *dcc) {
  if (kind & FFV_FK_BC) {  // neighbour is the forest root (level 0): no branch taken
    *dcf = 0.0;
    *dcc = 0.0;
  } else if (kind == FFV_FK_SAME) {
    double d = m->geom[l].h;
    *dcf = 0.5 * d;
    *dcc = d;
  } else if (kind == FFV_FK_FINER) {  // level_diff == 1: to the neighbour's parent
    double d = m->geom[l].h;
    *dcf = 0.5 * d;
    *dcc = 0.5 * d + 0.25 * d;
  } else {  // level_diff == -1: from this cell's parent
    double d = m->geom[l - 1].h;
    *dcf = 0.25 * d;
    *dcc = 0.25 * d + 0.5 * d;
  }
}

extern "C" int ffv_mesh_export(const ffv_mesh *m, int32_t *bc, int32_t *lfc_neigs,
                               int32_t *neigfc, int32_t *nb, double *area, double *nrm,
                               double *dist_cf, double *dist_cc, double *vol,
                               double *centroid) {
  if (!m) return FFV_ERR_ARG;
  for (int64_t c = 0; c < m->n; c++) {
    uint32_t info = m->info[c];
    int l = ffv_info_level(info);
    if (vol) vol[c] = m->geom[l].vol;
    if (centroid) {
      double h = m->geom[l].h;
      for (int a = 0; a < 3; a++) {
        double lo = (double)m->tree_ijk[3 * c + a] * m->desc.tree_edge +
                    (double)m->cell_ijk[3 * c + a] * h;
        // meshproperties.c:27-38: mean of the eight nodes, four at lo and four at lo+h
        centroid[3 * c + a] = (4.0 * lo + 4.0 * (lo + h)) / 8.0;
      }
    }
    for (int f = 0; f < 6; f++) {
      int64_t r = 6 * c + f;
      uint32_t kind = ffv_face_kind(info, f);
      if (bc) bc[r] = (kind & FFV_FK_BC) ? (int32_t)(kind & 7u) : 0;
      if (lfc_neigs) lfc_neigs[r] = (kind & FFV_FK_BC) ? 0 : (kind == FFV_FK_FINER ? 4 : 1);
      if (neigfc) neigfc[r] = ffv_face_opp[f];
      if (nb) {
        for (int k = 0; k < 4; k++) nb[4 * r + k] = -1;
        if (kind == FFV_FK_SAME || kind == FFV_FK_COARSER) nb[4 * r] = m->nbr[r];
        if (kind == FFV_FK_FINER)
          for (int k = 0; k < 4; k++) nb[4 * r + k] = m->sub[4 * m->nbr[r] + k];
      }
      if (area) {
        for (int k = 0; k < 4; k++) area[4 * r + k] = 0.0;
        if (kind == FFV_FK_FINER)
          for (int k = 0; k < 4; k++) area[4 * r + k] = m->geom[l + 1].area;
        else
          area[4 * r] = m->geom[l].area;
      }
      if (nrm) {
        const ffv_face_frame &fr = m->frame[f];
        double *v = nrm + 9 * r;
        for (int k = 0; k < 9; k++) v[k] = 0.0;
        v[fr.n_axis] = fr.n_sign;
        v[3 + fr.t1_axis] = fr.t1_sign;
        v[6 + fr.t2_axis] = fr.t2_sign;
      }
      double dcf, dcc;
      face_dist(m, l, kind, &dcf, &dcc);
      if (dist_cf) dist_cf[r] = dcf;
      if (dist_cc) dist_cc[r] = dcc;
    }
  }
  return FFV_OK;
}
