// One refineh pass on the host tables: the new leaf list (refineh.c:3-57 -- merges of eight
// sibling leaves that all want a coarser level, splits of leaves that want a finer one) and
// its face tables, rebuilt only where the pass changed something.
//
// A leaf that is kept and none of whose face neighbours splits or merges has the faces it
// had, with renumbered neighbours: its table rows are copied through the old-to-new index
// map.  Every other leaf (a child of a split, a merged parent, a kept leaf beside either)
// finds its neighbours by binary search in the new leaves' Morton keys, which are sorted in
// leaf order: the leaf whose key range holds the first point of the neighbouring cell of the
// same level is that cell, its parent (the neighbour is coarser) or a descendant (the region
// is refined: the four subface leaves are then looked up the same way and must be one level
// finer).  Subface groups are
// numbered in cell order, as ffv_mesh_build numbers them, so the tables equal the full
// builder's for the same leaves.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <new>
#include <vector>

#include "ffv_internal.h"

extern "C" void ffv_mesh_free(ffv_mesh *m);

namespace {

constexpr int kDepth = FFV_MAX_LEVEL - 1;  // Morton digits below the tree at the finest level

// The per-leaf arrays are left uninitialised when allocated and written in full by the
// parallel passes below, which thereby also take their first-touch page faults in parallel
// (a resized vector would fill them on one thread first).
template <typename T>
std::unique_ptr<T[]> uninit(int64_t n) {
  return std::unique_ptr<T[]>(new (std::nothrow) T[n > 0 ? n : 1]);
}

struct Leaves {
  int32_t *tij = nullptr, *cij = nullptr;  // new leaves in leaf order (the new mesh's arrays)
  std::unique_ptr<int32_t[]> lev;
  int64_t *src = nullptr;                // old leaf copied or split (>= 0), -1 - j merged from j..j+7
  std::unique_ptr<int64_t[]> own_src;    // src's storage when the caller does not want it
  std::unique_ptr<int32_t[]> old2new;    // kept old leaves' new index, else -1
  std::unique_ptr<uint8_t[]> what;       // per old leaf: 0 absorbed, 1 kept, 2 merged parent, 8 split
  std::vector<int64_t> tsum;             // new leaves before each chunk of old leaves
  int64_t nn = 0;
};

// the pass's new leaves, counted: a per-old-leaf count and a prefix sum (a leaf whose
// target is not below its level cannot be part of a merge: no group lookup)
int count_leaves(const ffv_mesh *m, const int32_t *split, int nth, Leaves &L) {
  const int64_t n = m->n;
  L.what = uninit<uint8_t>(n);
  if (!L.what) return FFV_ERR_NOMEM;
  std::vector<int64_t> &tsum = L.tsum;
  tsum.assign(nth + 1, 0);
  std::vector<char> bad(nth, 0);
  parallel_chunks(n, nth, [&](int t, int64_t a, int64_t b) {
    int64_t acc = 0;
    for (int64_t c = a; c < b; c++) {
      const int l = ffv_info_level(m->info[c]);
      const int64_t g = (l > 1 && split[c] < l) ? ffv_sibling_group(m, c) : -1;
      bool merge = g >= 0;
      for (int q = 0; q < 8 && merge; q++) merge = split[g + q] < l;
      uint8_t k;
      if (merge) k = (g == c) ? 2 : 0;
      else if (split[c] > l) k = 8;
      else k = 1;
      if (k == 8 && l + 1 > FFV_MAX_LEVEL) bad[t] = 1;
      L.what[c] = k;
      acc += k == 2 ? 1 : k;
    }
    tsum[t + 1] = acc;
  });
  if (std::any_of(bad.begin(), bad.end(), [](char x) { return x != 0; })) return FFV_ERR_TABLE;
  for (int t = 0; t < nth; t++) tsum[t + 1] += tsum[t];
  L.nn = tsum[nth];
  return FFV_OK;
}

// the new leaves written in the order one sweep in leaf order emits them, into L.tij / L.cij
bool fill_leaves(const ffv_mesh *m, int nth, Leaves &L) {
  const int64_t n = m->n, nn = L.nn;
  const std::vector<int64_t> &tsum = L.tsum;
  L.lev = uninit<int32_t>(nn);
  L.old2new = uninit<int32_t>(n);
  if (!L.lev || !L.old2new) return false;
  parallel_chunks(n, nth, [&](int t, int64_t a, int64_t b) {
    int64_t o = tsum[t];
    for (int64_t c = a; c < b; c++) {
      const uint8_t k = L.what[c];
      L.old2new[c] = k == 1 ? (int32_t)o : -1;
      if (k == 0) continue;
      const int l = ffv_info_level(m->info[c]);
      const int32_t *tr = m->tree_ijk + 3 * c, *x = m->cell_ijk + 3 * c;
      if (k == 2) {  // merge.c: the parent of eight leaves
        for (int d = 0; d < 3; d++) {
          L.tij[3 * o + d] = tr[d];
          L.cij[3 * o + d] = x[d] >> 1;
        }
        L.lev[o] = l - 1;
        L.src[o] = -1 - c;
        o++;
      } else if (k == 8) {  // split.c: eight children in child order, corner q at (bit1, bit0, bit2)
        for (int q = 0; q < 8; q++, o++) {
          for (int d = 0; d < 3; d++) L.tij[3 * o + d] = tr[d];
          L.cij[3 * o] = 2 * x[0] + ((q >> 1) & 1);
          L.cij[3 * o + 1] = 2 * x[1] + (q & 1);
          L.cij[3 * o + 2] = 2 * x[2] + ((q >> 2) & 1);
          L.lev[o] = l + 1;
          L.src[o] = c;
        }
      } else {
        for (int d = 0; d < 3; d++) {
          L.tij[3 * o + d] = tr[d];
          L.cij[3 * o + d] = x[d];
        }
        L.lev[o] = l;
        L.src[o] = c;
        o++;
      }
    }
  });
  return true;
}

// rank of each tree in Morton order of its coordinates, by linear index (i * ny + j) * nz + k
std::vector<uint64_t> tree_ranks(const int32_t nt[3]) {
  const int64_t T = (int64_t)nt[0] * nt[1] * nt[2];
  std::vector<std::pair<uint64_t, int64_t>> k(T);
  for (int64_t t = 0; t < T; t++)
    k[t] = {ffv_morton((uint32_t)(t / ((int64_t)nt[1] * nt[2])), (uint32_t)((t / nt[2]) % nt[1]),
                       (uint32_t)(t % nt[2])),
            t};
  std::sort(k.begin(), k.end());
  std::vector<uint64_t> rank(T);
  for (int64_t r = 0; r < T; r++) rank[k[r].second] = (uint64_t)r;
  return rank;
}

}  // namespace

extern "C" int ffv_mesh_adapt(const ffv_mesh *m, const int32_t *split, ffv_mesh **out,
                              int64_t *src) {
  if (!m || !split || !out) return FFV_ERR_ARG;
  *out = nullptr;
  const int nth = host_threads();
  Leaves L;
  int rc = count_leaves(m, split, nth, L);
  if (rc != FFV_OK) return rc;
  const int64_t nn = L.nn;
  if (nn > INT32_MAX) return FFV_ERR_TABLE;
  ffv_mesh *nm = new (std::nothrow) ffv_mesh();
  if (!nm) return FFV_ERR_NOMEM;
  memset(nm, 0, sizeof(*nm));
  nm->desc = m->desc;
  nm->n = nn;
  memcpy(nm->frame, m->frame, sizeof(m->frame));
  memcpy(nm->geom, m->geom, sizeof(m->geom));
  nm->info = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nn ? nn : 1));
  nm->nbr = (int32_t *)malloc(sizeof(int32_t) * 6 * (size_t)(nn ? nn : 1));
  nm->tree_ijk = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nn ? nn : 1));
  nm->cell_ijk = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nn ? nn : 1));
  if (!nm->info || !nm->nbr || !nm->tree_ijk || !nm->cell_ijk) {
    ffv_mesh_free(nm);
    return FFV_ERR_NOMEM;
  }
  L.tij = nm->tree_ijk;
  L.cij = nm->cell_ijk;
  if (src) {
    L.src = src;
  } else {
    L.own_src = uninit<int64_t>(nn);
    if (!L.own_src) {
      ffv_mesh_free(nm);
      return FFV_ERR_NOMEM;
    }
    L.src = L.own_src.get();
  }
  if (!fill_leaves(m, nth, L)) {
    ffv_mesh_free(nm);
    return FFV_ERR_NOMEM;
  }
  const int32_t *NT = m->desc.ntrees;
  const std::vector<uint64_t> rank = tree_ranks(NT);
  if (rank.size() >= (1ull << (64 - 3 * kDepth))) {
    ffv_mesh_free(nm);
    return FFV_ERR_TABLE;
  }
  auto lin = [&](int64_t i, int64_t j, int64_t k) { return (i * NT[1] + j) * NT[2] + k; };
  // the key of the first point of the level-l cell at global coordinates g (level l)
  auto point_key = [&](int l, const int64_t g[3]) {
    const int64_t t0 = g[0] >> (l - 1), t1 = g[1] >> (l - 1), t2 = g[2] >> (l - 1);
    const int sh = kDepth - (l - 1);
    return (rank[lin(t0, t1, t2)] << (3 * kDepth)) |
           ffv_morton((uint32_t)((g[0] - (t0 << (l - 1))) << sh),
                      (uint32_t)((g[1] - (t1 << (l - 1))) << sh),
                      (uint32_t)((g[2] - (t2 << (l - 1))) << sh));
  };
  auto key_of = [&](int64_t j) {
    const int l = L.lev[j];
    const int64_t g[3] = {((int64_t)L.tij[3 * j] << (l - 1)) + L.cij[3 * j],
                          ((int64_t)L.tij[3 * j + 1] << (l - 1)) + L.cij[3 * j + 1],
                          ((int64_t)L.tij[3 * j + 2] << (l - 1)) + L.cij[3 * j + 2]};
    return point_key(l, g);
  };
  // the new leaves' keys ascend in leaf order: the old leaves' did (the builder sorts them),
  // and a split's children or a merge's parent take the key range of what they replace.  The
  // keys are formed during the search, for the few leaves that search: the last leaf whose
  // key is not above pk
  auto find = [&](uint64_t pk) {
    int64_t lo = 0, hi = nn;  // the answer + 1 lies in [lo, hi]
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (key_of(mid) <= pk) lo = mid + 1;
      else hi = mid;
    }
    return lo - 1;
  };
  // an old leaf whose rows can be copied: kept, and no face neighbour splits or merges
  auto copyable = [&](int64_t c) {
    if (L.what[c] != 1) return false;
    const uint32_t info = m->info[c];
    for (int f = 0; f < 6; f++) {
      const uint32_t kind = ffv_face_kind(info, f);
      if (kind & FFV_FK_BC) continue;
      const int32_t s = m->nbr[6 * c + f];
      if (kind == FFV_FK_FINER) {
        for (int q = 0; q < 4; q++)
          if (L.what[m->sub[4 * (int64_t)s + q]] != 1) return false;
      } else if (L.what[s] != 1) {
        return false;
      }
    }
    return true;
  };

  std::vector<std::vector<int32_t>> csub(nth);
  std::vector<int> crc(nth, FFV_OK);
  std::vector<int> tmin(nth, FFV_MAX_LEVEL + 1), tmax(nth, 0);
  // per-thread results are kept in locals and stored once: the threads' slots share cache
  // lines, and writing them per leaf made every store a coherence miss
  parallel_chunks(nn, nth, [&](int t, int64_t a, int64_t b) {
    std::vector<int32_t> &sub = csub[t];
    int lmin = FFV_MAX_LEVEL + 1, lmax = 0, err = FFV_OK;
    for (int64_t j = a; j < b && err == FFV_OK; j++) {
      const int l = L.lev[j];
      lmin = std::min(lmin, l);
      lmax = std::max(lmax, l);
      const int64_t s = L.src[j];
      if (s >= 0 && copyable(s)) {  // the old rows, renumbered
        const uint32_t info = m->info[s];
        for (int f = 0; f < 6; f++) {
          const uint32_t kind = ffv_face_kind(info, f);
          const int32_t o = m->nbr[6 * s + f];
          int32_t slot = -1;
          if (kind == FFV_FK_FINER) {
            slot = (int32_t)(sub.size() / 4);  // shifted by the chunk's offset below
            for (int q = 0; q < 4; q++) sub.push_back((int32_t)L.old2new[m->sub[4 * (int64_t)o + q]]);
          } else if (!(kind & FFV_FK_BC)) {
            slot = (int32_t)L.old2new[o];
          }
          nm->nbr[6 * j + f] = slot;
        }
        nm->info[j] = info;
        continue;
      }
      uint32_t info = (uint32_t)l << 24;
      const int64_t gx[3] = {((int64_t)L.tij[3 * j] << (l - 1)) + L.cij[3 * j],
                             ((int64_t)L.tij[3 * j + 1] << (l - 1)) + L.cij[3 * j + 1],
                             ((int64_t)L.tij[3 * j + 2] << (l - 1)) + L.cij[3 * j + 2]};
      for (int f = 0; f < 6; f++) {
        const ffv_face_frame &fr = m->frame[f];
        const int ax = fr.side_axis;
        int64_t g[3] = {gx[0], gx[1], gx[2]};
        g[ax] += fr.side_dir;
        const int64_t ext = (int64_t)NT[ax] << (l - 1);
        uint32_t kind;
        int32_t slot = -1;
        if (g[ax] < 0 || g[ax] >= ext) {
          const int side = 2 * ax + (fr.side_dir > 0 ? 1 : 0);
          kind = FFV_FK_BC | (uint32_t)m->desc.bc[side];
        } else {
          const int64_t hit = find(point_key(l, g));
          const int lh = hit >= 0 ? L.lev[hit] : 0;
          if (lh == l) {
            kind = FFV_FK_SAME;
            slot = (int32_t)hit;
          } else if (lh == l - 1) {
            kind = FFV_FK_COARSER;
            slot = (int32_t)hit;
          } else if (lh > l) {
            // the region is refined (its first corner may lie deeper on the far side); the
            // four finer neighbours: subface k touches node ffv_face_nodes[f][k] of this face
            int32_t ids[4];
            for (int k = 0; k < 4 && err == FFV_OK; k++) {
              const int q = ffv_face_nodes[f][k];
              const int cb[3] = {ffv_corner_x(q), ffv_corner_y(q), ffv_corner_z(q)};
              int64_t fg[3];
              for (int d = 0; d < 3; d++)
                fg[d] = 2 * g[d] + (d == ax ? (fr.side_dir > 0 ? 0 : 1) : cb[d]);
              const int64_t h2 = find(point_key(l + 1, fg));
              if (h2 < 0 || L.lev[h2] != l + 1) err = FFV_ERR_BALANCE;
              ids[k] = (int32_t)h2;
            }
            if (err != FFV_OK) break;
            kind = FFV_FK_FINER;
            slot = (int32_t)(sub.size() / 4);
            sub.insert(sub.end(), ids, ids + 4);
          } else {
            err = FFV_ERR_BALANCE;
            break;
          }
        }
        info |= kind << (4 * f);
        nm->nbr[6 * j + f] = slot;
      }
      nm->info[j] = info;
    }
    crc[t] = err;
    tmin[t] = lmin;
    tmax[t] = lmax;
  });
  rc = FFV_OK;
  for (int t = 0; t < nth && rc == FFV_OK; t++) rc = crc[t];
  if (rc != FFV_OK) {
    ffv_mesh_free(nm);
    return rc;
  }
  // subface groups numbered in cell order: each chunk's groups shifted by the groups before
  // it (the chunks are parallel_chunks' over nn, as above)
  std::vector<size_t> off(nth + 1, 0);
  for (int t = 0; t < nth; t++) off[t + 1] = off[t] + csub[t].size();
  nm->nsub = (int32_t)(off[nth] / 4);
  nm->sub = (int32_t *)malloc(sizeof(int32_t) * (off[nth] ? off[nth] : 4));
  if (!nm->sub) {
    ffv_mesh_free(nm);
    return FFV_ERR_NOMEM;
  }
  parallel_chunks(nn, nth, [&](int t, int64_t a, int64_t b) {
    const int32_t shift = (int32_t)(off[t] / 4);
    if (shift)
      for (int64_t c = a; c < b; c++)
        for (int f = 0; f < 6; f++)
          if (ffv_face_kind(nm->info[c], f) == FFV_FK_FINER) nm->nbr[6 * c + f] += shift;
    if (!csub[t].empty()) memcpy(nm->sub + off[t], csub[t].data(), sizeof(int32_t) * csub[t].size());
  });
  nm->min_level = *std::min_element(tmin.begin(), tmin.end());
  nm->max_level = *std::max_element(tmax.begin(), tmax.end());
  if (nn == 0) nm->min_level = nm->max_level = 0;
  *out = nm;
  return FFV_OK;
}
