// Host side of the refinement tags: the reference's 2:1 smoothing of the per-leaf target
// levels (criterionsmth.c:3-58), on the owner-sorted face tables.
//
// The reference sweeps its leaf list in order and updates `split` in place, so a leaf sees
// the values its predecessors already changed in the same sweep; the sweeps here keep that
// order (leaf order = the tables' cell order).  Siblings (the eight children of one parent
// octant) are the leaves of one tree with the same level and the same parent coordinates.
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <unordered_map>
#include <vector>

#include "ffv_internal.h"

extern "C" int ffv_tags_smooth(const ffv_mesh *m, int32_t level_max, int32_t *split) {
  if (!m || !split || level_max < 0) return FFV_ERR_ARG;
  const int64_t n = m->n;
  // sibling groups: key = (tree, level, parent coordinates)
  std::vector<int64_t> group(n, -1);
  std::vector<int32_t> gcount;
  std::vector<int64_t> gfirst;  // members of a group, as a linked list through gnext
  std::vector<int64_t> gnext(n, -1);
  {
    struct Key {
      uint64_t a, b;
      bool operator==(const Key &o) const { return a == o.a && b == o.b; }
    };
    struct KeyHash {
      size_t operator()(const Key &k) const {
        return (size_t)(k.a * 0x9E3779B97F4A7C15ull ^ (k.b + 0x632BE59BD9B4E019ull + (k.a << 6)));
      }
    };
    std::unordered_map<Key, int64_t, KeyHash> key_to_group;
    key_to_group.reserve((size_t)n);
    const uint64_t nt0 = (uint64_t)m->desc.ntrees[0], nt1 = (uint64_t)m->desc.ntrees[1];
    for (int64_t c = 0; c < n; c++) {
      const int l = ffv_info_level(m->info[c]);
      if (l <= 1) continue;
      const int32_t *t = m->tree_ijk + 3 * c, *x = m->cell_ijk + 3 * c;
      const uint64_t tree = (uint64_t)t[0] + nt0 * ((uint64_t)t[1] + nt1 * (uint64_t)t[2]);
      const Key key{tree | ((uint64_t)l << 48),
                    (uint64_t)(x[0] >> 1) | ((uint64_t)(x[1] >> 1) << 21) |
                        ((uint64_t)(x[2] >> 1) << 42)};
      auto it = key_to_group.find(key);
      int64_t g;
      if (it == key_to_group.end()) {
        g = (int64_t)gcount.size();
        key_to_group.emplace(key, g);
        gcount.push_back(0);
        gfirst.push_back(-1);
      } else {
        g = it->second;
      }
      group[c] = g;
      gnext[c] = gfirst[g];
      gfirst[g] = c;
      gcount[g]++;
    }
  }
  auto level = [&](int64_t c) { return (int32_t)ffv_info_level(m->info[c]); };
  for (int32_t pass = 0; pass < level_max + 1; pass++) {
    // criterionsmth.c:14-33: a leaf coarsens only with all eight siblings, refines by one
    for (int64_t c = 0; c < n; c++) {
      const int32_t l = level(c);
      if (l > 1) {
        const int64_t g = group[c];
        int imerge = 0;
        for (int64_t k = gfirst[g]; k >= 0; k = gnext[k])
          if (split[k] < level(k)) imerge++;
        if (imerge == 8) split[c] = l - 1;
        else if (l > split[c]) split[c] = l;
      }
      if (l < split[c]) split[c] = l + 1;
    }
    // criterionsmth.c:37-51: at most one level below any face neighbour
    for (int64_t c = 0; c < n; c++) {
      int32_t mx = 1;
      const uint32_t info = m->info[c];
      for (int f = 0; f < 6; f++) {
        const uint32_t kind = ffv_face_kind(info, f);
        if (kind & FFV_FK_BC) continue;
        const int32_t s = m->nbr[6 * c + f];
        if (kind == FFV_FK_FINER) {
          for (int q = 0; q < 4; q++) mx = std::max(split[m->sub[4 * (int64_t)s + q]], mx);
        } else {
          mx = std::max(split[s], mx);
        }
      }
      if (mx - split[c] > 1) split[c] = mx - 1;
    }
  }
  return FFV_OK;
}
