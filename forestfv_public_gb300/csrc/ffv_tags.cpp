// Host side of the refinement tags: the reference's 2:1 smoothing of the per-leaf target
// levels (criterionsmth.c:3-58), on the owner-sorted face tables.
//
// The reference sweeps its leaf list in order and updates `split` in place, so a leaf sees
// the values its predecessors already changed in the same sweep; the sweeps here keep that
// order (leaf order = the tables' cell order).  Siblings (the eight children of one parent
// octant) are consecutive in that order.
#include <stdint.h>
#include <stdlib.h>

#include <string.h>

#include <algorithm>
#include <functional>
#include <memory>
#include <queue>
#include <vector>

#include "ffv_internal.h"

extern "C" int ffv_tags_smooth(const ffv_mesh *m, int32_t level_max, int32_t *split) {
  if (!m || !split || level_max < 0) return FFV_ERR_ARG;
  const int64_t n = m->n;
  const int nth = host_threads();
  auto level = [&](int64_t c) { return (int32_t)ffv_info_level(m->info[c]); };
  // per-leaf byte arrays, filled in parallel (a value-initialised vector fills them, and
  // takes their first-touch page faults, on one thread)
  auto bytes = [&](uint8_t v) {
    std::unique_ptr<uint8_t[]> p(new uint8_t[n > 0 ? n : 1]);
    uint8_t *q = p.get();
    parallel_chunks(n, nth, [&](int, int64_t a, int64_t b) { memset(q + a, v, (size_t)(b - a)); });
    return p;
  };
  // a leaf's complete group of eight sibling leaves (first leaf, or -1), looked up once and
  // remembered as one byte (0 not looked up, 1 in a complete group, 2 not); each entry is
  // written only by the thread that evaluates its own leaf
  const std::unique_ptr<uint8_t[]> gknown_b = bytes(0);
  uint8_t *const gknown = gknown_b.get();
  auto group_of = [&](int64_t c) -> int64_t {
    const uint8_t f = gknown[c];
    if (f == 0) {
      const int64_t g = ffv_sibling_group(m, c);
      gknown[c] = g >= 0 ? 1 : 2;
      return g;
    }
    if (f == 2) return -1;
    const int32_t *x = m->cell_ijk + 3 * c;
    return c - (((x[0] & 1) << 1) | (x[1] & 1) | ((x[2] & 1) << 2));
  };
  // criterionsmth.c:14-33: a leaf coarsens only with all eight siblings, refines by one.
  // A leaf whose target is not below its level counts itself out of the eight, so its
  // sibling group is only looked up for targets below the level.
  auto rule1 = [&](int64_t c) {
    const int32_t l = level(c);
    int32_t v = split[c];
    if (l > 1 && v < l) {
      // only leaf children count (criterionsmth.c:19-21): a group with a refined sibling
      // cannot reach eight
      const int64_t g = group_of(c);
      int imerge = 0;
      if (g >= 0)
        for (int64_t q = g; q < g + 8; q++)
          if (split[q] < level(q)) imerge++;
      v = imerge == 8 ? l - 1 : l;
    }
    if (l < v) v = l + 1;
    return v;
  };
  // criterionsmth.c:37-51: at most one level below any face neighbour
  auto rule2 = [&](int64_t c) {
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
    return mx - split[c] > 1 ? mx - 1 : split[c];
  };
  // A sweep updates split in place in leaf order, each leaf seeing its predecessors' new
  // values.  The 2:1 rule's sweep runs as a worklist with the same result: the leaves are first evaluated on
  // the sweep's input in parallel, and those whose value would change are visited in leaf
  // order; when a visited leaf changes, the later leaves that read its value (its sibling
  // group for the coarsening rule, its face neighbours for the 2:1 rule) join the worklist.
  // A leaf never on the list sees, when the sweep reaches it, exactly the inputs of the
  // parallel evaluation, so its value does not change -- as in the full sweep.  Earlier
  // leaves that read a changed value are not revisited in this sweep (the full sweep has
  // passed them too); the next pass's evaluation finds them.  That evaluation visits only
  // "dirty" leaves: all at first, afterwards those one of whose inputs (their own value, a
  // sibling's or a face neighbour's, per rule) changed since they were last evaluated -- a
  // leaf found unchanged stays unchanged until then.  A sweep with no dirty leaf at all is
  // skipped (any1 / any2: some leaf of the rule is dirty).
  const std::unique_ptr<uint8_t[]> queued_b = bytes(0), dirty1_b = bytes(1), dirty2_b = bytes(1);
  uint8_t *const queued = queued_b.get(), *const dirty1 = dirty1_b.get(), *const dirty2 = dirty2_b.get();
  bool any1 = true, any2 = true;
  // the readers of split[c]: c itself and, for the coarsening rule, its siblings (which
  // read only whether split[c] is below the level: `flipped`), for the 2:1 rule its face
  // neighbours
  auto mark_deps = [&](int64_t c, bool siblings, bool flipped, auto &&fn) {
    fn(c);
    if (siblings) {
      if (!flipped) return;
      const int64_t g = group_of(c);
      if (g >= 0)
        for (int64_t q = g; q < g + 8; q++) fn(q);
    } else {
      const uint32_t info = m->info[c];
      for (int f = 0; f < 6; f++) {
        const uint32_t kind = ffv_face_kind(info, f);
        if (kind & FFV_FK_BC) continue;
        const int32_t s = m->nbr[6 * c + f];
        if (kind == FFV_FK_FINER) {
          for (int q = 0; q < 4; q++) fn(m->sub[4 * (int64_t)s + q]);
        } else {
          fn(s);
        }
      }
    }
  };
  auto sweep = [&](auto rule, bool sibling_deps, uint8_t *dirty, bool &any, uint8_t *dirty_other,
                   bool &any_other) -> bool {
    if (!any) return false;
    any = false;
    std::vector<std::vector<int64_t>> found(nth);
    parallel_chunks(n, nth, [&](int t, int64_t a, int64_t b) {
      for (int64_t c = a; c < b; c++) {
        if (!dirty[c]) continue;
        dirty[c] = 0;
        if (rule(c) != split[c]) found[t].push_back(c);
      }
    });
    std::priority_queue<int64_t, std::vector<int64_t>, std::greater<int64_t>> work;
    for (auto &v : found)
      for (int64_t c : v) {
        work.push(c);
        queued[c] = 1;
      }
    if (work.empty()) return false;
    while (!work.empty()) {
      const int64_t c = work.top();
      work.pop();
      queued[c] = 0;
      const int32_t v = rule(c);
      if (v == split[c]) continue;
      const int32_t lc = level(c);
      const bool flipped = (split[c] < lc) != (v < lc);
      split[c] = v;
      // this rule's readers of split[c]: later ones in this sweep, earlier ones (and c
      // itself, whose rule reads its own value) in the next pass
      mark_deps(c, sibling_deps, flipped, [&](int64_t d) {
        if (d > c) {
          if (!queued[d]) {
            queued[d] = 1;
            work.push(d);
          }
        } else {
          dirty[d] = 1;
          any = true;
        }
      });
      // the other rule's readers: at its next sweep
      mark_deps(c, !sibling_deps, flipped, [&](int64_t d) { dirty_other[d] = 1; });
      any_other = true;
    }
    return true;
  };
  // The coarsening rule reads only the leaf's own sibling group, and a group's eight leaves
  // are consecutive in leaf order: its in-order sweep is the groups' own in-order sweeps,
  // independent of one another.  It runs in parallel over chunks that start and end on group
  // boundaries, each group in order.  A leaf's rule only reads its group when some leaf of
  // the eight is below its level; otherwise the leaves are swept one by one.  A group that
  // changed is evaluated again at the next pass (its earlier leaves read the later ones' old
  // values), one that did not is a fixed point until an input changes.
  auto align = [&](int64_t x) -> int64_t {
    if (x <= 0 || x >= n) return x;
    const int64_t g = ffv_sibling_group(m, x);
    return g >= 0 ? g : x;
  };
  // 1 + the pass in which the coarsening rule last changed the leaf, modulo 256 (a stale
  // equal value after 256 passes would only make a leaf dirty that need not be)
  const std::unique_ptr<uint8_t[]> changed_in_b = bytes(0);
  uint8_t *const changed_in = changed_in_b.get();
  std::vector<std::vector<int64_t>> chg(nth);  // the leaves each thread's sweep changed
  auto sweep1 = [&](int32_t pass) -> bool {
    if (!any1) return false;
    any1 = false;
    parallel_chunks(n, nth, [&](int t, int64_t a, int64_t b) {
      a = align(a);
      b = align(b);
      chg[t].clear();
      auto visit = [&](int64_t c) -> bool {
        const int32_t v = rule1(c);
        if (v == split[c]) return false;
        split[c] = v;
        changed_in[c] = (uint8_t)(pass + 1);
        chg[t].push_back(c);
        return true;
      };
      for (int64_t c = a; c < b;) {
        const int32_t *x = m->cell_ijk + 3 * c;
        bool below = false;
        if ((x[0] & 1) == 0 && (x[1] & 1) == 0 && (x[2] & 1) == 0 && c + 8 <= b)
          for (int64_t q = c; q < c + 8 && !below; q++) below = split[q] < level(q);
        if (below && group_of(c) == c) {
          bool dirty = false;
          for (int64_t q = c; q < c + 8; q++) dirty = dirty || dirty1[q];
          if (dirty) {
            bool ch = false;
            for (int64_t q = c; q < c + 8; q++) {
              dirty1[q] = 0;
              ch = visit(q) || ch;
            }
            if (ch)
              for (int64_t q = c; q < c + 8; q++) dirty1[q] = 1;
          }
          c += 8;
        } else {
          if (dirty1[c]) {
            dirty1[c] = 0;
            visit(c);
          }
          c++;
        }
      }
    });
    size_t nchg = 0;
    for (int t = 0; t < nth; t++) nchg += chg[t].size();
    if (nchg == 0) return false;
    any1 = true;  // the groups that changed were marked dirty again
    any2 = true;  // and their leaves' face neighbours, below
    // the 2:1 rule's readers of a changed leaf: itself and its face neighbours -- marked
    // from the lists when they are short, else gathered by each reader over all leaves (the
    // face relation is symmetric)
    if ((int64_t)nchg * 16 < n) {
      for (int t = 0; t < nth; t++)
        for (int64_t c : chg[t]) mark_deps(c, false, false, [&](int64_t d) { dirty2[d] = 1; });
      return true;
    }
    parallel_chunks(n, nth, [&](int, int64_t a, int64_t b) {
      for (int64_t c = a; c < b; c++) {
        const uint8_t mark = (uint8_t)(pass + 1);
        bool hit = changed_in[c] == mark;
        const uint32_t info = m->info[c];
        for (int f = 0; f < 6 && !hit; f++) {
          const uint32_t kind = ffv_face_kind(info, f);
          if (kind & FFV_FK_BC) continue;
          const int32_t s = m->nbr[6 * c + f];
          if (kind == FFV_FK_FINER) {
            for (int q = 0; q < 4; q++) hit = hit || changed_in[m->sub[4 * (int64_t)s + q]] == mark;
          } else {
            hit = changed_in[s] == mark;
          }
        }
        if (hit) dirty2[c] = 1;
      }
    });
    return true;
  };
  // A pass is a function of `split` alone: once one changes nothing, every later pass
  // would see the same input and change nothing either, so the passes end there.
  for (int32_t pass = 0; pass < level_max + 1; pass++) {
    const bool c1 = sweep1(pass);
    const bool c2 = sweep(rule2, false, dirty2, any2, dirty1, any1);
    if (!c1 && !c2) break;
  }
  return FFV_OK;
}

// what one refineh pass (ffv_adapt) would do with these targets: leaves that split, and
// complete groups of eight sibling leaves that merge (refineh.c:10-57)
extern "C" int ffv_adapt_changes(const ffv_mesh *m, const int32_t *split, int64_t *nsplit,
                                 int64_t *nmerge) {
  if (!m || !split || !nsplit || !nmerge) return FFV_ERR_ARG;
  const int nth = host_threads();
  std::vector<int64_t> ns(nth, 0), nm(nth, 0);
  parallel_chunks(m->n, nth, [&](int t, int64_t a, int64_t b) {
    int64_t s_ = 0, m_ = 0;  // counted in locals: the threads' slots share cache lines
    for (int64_t c = a; c < b; c++) {
      const int32_t l = (int32_t)ffv_info_level(m->info[c]);
      if (split[c] > l) s_++;
      // a group merges only if its first leaf (like all eight) wants a coarser level: the
      // group is looked up only then
      if (l > 1 && split[c] < l && ffv_sibling_group(m, c) == c) {
        bool all = true;
        for (int q = 0; q < 8 && all; q++) all = split[c + q] < l;
        m_ += all ? 1 : 0;
      }
    }
    ns[t] = s_;
    nm[t] = m_;
  });
  *nsplit = 0;
  *nmerge = 0;
  for (int t = 0; t < nth; t++) {
    *nsplit += ns[t];
    *nmerge += nm[t];
  }
  return FFV_OK;
}
