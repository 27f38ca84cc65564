// Internal declarations shared by the mesh builder (host C++) and the device code.
#pragma once
#include <stdint.h>

#include "../../include/ffv.h"

#ifdef __CUDACC__
#define FFV_HD __host__ __device__
#else
#define FFV_HD
#endif

// Face kinds, 4 bits per face in a cell's info word (bits 4f..4f+3); level in bits 24..31.
#define FFV_FK_SAME 0u     // one neighbour, same level (1:1 face)
#define FFV_FK_COARSER 1u  // one neighbour, one level coarser (this cell is the fine side)
#define FFV_FK_FINER 2u    // four neighbours, one level finer (subfaces)
#define FFV_FK_BC 8u       // boundary: 8 | bc code

FFV_HD static inline uint32_t ffv_face_kind(uint32_t info, int f) { return (info >> (4 * f)) & 15u; }
FFV_HD static inline int ffv_info_level(uint32_t info) { return (int)(info >> 24); }

// Hex corner k of a tree or child sits at (x, y, z) = (bit1(k), bit0(k), bit2(k)).  This is
// the node order under which the reference's face normals (normalvector.c:23-29 applied to
// the face-node table operatetp.c:64-69) point into the cell and its six-tet volume
// (meshproperties.c:83-123) comes out negative -- the handedness its update
// S = SN - DT/Vol*RHS needs to be upwind.  Child index = corner index (split.c:69-93).
static inline int ffv_corner_x(int k) { return (k >> 1) & 1; }
static inline int ffv_corner_y(int k) { return k & 1; }
static inline int ffv_corner_z(int k) { return (k >> 2) & 1; }

// Face f of a hex: its four nodes (operatetp.c:64-69, typ 0) and opposite face
// (operatetp.c:268-279, fcopp).
static const int ffv_face_nodes[6][4] = {{0, 1, 5, 4}, {3, 7, 5, 1}, {2, 6, 7, 3},
                                         {2, 0, 4, 6}, {2, 3, 1, 0}, {6, 4, 5, 7}};
static const int ffv_face_opp[6] = {2, 3, 0, 1, 5, 4};

// Per-face frame for the Cartesian forest, derived by the builder from the reference's
// normal/tangent formulas: component `axis` of the vector times `sign` (+1/-1).
struct ffv_face_frame {
  int8_t n_axis, n_sign, t1_axis, t1_sign, t2_axis, t2_sign;
  int8_t side_axis, side_dir;  // domain axis this face looks along, and -1 / +1
};

struct ffv_level_geom {
  double h;          // cell edge
  double vol;        // signed volume as meshproperties.c:76-124 computes it
  double area;       // face area as meshproperties.c:42-73 computes it
  double inv_unused;
};

// first cell of the complete group of eight sibling leaves that holds cell c, or -1 when
// some sibling is not a leaf (then the group is not in the table).  In the tables' cell
// order (depth-first by child index) the eight children of a parent are consecutive, and
// child k of a parent sits at cell coordinates 2p + (bit1 k, bit0 k, bit2 k).
// Morton key whose base-8 digits are child indices (corner bit k: x = bit1, y = bit0,
// z = bit2), so that sorting by it reproduces the depth-first child order; 21 bits a lane
static inline uint64_t ffv_spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffffULL;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}
static inline uint64_t ffv_morton(uint32_t x, uint32_t y, uint32_t z) {
  return (ffv_spread3(x) << 1) | ffv_spread3(y) | (ffv_spread3(z) << 2);
}

struct ffv_mesh;
int64_t ffv_sibling_group(const ffv_mesh *m, int64_t c);

#ifdef __cplusplus
#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

inline int host_threads() {
  return (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
}

// Worker threads kept for the process's lifetime, so that a parallel loop does not pay for
// starting and joining its threads (~15 us each): a regrid runs dozens of short loops.
// run(n, fn) calls fn(0) on the calling thread and fn(1..n-1) on workers, and returns once
// all have finished.  It declines (returns false, the caller then starts threads of its own)
// when the pool is busy with another caller's loop, when called from inside a loop, when n
// exceeds its workers, or in a child process forked after the workers started (they do not
// exist there).  The pool is never destroyed: its threads wait on a condition variable and
// end with the process.
class HostPool {
 public:
  static HostPool &instance() {
    static HostPool *p = new HostPool();
    return *p;
  }
  bool run(int n, const std::function<void(int)> &fn) {
    if (n < 2 || in_loop() || getpid() != pid_ || n - 1 > (int)workers_.size()) return false;
    std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
    if (!busy.owns_lock()) return false;
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &fn;
      last_ = n - 1;
      remaining_ = n - 1;
      ++gen_;
    }
    cv_.notify_all();
    in_loop() = true;
    fn(0);
    in_loop() = false;
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return remaining_ == 0; });
    job_ = nullptr;
    return true;
  }

 private:
  HostPool() : pid_(getpid()) {
    for (int t = 1; t < host_threads(); t++) workers_.emplace_back([this, t] { loop(t); });
  }
  static bool &in_loop() {
    static thread_local bool f = false;
    return f;
  }
  void loop(int t) {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(int)> *job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (t > last_) continue;  // not one of this loop's threads
        job = job_;
      }
      in_loop() = true;
      (*job)(t);
      in_loop() = false;
      std::lock_guard<std::mutex> lk(mu_);
      if (--remaining_ == 0) done_.notify_one();
    }
  }
  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)> *job_ = nullptr;
  int last_ = 0, remaining_ = 0;
  uint64_t gen_ = 0;
};

// fn(thread, begin, end) on nthreads contiguous chunks of [0, n), the calling thread taking
// the first.  Loops over at least 2^20 elements run on the pool's workers when it takes them
// (the pool is created by the first such loop: a process that only ever runs small meshes
// keeps no idle threads), others on threads started here.
template <typename Fn>
inline void parallel_chunks(int64_t n, int nthreads, Fn fn) {
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  auto part = [&](int t) { fn(t, std::min(n, t * chunk), std::min(n, (t + 1) * chunk)); };
  if (nthreads < 2) {
    part(0);
    return;
  }
  if (n >= ((int64_t)1 << 20) && HostPool::instance().run(nthreads, std::function<void(int)>(part)))
    return;
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; t++) pool.emplace_back([&, t] { part(t); });
  part(0);
  for (auto &th : pool) th.join();
}
#endif

struct ffv_mesh {
  ffv_forest_desc desc;
  int64_t n;
  int32_t nsub;         // number of 4-subface groups
  int32_t min_level, max_level;
  uint32_t *info;       // [n]
  int32_t *nbr;         // [6n]: neighbour cell (kinds 0,1), subface group (kind 2), -1
  int32_t *sub;         // [4 nsub]
  int32_t *tree_ijk;    // [3n] canonical order
  int32_t *cell_ijk;    // [3n]
  ffv_face_frame frame[6];
  ffv_level_geom geom[FFV_MAX_LEVEL + 2];
};
