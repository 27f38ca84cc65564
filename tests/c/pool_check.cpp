// Host check of parallel_chunks and its persistent worker pool (ffv_internal.h): every
// element of large loops visited exactly once, loops nested inside loops, two threads
// running loops at the same time, and a child process forked after the workers started
// (the pool declines there and the loop starts its own threads).  Exits nonzero on a wrong
// count; a deadlock shows as the test's timeout.
#include <sys/wait.h>
#include <unistd.h>

#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "ffv_internal.h"

static int check_loop(int64_t n, int nth) {
  std::vector<std::atomic<int>> hit(n);
  for (auto &h : hit) h.store(0);
  parallel_chunks(n, nth, [&](int, int64_t a, int64_t b) {
    for (int64_t i = a; i < b; i++) hit[i].fetch_add(1);
  });
  for (int64_t i = 0; i < n; i++)
    if (hit[i].load() != 1) return 1;
  return 0;
}

int main() {
  const int nth = host_threads();
  const int64_t big = (int64_t)3 << 20;  // above the pool's threshold
  int bad = 0;
  for (int rep = 0; rep < 20; rep++) bad += check_loop(big + rep, nth);
  bad += check_loop(1000, nth);  // below the threshold: threads started per loop
  // nested: the inner loops run inside the pool's loop (the pool declines them)
  std::atomic<int64_t> total{0};
  parallel_chunks(big, nth, [&](int t, int64_t a, int64_t b) {
    if (t == 0) {
      std::atomic<int64_t> inner{0};
      parallel_chunks(big, nth, [&](int, int64_t x, int64_t y) { inner += y - x; });
      if (inner.load() != big) total += 1 << 30;
    }
    total += b - a;
  });
  if (total.load() != big) bad++;
  // two callers at once: one gets the pool, the other starts threads of its own
  std::vector<std::thread> callers;
  std::atomic<int> cbad{0};
  for (int k = 0; k < 2; k++)
    callers.emplace_back([&] {
      for (int rep = 0; rep < 10; rep++) cbad += check_loop(big, nth);
    });
  for (auto &c : callers) c.join();
  bad += cbad.load();
  // a child forked after the workers started
  fflush(stdout);
  const pid_t pid = fork();
  if (pid == 0) _exit(check_loop(big, nth) ? 3 : 0);
  int status = 0;
  waitpid(pid, &status, 0);
  if (!WIFEXITED(status) || WEXITSTATUS(status) != 0) bad++;
  printf("%d threads: %d failures\n", nth, bad);
  return bad ? 1 : 0;
}
