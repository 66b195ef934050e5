// Checks of the host thread pool (spearfish_gb300/csrc/sf_hostpool.h), built and run by
// tests/test_hostpool.py on the CPU: every index of [0, n) is visited once, chunks are
// contiguous and numbered as chunks_for says, the same arguments give the same chunks, and
// several threads may split work over the pool at once (the pool's workers serve them all).
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "sf_hostpool.h"

using sfe::chunks_for;
using sfe::parallel_chunks;

static int check_cover(size_t n, size_t min_per, int max_t) {
  std::vector<std::atomic<int>> seen(n);
  for (auto& s : seen) s.store(0);
  std::vector<std::pair<size_t, size_t>> range(max_t + 1, {SIZE_MAX, 0});
  std::vector<std::atomic<int>> calls(max_t + 1);
  for (auto& c : calls) c.store(0);
  parallel_chunks(n, min_per, max_t, [&](size_t b, size_t e, int k) {
    if (k < 0 || k > max_t) return;
    calls[k]++;
    range[k] = {b, e};
    for (size_t q = b; q < e; ++q) seen[q]++;
  });
  for (size_t q = 0; q < n; ++q)
    if (seen[q].load() != 1) {
      std::printf("FAIL cover n=%zu min=%zu t=%d: index %zu seen %d times\n", n, min_per, max_t, q,
                  seen[q].load());
      return 1;
    }
  const size_t t = chunks_for(n, min_per, max_t);
  size_t at = 0;
  for (size_t k = 0; k < t; ++k) {
    if (calls[k].load() != 1 || range[k].first != at) {
      std::printf("FAIL chunks n=%zu min=%zu t=%d: chunk %zu\n", n, min_per, max_t, k);
      return 1;
    }
    at = range[k].second;
  }
  for (int k = (int)t; k <= max_t; ++k)
    if (calls[k].load() != 0) {
      std::printf("FAIL extra chunk %d (t=%zu)\n", k, t);
      return 1;
    }
  if (n > 0 && at != n) {
    std::printf("FAIL chunks end at %zu of %zu\n", at, n);
    return 1;
  }
  return 0;
}

int main() {
  int bad = 0;
  const size_t sizes[] = {0, 1, 2, 7, 2047, 2048, 4095, 4096, 4097, 10001, 16411, 65536, 200003};
  for (size_t n : sizes)
    for (size_t min_per : {size_t(0), size_t(1), size_t(2048), size_t(4096)})
      for (int t : {1, 2, 8}) bad |= check_cover(n, min_per, t);
  // The same arguments give the same chunks.
  for (int rep = 0; rep < 3; ++rep) {
    std::vector<size_t> a(9, SIZE_MAX), b(9, SIZE_MAX);
    parallel_chunks(100000, 2048, 8, [&](size_t s, size_t, int k) { a[k] = s; });
    parallel_chunks(100000, 2048, 8, [&](size_t s, size_t, int k) { b[k] = s; });
    if (a != b) {
      std::printf("FAIL chunks differ between calls\n");
      bad = 1;
    }
  }
  // Four threads split work over the pool at once, many times over.
  std::atomic<int> fails{0};
  std::vector<std::thread> th;
  for (int w = 0; w < 4; ++w)
    th.emplace_back([&, w] {
      for (int it = 0; it < 300; ++it) {
        const size_t n = 4096 + 977 * (size_t)((w * 31 + it) % 40);
        std::atomic<uint64_t> sum{0};
        parallel_chunks(n, 1024, 8, [&](size_t b, size_t e, int) {
          uint64_t s = 0;
          for (size_t q = b; q < e; ++q) s += q;
          sum += s;
        });
        if (sum.load() != (uint64_t)n * (n - 1) / 2) fails++;
      }
    });
  for (auto& t : th) t.join();
  if (fails.load()) {
    std::printf("FAIL concurrent callers: %d wrong sums\n", fails.load());
    bad = 1;
  }
  std::printf(bad ? "FAILED\n" : "OK workers=%zu\n", sfe::HostPool::get().workers());
  return bad;
}
