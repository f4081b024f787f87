// host_pool.h -- independent pieces of host-driven GPU work run side by side:
// fn(i, stream) for every i < n on up to `workers` host threads, each with a
// stream of its own, so that one piece's synchronisations and launches overlap
// another's kernels.  Every stream is synchronised before the call returns.
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace dmsc {

// Returns 0, or the first nonzero result of fn (the remaining pieces are
// then skipped); -1 when a stream could not be created.
template <class F>
int for_each_on_streams(int device, int n, int workers, F fn) {
  std::atomic<int> next{0}, rc{0};
  auto work = [&] {
    cudaSetDevice(device);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      int z = 0;
      rc.compare_exchange_strong(z, -1);
      return;
    }
    for (int i; rc.load() == 0 && (i = next.fetch_add(1)) < n;) {
      const int r = fn(i, s);
      if (r != 0) {
        int z = 0;
        rc.compare_exchange_strong(z, r);
      }
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  };
  const int k = std::max(1, std::min(workers, n));
  std::vector<std::thread> th;
  for (int t = 1; t < k; ++t) th.emplace_back(work);
  work();
  for (auto &t : th) t.join();
  return rc.load();
}

}  // namespace dmsc
