// host_pool.cpp -- reusable page-locked host blocks for result sets.
//
// A result set's arrays are written by device-to-host copies.  Into freshly
// malloc'ed memory those copies first fault every page in; into page-locked
// blocks kept across calls they run at the link's full rate.  Blocks freed
// through host_pool_free go back to a size-ordered free list (up to a cap) for
// the next result set; small arrays stay on malloc.
#include "host_pool.hpp"

#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>

namespace hpgbwt {

namespace {

constexpr size_t kSmall = 1u << 20;         // below this: plain malloc
constexpr size_t kRound = 2u << 20;         // page-locked blocks in 2 MiB steps
constexpr size_t kKeep = 8ull << 30;        // free bytes kept for reuse

struct Pool {
  std::mutex mu;
  std::unordered_map<void*, size_t> live;   // page-locked block -> size
  std::multimap<size_t, void*> idle;        // size -> free page-locked block
  size_t idle_bytes = 0;
};

Pool& pool() {
  static Pool* p = new Pool();  // never destroyed: blocks may outlive static teardown
  return *p;
}

}  // namespace

void* host_pool_alloc(size_t bytes) {
  if (bytes < kSmall) return std::malloc(bytes ? bytes : 1);
  Pool& P = pool();
  {
    std::lock_guard<std::mutex> lk(P.mu);
    auto it = P.idle.lower_bound(bytes);
    if (it != P.idle.end() && it->first <= 4 * bytes + kRound) {
      void* q = it->second;
      P.live[q] = it->first;
      P.idle_bytes -= it->first;
      P.idle.erase(it);
      return q;
    }
  }
  const size_t size = (bytes + kRound - 1) / kRound * kRound;
  void* q = nullptr;
  if (cudaHostAlloc(&q, size, cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    return std::malloc(bytes);
  }
  std::lock_guard<std::mutex> lk(P.mu);
  P.live[q] = size;
  return q;
}

void host_pool_free(void* q) {
  if (!q) return;
  Pool& P = pool();
  std::unique_lock<std::mutex> lk(P.mu);
  auto it = P.live.find(q);
  if (it == P.live.end()) {
    lk.unlock();
    std::free(q);
    return;
  }
  const size_t size = it->second;
  P.live.erase(it);
  if (P.idle_bytes + size <= kKeep) {
    P.idle.emplace(size, q);
    P.idle_bytes += size;
    return;
  }
  lk.unlock();
  cudaFreeHost(q);
}

}  // namespace hpgbwt
