// gpu_sa.cu -- suffix array of a DNA text on the GPU, for the index builder.
//
// Prefix doubling: every suffix starts with a 64-bit key packing its first 21
// symbols (3 bits each, 0 past the end, so the terminator sorts first), then
// each round sorts (rank of the first h symbols, rank of the next h) pairs
// with a device radix sort, renumbers the groups of equal keys by a scan and
// doubles h, until every suffix has its own group.  The result is the unique
// suffix array of X followed by the terminator, the same array the host
// SA-IS (sais.hpp) returns, so every table derived from it -- and every index
// file -- is byte-identical.  A 3.1 Gbp genome takes about 100 GB of device
// memory (two key and two index buffers, ranks, group ids).
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdint>
#include <string>

#include "gpu_sa.hpp"
#include "kernels.cuh"

namespace hpgbwt {

namespace {

constexpr int kPack = 21;  // symbols in the first key (3 bits each)

__global__ void init_keys_kernel(const uint8_t* __restrict__ X, uint64_t n, uint64_t* __restrict__ key,
                                 uint32_t* __restrict__ idx) {
  const uint64_t N = n + 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t k = 0;
    for (int t = 0; t < kPack; ++t) {
      const uint64_t p = i + t;
      k = (k << 3) | (p < n ? (uint64_t)(X[p] & 3u) + 1u : 0u);
    }
    key[i] = k;
    idx[i] = (uint32_t)i;
  }
}

// head[j] = 1 where sorted key j starts a new group.
__global__ void heads_kernel(const uint64_t* __restrict__ key, uint64_t N, uint32_t* __restrict__ head) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (uint64_t)gridDim.x * blockDim.x)
    head[j] = (j == 0 || key[j] != key[j - 1]) ? 1u : 0u;
}

// rank[idx[j]] = group number (1-based) of sorted position j.
__global__ void scatter_rank_kernel(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ group, uint64_t N,
                                    uint32_t* __restrict__ rank) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (uint64_t)gridDim.x * blockDim.x)
    rank[idx[j]] = group[j];
}

// Next round's key of every suffix: (rank of its first h symbols, rank of the
// h after them; 0 once they start past the terminator).
__global__ void pair_keys_kernel(const uint32_t* __restrict__ rank, uint64_t N, uint64_t h, uint64_t* __restrict__ key,
                                 uint32_t* __restrict__ idx) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    key[i] = ((uint64_t)rank[i] << 32) | (i + h < N ? rank[i + h] : 0u);
    idx[i] = (uint32_t)i;
  }
}

struct DevArrays {
  void* p[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  ~DevArrays() {
    for (void* q : p) cudaFree(q);
  }
};

int bits_for(uint64_t v) {
  int b = 0;
  while (b < 64 && (v >> b)) ++b;
  return b;
}

}  // namespace

int gpu_suffix_array(const uint8_t* X, uint64_t n, int device, uint32_t* sa, std::string* err) {
  const uint64_t N = n + 1;
  if (N >= 0xFFFFFFFFull) {
    *err = "genome too large for 32-bit suffix-array entries";
    return -1;
  }
  auto fail = [&](const char* what, cudaError_t ce) {
    *err = std::string("GPU suffix array: ") + what + ": " + cudaGetErrorString(ce);
    cudaGetLastError();
    return -1;
  };
  cudaError_t ce;
  if ((ce = cudaSetDevice(device)) != cudaSuccess) return fail("cudaSetDevice", ce);
  cudaStream_t s;
  if ((ce = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", ce);
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  DevArrays a;
  uint8_t* dX = nullptr;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *i0 = nullptr, *i1 = nullptr, *rank = nullptr, *group = nullptr;
  if ((ce = cudaMalloc(&a.p[0], n ? n : 1)) != cudaSuccess || (ce = cudaMalloc(&a.p[1], N * 8)) != cudaSuccess ||
      (ce = cudaMalloc(&a.p[2], N * 8)) != cudaSuccess || (ce = cudaMalloc(&a.p[3], N * 4)) != cudaSuccess ||
      (ce = cudaMalloc(&a.p[4], N * 4)) != cudaSuccess || (ce = cudaMalloc(&a.p[5], N * 4)) != cudaSuccess ||
      (ce = cudaMalloc(&a.p[6], N * 4)) != cudaSuccess)
    return fail("out of device memory", ce);
  dX = static_cast<uint8_t*>(a.p[0]);
  k0 = static_cast<uint64_t*>(a.p[1]);
  k1 = static_cast<uint64_t*>(a.p[2]);
  i0 = static_cast<uint32_t*>(a.p[3]);
  i1 = static_cast<uint32_t*>(a.p[4]);
  rank = static_cast<uint32_t*>(a.p[5]);
  group = static_cast<uint32_t*>(a.p[6]);
  if (n && (ce = cudaMemcpyAsync(dX, X, n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail("upload text", ce);

  // temporary storage for the sort and the scan (sized for the largest call)
  size_t sort_bytes = 0, scan_bytes = 0;
  {
    cub::DoubleBuffer<uint64_t> K(k0, k1);
    cub::DoubleBuffer<uint32_t> V(i0, i1);
    if ((ce = cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, K, V, (int64_t)N, 0, 64, s)) != cudaSuccess)
      return fail("sort size", ce);
    if ((ce = cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, group, group, (int64_t)N, s)) != cudaSuccess)
      return fail("scan size", ce);
  }
  if ((ce = cudaMalloc(&a.p[7], std::max(sort_bytes, scan_bytes))) != cudaSuccess)
    return fail("out of device memory (sort)", ce);
  void* tmp = a.p[7];
  const unsigned grid = 152u * 32u;

  count_launches(1);
  init_keys_kernel<<<grid, 256, 0, s>>>(dX, n, k0, i0);
  int end_bit = 3 * kPack;
  uint64_t h = kPack;
  uint32_t* sorted_idx = i0;
  for (int round = 0; round < 64; ++round) {
    cub::DoubleBuffer<uint64_t> K(k0, k1);
    cub::DoubleBuffer<uint32_t> V(i0, i1);
    size_t tb = sort_bytes;
    if ((ce = cub::DeviceRadixSort::SortPairs(tmp, tb, K, V, (int64_t)N, 0, end_bit, s)) != cudaSuccess)
      return fail("sort", ce);
    count_launches(1);
    heads_kernel<<<grid, 256, 0, s>>>(K.Current(), N, group);
    tb = scan_bytes;
    if ((ce = cub::DeviceScan::InclusiveSum(tmp, tb, group, group, (int64_t)N, s)) != cudaSuccess)
      return fail("scan", ce);
    uint32_t groups = 0;
    if ((ce = cudaMemcpyAsync(&groups, group + (N - 1), 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail("group count", ce);
    sorted_idx = V.Current();
    if ((uint64_t)groups == N) break;  // every suffix is in its own group: the order is final
    count_launches(1);
    scatter_rank_kernel<<<grid, 256, 0, s>>>(sorted_idx, group, N, rank);
    // the next round's keys and indices overwrite this round's sorted ones,
    // which are no longer needed once the ranks are scattered
    k0 = K.Current();
    k1 = K.Alternate();
    i0 = V.Current();
    i1 = V.Alternate();
    count_launches(1);
    pair_keys_kernel<<<grid, 256, 0, s>>>(rank, N, h, k0, i0);
    end_bit = 32 + bits_for(groups);
    h *= 2;
    if (round == 63) {
      *err = "GPU suffix array: prefix doubling did not converge";
      return -1;
    }
  }
  if ((ce = cudaMemcpyAsync(sa, sorted_idx, N * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (ce = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail("download", ce);
  return 0;
}

}  // namespace hpgbwt
