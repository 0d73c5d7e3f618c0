// gather_bench.cu -- the random-sector gather ceiling the search kernels are
// measured against.
//
// Every FM-index step is a dependent load of one random 32-byte sector (the
// next address depends on the loaded counts).  This microbenchmark runs the
// same access pattern without the rank arithmetic: each thread follows a
// chain of random sectors over a buffer the size of the index, the next
// sector derived from the bytes just loaded.  Its rate (sectors/s) with full
// occupancy is the ceiling for latency-bound FM-index search on this GPU.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "fm_device.cuh"

namespace hpgbwt {

namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__global__ void gather_fill_kernel(uint4* buf, uint64_t n16, uint32_t seed) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t h = mix32((uint32_t)i ^ seed);
    buf[i] = make_uint4(h, mix32(h + 1), mix32(h + 2), mix32(h + 3));
  }
}

__global__ void __launch_bounds__(128) gather_chain_kernel(const uint4* __restrict__ buf, uint32_t nsec,
                                                            uint32_t steps, uint32_t seed, uint32_t work,
                                                            unsigned long long* sink) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t x = (uint32_t)(((uint64_t)mix32(tid ^ seed) * nsec) >> 32);
  uint32_t acc = 0;
  for (uint32_t s = 0; s < steps; ++s) {
    const uint4 a = __ldg(buf + 2ull * x);
    const uint4 b = __ldg(buf + 2ull * x + 1);
    uint32_t h = a.x + s + b.z;
    for (uint32_t w = 0; w < work; ++w) h = mix32(h);  // dependent ALU work between gathers
    acc += a.y ^ b.w;
    x = (uint32_t)(((uint64_t)mix32(h) * nsec) >> 32);
  }
  if (acc == 0x9E3779B9u) atomicAdd(sink, 1ull);
}

}  // namespace

// Sectors per second of dependent random 32-byte sector reads over a buffer
// of `bytes`, with `blocks` x 128 threads each following `steps` hops and
// `work` dependent hash rounds between hops.
int gather_ceiling(int device, size_t bytes, uint32_t blocks, uint32_t steps, double* sectors_per_s,
                   std::string* err, uint32_t work) {
  if (cudaSetDevice(device) != cudaSuccess) {
    *err = "cudaSetDevice failed";
    return -1;
  }
  const uint64_t nsec = bytes / 32;
  if (nsec < 1 || nsec >= (1ull << 32)) {
    *err = "gather buffer must hold 1 .. 2^32-1 sectors";
    return -1;
  }
  uint4* buf = nullptr;
  unsigned long long* sink = nullptr;
  if (cudaMalloc(&buf, nsec * 32) != cudaSuccess || cudaMalloc(&sink, 8) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(buf);
    *err = "out of device memory (gather buffer)";
    return -1;
  }
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  gather_fill_kernel<<<1024, 256, 0, s>>>(buf, nsec * 2, 12345u);
  cudaMemsetAsync(sink, 0, 8, s);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  gather_chain_kernel<<<blocks, 128, 0, s>>>(buf, (uint32_t)nsec, steps / 4 + 1, 7u, work, sink);  // warm-up
  cudaEventRecord(a, s);
  gather_chain_kernel<<<blocks, 128, 0, s>>>(buf, (uint32_t)nsec, steps, 99u, work, sink);
  cudaEventRecord(b, s);
  cudaError_t ce = cudaStreamSynchronize(s);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(s);
  cudaFree(buf);
  cudaFree(sink);
  if (ce != cudaSuccess) {
    *err = std::string("gather kernel: ") + cudaGetErrorString(ce);
    return -1;
  }
  *sectors_per_s = (double)blocks * 128.0 * steps / (ms * 1e-3);
  return 0;
}

}  // namespace hpgbwt
