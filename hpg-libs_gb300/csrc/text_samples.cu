// text_samples.cu -- the locate layer's text-sampled suffix array, derived on
// the device from the reference's row-sampled one when an index is opened.
//
// The reference keeps the SA values of the rows whose index is a multiple of
// the ratio (S.vec / Si.vec, S[i / ratio] = SA[i]) and locates a row by walking
// LF until it meets such a row (csafm.h:208-235).  The walk length is then
// geometric, mean ratio - 1 and unbounded, and a batch's locate pass ends with
// its few longest dependent chains.  The same ratio taken over text positions
// bounds every walk at ratio - 1 steps: the rows whose SA value is a multiple
// of the ratio are marked (uint4 per 64 rows: marked rows before the block, then
// the block's bits for rows 0..31 and 32..63) and their SA values kept in row
// order (T).  A row's SA value is the same number either way; only the walk
// that finds it is shorter.  The index files stay the reference's.
//
// Derivation: LF takes the row of text position p to the row of p - 1 (mod
// n + 1) and is one cycle over the n + 1 rows, which the reference's sampled
// rows cut into segments.  One walk per sampled row, from it up to the next
// sampled row, thus visits every row exactly once with its SA value known:
// n + 1 LF steps in all, run twice (mark the rows, then fill T by their rank).
#include <cuda_runtime.h>

#include <string>

#include "engine_internal.hpp"
#include "fm_device.cuh"
#include "kernels.cuh"

namespace hpgbwt {

namespace {

// fill 0: set the mark bit of every text-sampled row; fill 1: write its SA
// value to its slot in T (the marks and their ranks are in place by then).
__global__ void text_walk_kernel(DevIndex X, uint32_t d, uint32_t n_samples, uint32_t* __restrict__ words,
                                 uint32_t* __restrict__ T, int fill) {
  const DevDir D = dir_of(X, d);
  const uint32_t n_rows = X.walk_mod;  // n + 1
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_samples; k += stride) {
    const uint64_t r0 = (uint64_t)k * X.ratio;
    if (r0 >= n_rows) break;  // k only grows in this loop
    uint32_t i = (uint32_t)r0, v = D.S[k];
    if (v >= n_rows) {  // an SA value outside [0, n]: a corrupt index
      atomicOr(X.err, kErrWalk);
      continue;
    }
    for (uint32_t steps = 0;; ++steps) {
      if (ratio_multiple(X, v)) {
        if (fill) {
          uint32_t slot;
          text_sampled(D.mark[i >> 6], i, slot);
          T[slot] = v;
        } else {
          atomicOr(&words[4u * (i >> 6) + 1u + ((i >> 5) & 1u)], 1u << (i & 31));
        }
      }
      i = lf_step(X, D, i);
      v = v ? v - 1u : n_rows - 1u;
      if (sampled_row(X, i)) break;
      if (steps >= n_rows) {  // LF is one cycle over n + 1 rows: only a corrupt index gets here
        atomicOr(X.err, kErrWalk);
        break;
      }
    }
  }
}

__global__ void mark_count_kernel(const uint4* __restrict__ mark, size_t ne, uint32_t* __restrict__ cnt) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (size_t)gridDim.x * blockDim.x) {
    const uint4 m = mark[e];
    cnt[e] = (uint32_t)(__popc(m.y) + __popc(m.z));
  }
}

__global__ void mark_rank_kernel(uint4* __restrict__ mark, size_t ne, const uint64_t* __restrict__ excl) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (size_t)gridDim.x * blockDim.x)
    mark[e].x = (uint32_t)excl[e];
}

}  // namespace

int build_text_samples(Engine* en, const uint32_t n_samples[2], std::string* err) {
  const uint32_t n_rows = en->X.walk_mod;
  const size_t ne = ((size_t)n_rows + 63) / 64;
  const uint64_t n_t = ((uint64_t)n_rows + en->X.ratio - 1) / en->X.ratio;  // multiples of the ratio in [0, n]
  const unsigned grid = (unsigned)en->num_sms * 8;
  uint32_t* cnt = nullptr;
  uint64_t* excl = nullptr;
  uint64_t* part = nullptr;
  auto fail = [&](const std::string& why) {
    cudaFree(cnt);
    cudaFree(excl);
    cudaFree(part);
    *err = why;
    return -1;
  };
  if (cudaMalloc(&cnt, ne * 4 + 4) != cudaSuccess || cudaMalloc(&excl, (ne + 1) * 8) != cudaSuccess ||
      cudaMalloc(&part, scan_parts(ne) * 8) != cudaSuccess) {
    cudaGetLastError();
    return fail("out of device memory (text-sampled suffix array)");
  }
  for (int d = 0; d < 2; ++d) {
    if (cudaMalloc(&en->d_mark[d], ne * sizeof(uint4)) != cudaSuccess ||
        cudaMalloc(&en->d_T[d], n_t * 4 + 4) != cudaSuccess) {
      cudaGetLastError();
      return fail("out of device memory (text-sampled suffix array)");
    }
    cudaMemset(en->d_mark[d], 0, ne * sizeof(uint4));
    count_launches(1);
    text_walk_kernel<<<grid, 256>>>(en->X, d, n_samples[d], reinterpret_cast<uint32_t*>(en->d_mark[d]), nullptr, 0);
    count_launches(2);
    mark_count_kernel<<<grid, 256>>>(en->d_mark[d], ne, cnt);
    launch_scan(cnt, ne, excl, part, 0);
    mark_rank_kernel<<<grid, 256>>>(en->d_mark[d], ne, excl);
    uint64_t total = 0;
    if (cudaMemcpy(&total, excl + ne, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(std::string("text-sampled suffix array: ") + cudaGetErrorString(cudaGetLastError()));
    uint32_t e_word = 0;
    cudaMemcpy(&e_word, en->d_err, 4, cudaMemcpyDeviceToHost);
    if (total != n_t || e_word)
      return fail("corrupt index: the LF walks from the sampled rows do not cover the suffix array once");
    en->X.dir[d].mark = en->d_mark[d];
    en->X.dir[d].T = en->d_T[d];
    count_launches(1);
    text_walk_kernel<<<grid, 256>>>(en->X, d, n_samples[d], nullptr, en->d_T[d], 1);
  }
  cudaError_t ce = cudaDeviceSynchronize();
  uint32_t e_word = 0;
  if (ce == cudaSuccess) ce = cudaMemcpy(&e_word, en->d_err, 4, cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return fail(std::string("text-sampled suffix array: ") + cudaGetErrorString(ce));
  if (e_word) return fail("corrupt index: the LF walks from the sampled rows do not cover the suffix array once");
  cudaFree(cnt);
  cudaFree(excl);
  cudaFree(part);
  return 0;
}

}  // namespace hpgbwt
