// map_device.cu -- device passes of the alignment-list layer (map_api.cpp):
// the exact search pair of bwt_map_exact_seq, the vector-search endpoints the
// anchor lists start from, and locating caller-chosen SA rows.
#include <cuda_runtime.h>

#include <vector>

#include "engine_internal.hpp"

namespace hpgbwt {

namespace {

// bwt_map_exact_seq (bwt.c:919-940): '+' BWExactSearchBackward over backward
// from the last base, '-' BWExactSearchForward over forward_rev from the
// first, both from the full interval; the interval where the search stopped
// (k = l + 1 when a base failed), as the reference's result keeps it.
__global__ void exact_api_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                 const uint8_t* __restrict__ ok, uint32_t n, uint4* __restrict__ out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint64_t b = offs[r];
  const int len = (int)(offs[r + 1] - b);
  uint4 o = make_uint4(1, 0, 1, 0);  // reads outside the alphabet: nothing to locate
  if (ok[r] && len >= 0 && len <= 32767) {
    const uint8_t* W = codes + b;
    uint32_t k = 0, l = X.top;
    for (int i = len - 1; i >= 0; --i) {
      bw_step(X, View{0, 0}, W[i], k, l);
      if (k > l) break;
    }
    o.x = k;
    o.y = l;
    k = 0;
    l = X.top;
    for (int i = 0; i < len; ++i) {
      bw_step(X, View{1, 1}, W[i], k, l);
      if (k > l) break;
    }
    o.z = k;
    o.w = l;
  }
  out[r] = o;
}

// The four vector searches of bwt.c:1940-1950, reduced to what the anchor
// lists use (bwt.c:2249-2271): good steps and the last good interval of each.
//   c 0: backward over backward ('+' BACKWARD)   c 1: forward over forward ('+' FORWARD)
//   c 2: forward over backward_rev ('-' BACKWARD) c 3: backward over forward_rev ('-' FORWARD)
__global__ void anchor_scan_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                   const uint8_t* __restrict__ ok, const uint32_t* __restrict__ reads, uint32_t m,
                                   uint4* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * m) return;
  const uint32_t r = reads[t >> 2], c = t & 3u;
  const uint64_t b = offs[r];
  const int len = (int)(offs[r + 1] - b);
  uint4 o = make_uint4(0, 1, 0, 0);  // no good step: no interval
  if (ok[r] && len > 0 && len <= 32767) {
    const uint8_t* W = codes + b;
    const View v = c == 0 ? View{0, 0} : c == 1 ? View{1, 0} : c == 2 ? View{0, 1} : View{1, 1};
    const bool backward = (c == 0 || c == 3);
    uint32_t k = 0, l = X.top, nt = 0, gk = 1, gl = 0;
    for (int s = 0; s < len; ++s) {
      bw_step(X, v, W[backward ? len - 1 - s : s], k, l);
      if (k > l) break;
      ++nt;
      gk = k;
      gl = l;
    }
    o = make_uint4(nt, gk, gl, 0);
  }
  out[t] = o;
}

// bwt_map_exact_seed (bwt.c:1232-1252): the seed W[first .. last] of a read,
// '+' BWExactSearchBackward over backward from `last`, '-' BWExactSearchForward
// over backward_rev (the backward index with complemented symbols) from
// `first`, both from the full interval; the interval where the search stopped.
__global__ void seed_search_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                   const uint8_t* __restrict__ ok, const uint4* __restrict__ seeds, uint32_t m,
                                   uint4* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const uint4 sd = seeds[t];
  const uint64_t b = offs[sd.x];
  const uint64_t len = offs[sd.x + 1] - b;
  uint4 o = make_uint4(1, 0, 1, 0);  // nothing to locate
  if (ok[sd.x] && sd.y <= sd.z && sd.z < len) {
    const uint8_t* W = codes + b;
    uint32_t k = 0, l = X.top;
    for (int64_t i = sd.z; i >= (int64_t)sd.y; --i) {
      bw_step(X, View{0, 0}, W[i], k, l);
      if (k > l) break;
    }
    o.x = k;
    o.y = l;
    k = 0;
    l = X.top;
    for (uint32_t i = sd.y; i <= sd.z; ++i) {
      bw_step(X, View{0, 1}, W[i], k, l);
      if (k > l) break;
    }
    o.z = k;
    o.w = l;
  }
  out[t] = o;
}

}  // namespace

int upload_reads(Engine* e, const char* seqs, const uint64_t* offs, size_t n, std::string* err) {
  cudaStream_t s = e->stream;
  const uint64_t total = n ? offs[n] - offs[0] : 0;
  if (!ensure(e, e->seqs, total + 16) || !ensure(e, e->offs, (n + 1) * 8) || !ensure(e, e->codes, total + 16) ||
      !ensure(e, e->ok, n + 16)) {
    *err = "out of device memory (reads)";
    return -1;
  }
  std::vector<uint64_t> rel(n + 1);
  for (size_t i = 0; i <= n; ++i) rel[i] = n ? offs[i] - offs[0] : 0;
  if (total) HPG_CUDA(cudaMemcpyAsync(e->seqs.p, seqs + offs[0], total, cudaMemcpyHostToDevice, s), "upload reads");
  HPG_CUDA(cudaMemcpyAsync(e->offs.p, rel.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s), "upload offsets");
  launch_encode(ptr<uint8_t>(e->seqs), total, ptr<uint64_t>(e->offs), (uint32_t)n, e->d_table, ptr<uint8_t>(e->codes),
                ptr<uint8_t>(e->ok), s);
  HPG_CUDA(cudaStreamSynchronize(s), "encode");  // `rel` is pageable and local
  return 0;
}

namespace {

int check_walk(Engine* e, std::string* err) {
  uint32_t derr = 0;
  HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
  if (derr) {
    cudaMemset(e->d_err, 0, 4);
    *err = "corrupt index: suffix-array walk did not reach a sampled row";
    return -1;
  }
  return 0;
}

}  // namespace

int engine_exact_api(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t* kl, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (n >= (1ull << 31)) {
    *err = "too many reads in one batch";
    return -1;
  }
  if (!n) return 0;
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, n * sizeof(uint4) + 16)) {
    *err = "out of device memory (exact intervals)";
    return -1;
  }
  cudaStream_t s = e->stream;
  count_launches(1);
  exact_api_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes), ptr<uint64_t>(e->offs),
                                                                ptr<uint8_t>(e->ok), (uint32_t)n, ptr<uint4>(e->slots));
  HPG_CUDA(cudaMemcpyAsync(kl, e->slots.p, n * sizeof(uint4), cudaMemcpyDeviceToHost, s), "exact intervals");
  HPG_CUDA(cudaStreamSynchronize(s), "exact search");
  return 0;
}

int engine_anchor_scan(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* reads, size_t m,
                       uint32_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, 4 * m * sizeof(uint4) + 16) || !ensure(e, e->rows, m * 4 + 16)) {
    *err = "out of device memory (anchor scan)";
    return -1;
  }
  cudaStream_t s = e->stream;
  HPG_CUDA(cudaMemcpyAsync(e->rows.p, reads, m * 4, cudaMemcpyHostToDevice, s), "anchor reads");
  count_launches(1);
  anchor_scan_kernel<<<(unsigned)((4 * m + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes),
                                                                      ptr<uint64_t>(e->offs), ptr<uint8_t>(e->ok),
                                                                      ptr<uint32_t>(e->rows), (uint32_t)m,
                                                                      ptr<uint4>(e->slots));
  HPG_CUDA(cudaMemcpyAsync(out, e->slots.p, 4 * m * sizeof(uint4), cudaMemcpyDeviceToHost, s), "anchor scan");
  HPG_CUDA(cudaStreamSynchronize(s), "anchor scan");
  return 0;
}

int engine_seed_search(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* seeds, size_t m,
                       uint32_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (m >= (1ull << 31)) {
    *err = "too many seeds in one call";
    return -1;
  }
  for (size_t i = 0; i < m; ++i)
    if (seeds[4 * i] >= n) {
      *err = "seed of a read outside the batch";
      return -1;
    }
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, 2 * m * sizeof(uint4) + 16)) {
    *err = "out of device memory (seeds)";
    return -1;
  }
  cudaStream_t s = e->stream;
  uint4* d_seeds = ptr<uint4>(e->slots);
  uint4* d_out = d_seeds + m;
  HPG_CUDA(cudaMemcpyAsync(d_seeds, seeds, m * sizeof(uint4), cudaMemcpyHostToDevice, s), "seeds");
  count_launches(1);
  seed_search_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes), ptr<uint64_t>(e->offs),
                                                                  ptr<uint8_t>(e->ok), d_seeds, (uint32_t)m, d_out);
  HPG_CUDA(cudaMemcpyAsync(out, d_out, m * sizeof(uint4), cudaMemcpyDeviceToHost, s), "seed intervals");
  HPG_CUDA(cudaStreamSynchronize(s), "seed search");
  return 0;
}

int engine_locate_rows(Engine* e, const MapRow* rows, size_t m, hpg_loc_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (m >= (1ull << 32)) {
    *err = "too many rows to locate in one call";
    return -1;
  }
  std::vector<RowItem> items(m);
  for (size_t i = 0; i < m; ++i) {
    if (rows[i].row > e->X.top) {
      *err = "row outside the suffix array";
      return -1;
    }
    items[i].row = rows[i].row;
    items[i].hit = (uint32_t)i;
    items[i].out = (uint32_t)i;
    items[i].phys_len = (rows[i].phys << 31) | (rows[i].key32 ? kRowKey32 : 0u) | (rows[i].len_calc & kRowLenMask);
  }
  if (!ensure(e, e->b_rowhit, m * sizeof(RowItem) + 16) || !ensure(e, e->locs, m * sizeof(hpg_loc_t) + 16) ||
      !ensure(e, e->b_ctr, 64)) {
    *err = "out of device memory (locate rows)";
    return -1;
  }
  cudaStream_t s = e->stream;
  HPG_CUDA(cudaMemcpyAsync(e->b_rowhit.p, items.data(), m * sizeof(RowItem), cudaMemcpyHostToDevice, s), "rows");
  launch_locate_items(e->X, static_cast<const RowItem*>(e->b_rowhit.p), m, ptr<hpg_loc_t>(e->locs),
                      ptr<unsigned int>(e->b_ctr) + 5, e->num_sms, s);
  HPG_CUDA(cudaMemcpyAsync(out, e->locs.p, m * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, s), "located rows");
  HPG_CUDA(cudaStreamSynchronize(s), "locate rows");
  return check_walk(e, err);
}

void engine_set_skip_locate(Engine* e, int on) { e->skip_locate = on != 0; }

std::mutex& map_api_mutex() {
  static std::mutex mu;
  return mu;
}
uint32_t engine_sa_top(Engine* e) { return e->X.top; }

}  // namespace hpgbwt
