// batched_dev.cuh -- device helpers shared by the batched search kernels
// (batched.cu: fused, split and lockstep forms; wave.cu: the warp-cooperative
// form): change-point encoding, order keys, chunked result slots.
#pragma once

#include <cooperative_groups.h>

#include "batched.cuh"
#include "search_core.cuh"

namespace hpgbwt {
namespace bdev {

namespace cg = cooperative_groups;

// Change-point entry types.
enum : uint32_t { kCpBwd = 0, kCpFwd = 1, kBlk1 = 2, kBlkN = 3 };
// Sub-operations of an entry: 0 deletion, then per base b: 1+3b aux step,
// 2+3b insertion, 3+3b mismatch; 13 = finished.
constexpr uint32_t kSubEnd = 13;

// Order keys: section << 28 | t << 8 | slot, following the helper's emission
// order: exact hit, j=1 block, backward j ascending, j=n-1 block, forward j descending.
__device__ __forceinline__ uint32_t order_key(uint32_t section, uint32_t t, uint32_t slot) {
  return (section << 28) | (t << 8) | slot;
}

// Pool slots are reserved per lane in chunks, so an emission normally waits on
// no atomic: the per-list arrival count is a fire-and-forget reduction and
// the list position is assigned later by the scatter kernel.
constexpr unsigned kResChunk = 8;

__device__ __forceinline__ void write_hit(const BatchedParams& p, unsigned slot, uint32_t rs, uint32_t key,
                                          uint32_t k, uint32_t l, uint32_t meta) {
  atomicAdd(&p.rs_count[rs], 1u);  // result unused: compiles to a reduction
  if (slot < p.res_cap) {
    PendingHit h;
    h.rs = rs;
    h.key = key;
    h.k = k;
    h.l = l;
    h.meta = meta;
    h.idx = 0;
    p.res[slot] = h;
  } else {
    atomicOr(p.status, kStatusResFull);
  }
}

__device__ __forceinline__ void emit_hit(const BatchedParams& p, uint32_t rs, uint32_t key, uint32_t k, uint32_t l,
                                         uint32_t meta) {
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(p.res_total, (unsigned)g.size());
  base = g.shfl(base, 0) + g.thread_rank();
  write_hit(p, base, rs, key, k, l, meta);
}

__device__ __forceinline__ unsigned claim(unsigned int* ctr, unsigned n) {
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(ctr, (unsigned)g.size() * n);
  return g.shfl(base, 0) + g.thread_rank() * n;
}

// Chunked pool slot for the calling lane (cold state c_res = next slot | left << 28).
__device__ __forceinline__ unsigned res_slot(const BatchedParams& p, uint32_t& c_res) {
  unsigned left = c_res >> 28;
  if (left == 0) {
    c_res = claim(p.res_total, kResChunk);
    left = kResChunk;
    if (c_res >= (1u << 28)) {  // beyond what the packed form holds: fall back to single slots
      c_res = 0;
      return claim(p.res_total, 1) | 0u;
    }
  }
  const unsigned slot = c_res & 0x0FFFFFFFu;
  c_res = (slot + 1) | ((left - 1) << 28);
  return slot;
}

// Lane modes.
enum : uint32_t { kNone = 0, kChain = 1, kCont = 2, kSingle = 3, kKmer = 4 };

// Cold lane state lives in shared memory (one word per lane and field), so
// that the registers hold only what every step touches.
//   meta: J (16 bits) | entry type << 16 | sub-operation << 18 | block err_pos << 22 | in entry << 24
//   misc: stack depth (4 bits) | chains left in the claimed chunk << 4
__device__ __forceinline__ uint32_t meta_j(uint32_t m) { return m & 0xFFFFu; }
__device__ __forceinline__ uint32_t meta_type(uint32_t m) { return (m >> 16) & 3u; }
__device__ __forceinline__ uint32_t meta_sub(uint32_t m) { return (m >> 18) & 15u; }
__device__ __forceinline__ uint32_t meta_bpos(uint32_t m) { return (m >> 22) & 3u; }
__device__ __forceinline__ bool meta_in(uint32_t m) { return (m >> 24) & 1u; }
__device__ __forceinline__ uint32_t make_meta(uint32_t j, uint32_t type, uint32_t sub, uint32_t bpos, bool in) {
  return j | (type << 16) | (sub << 18) | (bpos << 22) | ((in ? 1u : 0u) << 24);
}


}  // namespace bdev
}  // namespace hpgbwt
