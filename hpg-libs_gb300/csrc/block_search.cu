// block_search.cu -- the k-error block search of bwt_map_inexact_read_2
// (c/src/aligners/bwt/bwt.c:2313-2470): BWSearchCPU (search/search.c:1171-1405)
// on both strands with that function's fragment size max(len / 2, 30) -- one
// or two fragments, so one error.
//
// The reference keeps its partial results in lists: an exact-partial pass
// appends a branch point for every step where the interval size changes while
// the error bound D still allows an error (BWExactPartialResults*,
// search.c:471-646), then a branch pass extends each branch point by a
// deletion and, per base, an insertion and a mismatch (BWBranchFinalResults*,
// search.c:116-469).  A thread here runs one block of a (read, strand) and
// replays the walk instead of storing it:
//   * a first walk over the rest of the read counts the restarts D is made of
//     (calculateD*, search.c:1045-1169: D at a step is the number of restarts
//     still ahead, as a byte) and the branch points, so that a list that would
//     overflow is known before anything is emitted (the reference then drops
//     the block's branches);
//   * within the exact-partial range D is the total (the walk has not failed
//     yet) or the total minus one (the step where it fails), so the total is
//     all the second walk needs to emit the branches in the reference's order;
//     it stops at the last branch point.
// Every block stays on one physical index direction, and one launch per
// direction keeps that direction's occurrence blocks in L2; a merge then puts
// each list's two blocks together as the reference's single list.  Results go
// to a fixed number of slots per block; the few blocks with more results run
// again into their final range.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "engine_internal.hpp"
#include "host_pool.hpp"

namespace hpgbwt {

namespace {

constexpr uint32_t kBlockSlots = 4;  // result slots per block in the first pass
constexpr int kBlockTpb = 128;

struct ItemOut {
  hpg_hit_t* slot;  // the item's first result slot
  uint32_t room;    // slots available; results past them are counted only
  uint32_t cap;     // capacity of the reference's lists (max_results)
  uint32_t n;       // results kept (<= cap)
  uint32_t read;
  uint32_t strand;
  bool refused;     // a list refused a result (full)
  uint32_t sectors; // occurrence-block sectors the item read (census)
};

// BWiteration over a view; with C (the census instance) it also counts the
// 32-byte sectors it reads (one when k and l share an occurrence block, else two).
template <bool C>
__device__ __forceinline__ void step(const DevIndex& X, View v, uint32_t c, uint32_t& k, uint32_t& l, uint32_t& sec) {
  if (C) sec += (k >> 6) == (l >> 6) ? 1u : 2u;
  bw_step(X, v, c, k, l);
}

// add_result (search/results.h:93-103) on rl_final.
__device__ __forceinline__ bool emit(ItemOut& o, uint32_t dir, uint32_t nm, uint32_t kind, uint32_t base, int pos,
                                     uint32_t k, uint32_t l) {
  if (o.n >= o.cap) {
    o.refused = true;
    return false;
  }
  if (o.n < o.room) {
    hpg_hit_t h;
    h.read = o.read;
    h.strand = (uint8_t)o.strand;
    h.dir = (uint8_t)dir;
    h.nm = (uint8_t)nm;
    h.err_kind = (uint8_t)(nm ? kind : 0);
    h.err_base = (uint8_t)(nm ? base : 0);
    h.pad0 = 0;
    h.err_pos = (int16_t)(nm ? pos : 0);
    h.pad1 = 0;
    h.k = k;
    h.l = l;
    o.slot[o.n] = h;
  }
  ++o.n;
  return true;
}

// BWExactFinalResultForward (search/search.h:114-155): the block rule, then
// the walk over W[pos..end]; k, l are updated only when it survives.
template <bool C>
__device__ __forceinline__ bool final_forward(const DevIndex& X, View v, const uint8_t* W, int pos, int end, int bs,
                                              int last_block, uint32_t& k, uint32_t& l, uint32_t& sec) {
  const int cb = pos / bs;
  if (!(cb > last_block || pos == end + 1)) {
    if (cb < last_block) return false;
    if (pos % bs == 0) return false;
  }
  uint32_t a = k, b = l;
  for (int i = pos; i <= end; ++i) {
    step<C>(X, v, W[i], a, b, sec);
    if (a > b) return false;
  }
  k = a;
  l = b;
  return true;
}

// BWExactFinalResultBackward (search/search.h:67-112), over W[pos..start]
// downwards.  C division truncates toward zero (pos may be -1).
template <bool C>
__device__ __forceinline__ bool final_backward(const DevIndex& X, View v, const uint8_t* W, int pos, int start, int bs,
                                               int last_block, uint32_t& k, uint32_t& l, uint32_t& sec) {
  const int cb = pos / bs;
  if (!(cb < last_block || pos == start - 1)) {
    if (cb > last_block) return false;
    if ((pos + 1) % bs == 0) return false;
  }
  uint32_t a = k, b = l;
  for (int i = pos; i >= start; --i) {
    step<C>(X, v, W[i], a, b, sec);
    if (a > b) return false;
  }
  k = a;
  l = b;
  return true;
}

// The branches of one branch point (interval k..l before the step at `pos`)
// in BWBranchFinalResultsForward's order for a result without an earlier
// error (search.c:430-462): deletion, then per base an insertion and a
// mismatch.  The mismatch starts from the interval the insertion's extension
// left in the reference's result when that extension survived (the reference
// resets only `pos` there).  False when rl_final refused a result.
template <bool C>
__device__ bool branch_forward(const DevIndex& X, View v, const uint8_t* W, int pos, int end, int bs, uint32_t k,
                               uint32_t l, ItemOut& o) {
  constexpr uint32_t kDir = 1;
  uint32_t a = k, b = l;
  if (final_forward<C>(X, v, W, pos + 1, end, bs, 0, a, b, o.sectors) &&
      !emit(o, kDir, 1, HPG_BWT_DELETION, 0xFF, pos, a, b))
    return false;
  const uint32_t wp = W[pos];
  for (uint32_t c = 0; c < 4; ++c) {
    uint32_t ka = k, la = l;
    step<C>(X, v, c, ka, la, o.sectors);
    if (ka > la || c == wp) continue;
    uint32_t rk = ka, rl = la;
    a = ka;
    b = la;
    if (final_forward<C>(X, v, W, pos, end, bs, 0, a, b, o.sectors)) {
      if (!emit(o, kDir, 1, HPG_BWT_INSERTION, c, pos, a, b)) return false;
      rk = a;
      rl = b;
    }
    if (final_forward<C>(X, v, W, pos + 1, end, bs, 0, rk, rl, o.sectors) && !emit(o, kDir, 1, HPG_BWT_MISMATCH, c, pos, rk, rl))
      return false;
  }
  return true;
}

// BWBranchFinalResultsBackward (search.c:252-284), the same on the backward side.
template <bool C>
__device__ bool branch_backward(const DevIndex& X, View v, const uint8_t* W, int pos, int bs, uint32_t k, uint32_t l,
                                ItemOut& o) {
  constexpr uint32_t kDir = 0;
  constexpr int start = 0;
  uint32_t a = k, b = l;
  if (final_backward<C>(X, v, W, pos - 1, start, bs, 0, a, b, o.sectors) &&
      !emit(o, kDir, 1, HPG_BWT_DELETION, 0xFF, pos, a, b))
    return false;
  const uint32_t wp = W[pos];
  for (uint32_t c = 0; c < 4; ++c) {
    uint32_t ka = k, la = l;
    step<C>(X, v, c, ka, la, o.sectors);
    if (ka > la || c == wp) continue;
    uint32_t rk = ka, rl = la;
    a = ka;
    b = la;
    if (final_backward<C>(X, v, W, pos, start, bs, 0, a, b, o.sectors)) {
      if (!emit(o, kDir, 1, HPG_BWT_INSERTION, c, pos, a, b)) return false;
      rk = a;
      rl = b;
    }
    if (final_backward<C>(X, v, W, pos - 1, start, bs, 0, rk, rl, o.sectors) &&
        !emit(o, kDir, 1, HPG_BWT_MISMATCH, c, pos, rk, rl))
      return false;
  }
  return true;
}

// First walk of a block from the interval k..l at `from` towards `to` (step
// +1 or -1): the restart walk of calculateD* and, as its prefix up to the
// first empty interval, the exact-partial walk.  Returns the number of branch
// points that walk appends; `survive` whether it covers the whole range with
// a non-empty interval (then k, l hold that interval).
template <bool C>
__device__ uint32_t first_walk(const DevIndex& X, View v, const uint8_t* W, int from, int to, int dstep, uint32_t& k,
                               uint32_t& l, bool& survive, uint32_t& zt, uint32_t& sec) {
  uint32_t a = k, b = l;
  uint32_t z = 0, changes = 0;
  bool alive = true, failed_step = false;
  for (int i = from; i != to + dstep; i += dstep) {
    const int64_t before = (int64_t)b - (int64_t)a;
    step<C>(X, v, W[i], a, b, sec);
    if (alive) {
      if (a > b) {
        alive = false;
        failed_step = true;  // the step that empties the interval changes its size
      } else if ((int64_t)b - (int64_t)a != before) {
        ++changes;
      }
      if (alive) {
        k = a;
        l = b;
      }
    }
    if (a > b) {
      a = 0;
      b = X.top;
      ++z;
      // three restarts with too few steps left for the byte count to wrap: D
      // allows no error anywhere in the range, so there is no branch point
      if (z >= 3 && z + (uint32_t)(dstep > 0 ? to - i : i - to) < 256) break;
    }
  }
  survive = alive;
  zt = z & 255u;
  // D before the failing step is the total; at it, the total minus one (bytes)
  const bool bound_before = zt <= 1u;
  const bool bound_at = ((zt - 1u) & 255u) <= 1u;
  return (bound_before ? changes : 0u) + (failed_step && bound_at ? 1u : 0u);
}

__device__ __forceinline__ void put_anchor(hpg_block_anchor_t* anchor, uint32_t& aflag, uint32_t dir, int start,
                                           int end, int pos, uint32_t k, uint32_t l) {
  if (anchor) {
    hpg_block_anchor_t x;
    x.k = k;
    x.l = l;
    x.start = (int16_t)start;
    x.end = (int16_t)end;
    x.pos = (int16_t)pos;
    x.dir = (uint8_t)dir;
    x.pad = 0;
    *anchor = x;
  }
  aflag |= 1u;
}

// Fragments of a read: bwt.c:2408-2412 takes len / (num_errors + 1), at least
// 30, and BWSearchCPU divides the length by it (search.c:1175).
__device__ __forceinline__ int fragments_of(int len, int& frag) {
  frag = len / 2;
  if (frag < 30) frag = 30;
  return len / frag;
}

// The block of a (read, strand) that runs on physical index direction `phys`:
// 0 block 0 (or the one exact search of a single-fragment read), 1 the last
// block, -1 none.  Block 0 searches forward over `forward` ('+': the forward
// index; '-': backward_rev, the backward index), the last block backward over
// `backward` ('+': the backward index; '-': forward_rev, the forward index); a
// single-fragment read's exact search is on the backward index for both
// strands ('+' backward over backward, '-' forward over backward_rev).
__device__ __forceinline__ int part_on(uint32_t strand, int fragments, uint32_t phys) {
  if (fragments <= 1) return phys == 0 ? 0 : -1;
  return (strand ^ phys) ? 0 : 1;
}

// The views of a strand: type 1 ('+', strand 0) searches backward over
// `backward` and forward over `forward`; type 0 ('-', strand 1) over
// forward_rev and backward_rev (bwt.c:2440-2472).
__device__ __forceinline__ View backward_view(uint32_t strand) { return strand ? View{1, 1} : View{0, 0}; }
__device__ __forceinline__ View forward_view(uint32_t strand) { return strand ? View{0, 1} : View{1, 0}; }

// Head of one block of a (read, strand) (BWSearchCPU, search.c:1171-1405, with
// two fragments or fewer): the exact search of the block's fragment and its
// anchor.  A single-fragment read's one exact search is all its work (its
// result is emitted here).  True, with the fragment's interval in k, l, when
// the block goes on (its fragment matched and the lists have room).  aflag
// bit 0: the anchor was set; bit 1: the block-0 fragment matched (with lists
// of capacity 0 BWSearchCPU then returns before the last block).
// The first L steps of an exact search from the full interval over view v, W[from],
// W[from + dir], ..., by one lookup in the start table (L = X.kmer_len, the
// table's entries already hold the interval after those steps); true with
// k, l set when that interval is not empty, else the caller steps from the
// start (it needs the position where the search failed).  Not in the census
// instance, whose count stays that of the reference's steps.
template <bool C>
__device__ __forceinline__ bool start_lookup(const DevIndex& X, View v, const uint8_t* W, int from, int dir, int steps,
                                             uint32_t& k, uint32_t& l) {
  const uint32_t L = X.kmer_len;
  if (C || L == 0 || steps < (int)L) return false;
  uint32_t code = 0;
  for (uint32_t j = 0; j < L; ++j) {
    const uint32_t b = W[from + dir * (int)j];
    code = (code << 2) | (v.comp ? sel4(X.comp, b) : b);
  }
  const uint2 t = __ldg((v.d ? X.kmer[1] : X.kmer[0]) + code);
  if (t.x > t.y) return false;
  k = t.x;
  l = t.y;
  return true;
}

// The fragment walk of a block's head: view, first and last position, step
// direction, and the anchor's direction (1: forward from the read's start).
struct HeadWalk {
  View v;
  int from, to, dir;
  uint32_t adir;
  bool single;
};

__device__ __forceinline__ HeadWalk head_walk(int len, uint32_t strand, int part) {
  HeadWalk h;
  int frag = 30;
  const int fragments = fragments_of(len, frag);
  const int end = len - 1;
  h.single = fragments <= 1;
  if (h.single ? strand != 0 : part == 0) {
    // search.c:1191-1224 type 0 (one exact search forward from the first base), or
    // block 0 forward over W[0 .. frag-1] (search.c:1276-1311)
    h.v = forward_view(strand);
    h.from = 0;
    h.to = h.single ? end : frag - 1;
    h.dir = 1;
    h.adir = 1;
  } else {
    // type 1 (backward from the last base), or the last block backward over
    // W[frag .. len-1] (search.c:1360-1402)
    h.v = backward_view(strand);
    h.from = end;
    h.to = h.single ? 0 : frag;
    h.dir = -1;
    h.adir = 0;
  }
  return h;
}

// Steps of a head walk from position i with the non-empty interval k..l, while
// it stays non-empty, at most `budget` of them (negative: no limit); gk, gl keep
// the last non-empty interval.  True when the walk is over (it failed, i at the
// failing position, or it passed `to`); false when the budget ran out first.
template <bool C>
__device__ __forceinline__ bool head_steps(const DevIndex& X, const HeadWalk& h, const uint8_t* W, int& i,
                                           uint32_t& k, uint32_t& l, uint32_t& gk, uint32_t& gl, int budget,
                                           uint32_t& sec) {
  while (h.dir > 0 ? i <= h.to : i >= h.to) {
    if (budget-- == 0) return false;
    step<C>(X, h.v, W[i], k, l, sec);
    if (k > l) return true;
    gk = k;
    gl = l;
    i += h.dir;
  }
  return true;
}

// The end of a head: the anchor, then the single search's result, or the
// block's match (block 0's flag) and whether the block goes on to the tail.
__device__ __forceinline__ bool head_finish(const HeadWalk& h, int len, ItemOut& o, hpg_block_anchor_t* anchor,
                                            uint32_t& aflag, int i, uint32_t k, uint32_t l, uint32_t gk,
                                            uint32_t gl) {
  if (h.adir) put_anchor(anchor, aflag, 1, 0, i - 1, i, gk, gl);
  else put_anchor(anchor, aflag, 0, i + 1, len - 1, i, gk, gl);
  if (h.single) {
    if (k <= l) emit(o, h.adir, 0, 0, 0, 0, k, l);
    return false;
  }
  if (k > l) return false;
  if (h.adir) aflag |= 2u;  // block 0 matched
  if (o.cap == 0) {  // add_result(&r, rl_prev) returns from BWSearchCPU
    o.refused = true;
    return false;
  }
  return true;
}

// The head's first steps: the start-table lookup for the first L steps when
// the walk is that long (one lookup for them), from the full interval.
template <bool C>
__device__ __forceinline__ void head_start(const DevIndex& X, const HeadWalk& h, const uint8_t* W, int& i,
                                           uint32_t& k, uint32_t& l, uint32_t& gk, uint32_t& gl) {
  i = h.from;
  k = 0;
  l = X.top;
  gk = gl = 0;
  const int steps = h.dir > 0 ? h.to - h.from + 1 : h.from - h.to + 1;
  if (start_lookup<C>(X, h.v, W, h.from, h.dir, steps, k, l)) {
    gk = k;
    gl = l;
    i = h.from + h.dir * (int)X.kmer_len;
  }
}

template <bool C>
__device__ bool block_head(const DevIndex& X, const uint8_t* W, int len, uint32_t strand, int part, ItemOut& o,
                           hpg_block_anchor_t* anchor, uint32_t& aflag, uint32_t& k, uint32_t& l) {
  const HeadWalk h = head_walk(len, strand, part);
  int i;
  uint32_t gk, gl;
  head_start<C>(X, h, W, i, k, l, gk, gl);
  head_steps<C>(X, h, W, i, k, l, gk, gl, -1, o.sectors);
  return head_finish(h, len, o, anchor, aflag, i, k, l, gk, gl);
}

// Tail of a block whose fragment matched with interval k..l: the rest of the
// read (first walk, the complete result of block 0, the second walk and the
// branches), emitted as if the list were empty; the merge cuts the last
// block's results to the room block 0 left.
template <bool C>
__device__ void block_tail(const DevIndex& X, const uint8_t* W, int len, uint32_t strand, int part, ItemOut& o,
                           uint32_t k, uint32_t l) {
  int frag = 30;
  fragments_of(len, frag);
  const int end = len - 1;
  if (part == 0) {
    const View fw = forward_view(strand);
    // exact-partial range: pos = frag is past block 0, so the whole rest of
    // the read, and a walk that survives it is a result (complete search)
    uint32_t fk = k, fl = l, zt = 0;
    bool survive = false;
    const uint32_t points = first_walk<C>(X, fw, W, frag, end, 1, fk, fl, survive, zt, o.sectors);
    if (points > o.cap) {
      o.refused = true;  // rl_next overflows: the block's branches are dropped
      return;
    }
    if ((survive && !emit(o, 1, 0, 0, 0, 0, fk, fl)) || !points) return;
    // the second walk, up to the last branch point
    const bool ok_before = zt <= 1u, ok_at = ((zt - 1u) & 255u) <= 1u;
    uint32_t a = k, b = l, left = points;
    for (int p = frag; p <= end; ++p) {
      const uint32_t pk = a, pl = b;
      const int64_t before = (int64_t)b - (int64_t)a;
      step<C>(X, fw, W[p], a, b, o.sectors);
      const bool failed = a > b;
      const bool changed = failed || (int64_t)b - (int64_t)a != before;
      if (changed && (failed ? ok_at : ok_before)) {
        if (!branch_forward<C>(X, fw, W, p, end, frag, pk, pl, o) || --left == 0) break;
      }
      if (failed) break;
    }
    return;
  }
  const View bw = backward_view(strand);
  // exact-partial range: pos = frag - 1 is the first element of block 0
  // from above, so the rule walks the whole of it without completing
  uint32_t fk = k, fl = l, zt = 0;
  bool survive = false;
  const uint32_t points = first_walk<C>(X, bw, W, frag - 1, 0, -1, fk, fl, survive, zt, o.sectors);
  if (points > o.cap) {
    o.refused = true;
    return;
  }
  // the second walk, up to the last branch point
  const bool ok_before = zt <= 1u, ok_at = ((zt - 1u) & 255u) <= 1u;
  uint32_t a = k, b = l, left = points;
  for (int p = frag - 1; p >= 0 && left; --p) {
    const uint32_t pk = a, pl = b;
    const int64_t before = (int64_t)b - (int64_t)a;
    step<C>(X, bw, W[p], a, b, o.sectors);
    const bool failed = a > b;
    const bool changed = failed || (int64_t)b - (int64_t)a != before;
    if (changed && (failed ? ok_at : ok_before)) {
      if (!branch_backward<C>(X, bw, W, p, frag, pk, pl, o) || --left == 0) break;
    }
    if (failed) break;
  }
}

// Per-block state of a batch: list t = 2 * read + strand has blocks 2t (block
// 0 or the one exact search) and 2t + 1 (the last block).
struct PartState {
  hpg_hit_t* slots;               // kBlockSlots results per block (first pass)
  uint32_t* count;                // results per block, each as if alone in the list
  uint8_t* refused;               // a list of the block refused a result
  uint8_t* aflag;                 // put_anchor / block-0 match bits
  hpg_block_anchor_t* anchor;     // the block's anchor
  // results past the slots (tail pass): chunks of kOvfChunk, chained per block
  uint8_t* lost;                  // the pool ran out for this block: it runs again
  uint32_t* ovf_head;             // the block's first chunk
  uint32_t* ovf_next;             // the chunk after each chunk
  hpg_hit_t* ovf_hits;
  uint32_t* ovf_ctr;              // chunks handed out
  uint32_t ovf_cap;               // chunks in the pool
};

constexpr uint32_t kOvfChunk = 32;

// emit() in the tail pass: results past the block's slots go to chunks of the
// overflow pool (one atomic per chunk), so that the pack pass can place them
// and the block need not run again; when the pool runs out the block is marked
// lost and the retry pass runs it into its final range as before.
__device__ __forceinline__ bool emit_tail(ItemOut& o, const PartState& ps, uint32_t it, uint32_t& chunk, bool& lost,
                                          uint32_t dir, uint32_t nm, uint32_t kind, uint32_t base, int pos,
                                          uint32_t k, uint32_t l) {
  if (o.n >= o.cap) {
    o.refused = true;
    return false;
  }
  hpg_hit_t h;
  h.read = it >> 2;  // it = 2 * (2 * read + strand) + part
  h.strand = (uint8_t)((it >> 1) & 1u);
  h.dir = (uint8_t)dir;
  h.nm = (uint8_t)nm;
  h.err_kind = (uint8_t)(nm ? kind : 0);
  h.err_base = (uint8_t)(nm ? base : 0);
  h.pad0 = 0;
  h.err_pos = (int16_t)(nm ? pos : 0);
  h.pad1 = 0;
  h.k = k;
  h.l = l;
  if (o.n < kBlockSlots) {
    o.slot[o.n] = h;
  } else if (!lost) {
    const uint32_t j = o.n - kBlockSlots, off = j % kOvfChunk;
    if (off == 0) {
      const uint32_t nc = atomicAdd(ps.ovf_ctr, 1u);
      if (nc >= ps.ovf_cap) {
        lost = true;
      } else {
        if (j == 0) ps.ovf_head[it] = nc;
        else ps.ovf_next[chunk] = nc;
        chunk = nc;
      }
    }
    if (!lost) ps.ovf_hits[(uint64_t)chunk * kOvfChunk + off] = h;
  }
  ++o.n;
  return true;
}

// Warp-aggregated append of {it, k, l, w} to a queue.
__device__ __forceinline__ void queue_append(bool go, uint4* __restrict__ queue, uint32_t* __restrict__ n_queue,
                                             uint32_t it, uint32_t k, uint32_t l, uint32_t w) {
  const unsigned mask = __ballot_sync(__activemask(), go);
  if (go) {
    const uint32_t lane = threadIdx.x & 31u;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(n_queue, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    queue[base + (uint32_t)__popc(mask & ((1u << lane) - 1u))] = make_uint4(it, k, l, w);
  }
}

constexpr int kHeadSteps = 4;  // the head's steps past the start table before its walk is compacted

// Head pass over physical direction `phys`: thread g runs the head of the
// block of its list that is on that direction (the '+' lists in the first half
// of the threads, the '-' ones in the second, so that a warp's lanes run the
// same block code): the start-table lookup and up to kHeadSteps steps, which
// end most walks of the wrong strand.  Walks still going are appended to
// `cont` as {block, k, l, position} for block_head_rest_kernel, so that their
// long remainder runs in warps of walks that all go on; the blocks whose head
// ended here and go on are appended to `queue` as {block, k, l}.  One launch
// per direction, so that it reads one direction's occurrence blocks.
template <bool C>
__global__ void __launch_bounds__(kBlockTpb) block_head_kernel(
    DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs, const uint8_t* __restrict__ ok,
    uint32_t n_lists, uint32_t phys, uint32_t max_results, PartState ps, uint4* __restrict__ queue,
    uint32_t* __restrict__ n_queue, uint4* __restrict__ cont, uint32_t* __restrict__ n_cont,
    unsigned long long* census) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_lists) return;
  const uint32_t half = n_lists >> 1;
  const uint32_t list = g < half ? 2 * g : 2 * (g - half) + 1;
  const uint32_t read = list >> 1, strand = list & 1u;
  const uint64_t b0 = offs[read];
  const int len = (int)(offs[read + 1] - b0);
  bool go = false, more = false;
  uint32_t it = 0, k = 0, l = 0;
  int i = 0;
  if (ok[read] && len >= 3 && len <= 32767) {
    int frag = 30;
    const int part = part_on(strand, fragments_of(len, frag), phys);
    if (part >= 0) {
      it = 2 * list + (uint32_t)part;
      ItemOut o;
      o.slot = ps.slots + (uint64_t)it * kBlockSlots;
      o.room = kBlockSlots;
      o.cap = max_results;
      o.n = 0;
      o.read = read;
      o.strand = strand;
      o.refused = false;
      o.sectors = 0;
      const HeadWalk h = head_walk(len, strand, part);
      const uint8_t* W = codes + b0;
      uint32_t gk, gl;
      head_start<C>(X, h, W, i, k, l, gk, gl);
      if (!head_steps<C>(X, h, W, i, k, l, gk, gl, kHeadSteps, o.sectors)) {
        more = true;  // still matching: the rest of the walk in the compacted pass
      } else {
        uint32_t aflag = 0;
        go = head_finish(h, len, o, ps.anchor + it, aflag, i, k, l, gk, gl);
        ps.count[it] = o.n;
        ps.refused[it] = o.refused ? 1 : 0;
        ps.aflag[it] = (uint8_t)aflag;
      }
      if (C) atomicAdd(census, (unsigned long long)o.sectors);
    }
  }
  queue_append(go, queue, n_queue, it, k, l, 0u);
  queue_append(more, cont, n_cont, it, k, l, (uint32_t)i);
}

// The rest of the head walks block_head_kernel compacted: thread g resumes
// cont[g] at its position with its interval (non-empty, so also the last
// non-empty one), ends the walk, and appends the blocks that go on to `queue`.
template <bool C>
__global__ void __launch_bounds__(kBlockTpb) block_head_rest_kernel(
    DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs, const uint4* __restrict__ cont,
    const uint32_t* __restrict__ n_cont, uint32_t max_results, PartState ps, uint4* __restrict__ queue,
    uint32_t* __restrict__ n_queue, unsigned long long* census) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= *n_cont) return;
  const uint4 q = cont[g];
  const uint32_t it = q.x, list = it >> 1, part = it & 1u;
  const uint32_t read = list >> 1, strand = list & 1u;
  const uint64_t b0 = offs[read];
  const int len = (int)(offs[read + 1] - b0);
  ItemOut o;
  o.slot = ps.slots + (uint64_t)it * kBlockSlots;
  o.room = kBlockSlots;
  o.cap = max_results;
  o.n = 0;
  o.read = read;
  o.strand = strand;
  o.refused = false;
  o.sectors = 0;
  const HeadWalk h = head_walk(len, strand, (int)part);
  int i = (int)q.w;
  uint32_t k = q.y, l = q.z, gk = q.y, gl = q.z;
  head_steps<C>(X, h, codes + b0, i, k, l, gk, gl, -1, o.sectors);
  uint32_t aflag = 0;
  const bool go = head_finish(h, len, o, ps.anchor + it, aflag, i, k, l, gk, gl);
  ps.count[it] = o.n;
  ps.refused[it] = o.refused ? 1 : 0;
  ps.aflag[it] = (uint8_t)aflag;
  if (C) atomicAdd(census, (unsigned long long)o.sectors);
  queue_append(go, queue, n_queue, it, k, l, 0u);
}

// BWExactFinalResult{Forward,Backward}'s block rule (search.h:67-155) at the
// start position of an extension, for block 0 (part 0, forward) or the last
// block (part 1, backward); C division truncates toward zero (pos may be -1).
__device__ __forceinline__ bool ext_rule_ok(uint32_t part, int pos, int end, int bs) {
  const int cb = pos / bs;
  if (part == 0) {
    if (!(cb > 0 || pos == end + 1)) {
      if (cb < 0) return false;
      if (pos % bs == 0) return false;
    }
  } else {
    if (!(cb < 0 || pos == -1)) {
      if (cb > 0) return false;
      if ((pos + 1) % bs == 0) return false;
    }
  }
  return true;
}

// Lane modes of the persistent tail.  The first four make one backward-
// extension step per loop iteration; the others are transitions between them.
enum : uint32_t {
  kFirst = 0,   // first walk (restarts and branch points), position i
  kSecond,      // second walk, position i, up to the last branch point
  kExt,         // an extension of a branch (ekind) to the read's end, position ei
  kCStep,       // the branch point's step with base c
  kIdle,        // claim the next queued block
  kFirstEnd,    // the first walk is over
  kExtStart,    // check the block rule and range of an extension starting at ei
  kExtDone,     // an extension ended (esurv: it reached the read's end)
  kCNext,       // the next base of the branch point
  kBranchDone,  // the branch point's extensions are all done
  kFinish       // write the block's counts
};
enum : uint32_t { kExtDel = 0, kExtIns, kExtMis };

// Tail pass over the queued blocks of one direction, persistent: lane g takes
// the queued blocks g, g + G, g + 2G, ... (G lanes in the grid; no claim
// counter, whose atomics serialised on one address when lanes finished blocks
// one by one), runs each as a machine that takes one step per loop iteration
// whatever part of the block it is in (first walk, second walk, a branch
// point's base step or an extension), and starts the next when it is done, so
// a warp's lanes keep stepping together instead of waiting for the block with
// the most branches.  Same walks, branches, order and results as block_tail
// (which the retry pass runs).
template <bool C>
__global__ void __launch_bounds__(kBlockTpb) block_tail_kernel(
    DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs, const uint4* __restrict__ queue,
    const uint32_t* __restrict__ n_queue, uint32_t max_results, PartState ps, unsigned long long* census) {
  const uint32_t nq = *n_queue;
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t next = blockIdx.x * blockDim.x + threadIdx.x;
  // (register pressure: the block's part, strand and read come from `it`; the
  // interval before a branch point's step lives in a, b while the branch runs)
  const uint8_t* W = nullptr;
  int end = 0, frag = 30;
  uint32_t it = 0;
  ItemOut o;
  o.slot = nullptr;
  o.room = kBlockSlots;
  o.cap = max_results;
  o.n = 0;
  o.read = 0;
  o.strand = 0;
  o.refused = false;
  o.sectors = 0;
  uint32_t lane_sectors = 0;
  uint32_t mode = kIdle;
  int i = 0;
  uint32_t a = 0, b = 0;
  uint32_t z = 0, changes = 0, left = 0;
  bool alive = false, failed_step = false, ok_before = false, ok_at = false;
  uint32_t na = 0, nb = 0;
  bool sw_failed = false;
  int bp = 0;
  uint32_t c = 0, wp = 0, rk = 0, rl = 0;
  uint32_t ekind = 0, ea = 0, eb = 0;
  int ei = 0;
  bool esurv = false;
  uint32_t chunk = 0;  // the block's current overflow chunk
  bool lost = false;
  for (;;) {
    // transitions until the lane needs a step
    bool quit = false;
    while (mode >= kIdle) {
      if (mode == kIdle) {
        if (next >= nq) {
          quit = true;
          break;
        }
        const uint4 q = queue[next];
        next += stride;
        it = q.x;
        const uint32_t list = it >> 1, part = it & 1u;
        const uint32_t read = list >> 1;
        const uint64_t b0 = offs[read];
        const int len = (int)(offs[read + 1] - b0);
        W = codes + b0;
        frag = 30;
        fragments_of(len, frag);
        end = len - 1;
        o.slot = ps.slots + (uint64_t)it * kBlockSlots;
        o.n = 0;
        o.refused = false;
        o.sectors = 0;
        lost = false;
        a = q.y;  // the fragment's interval (read again from the queue for the second walk)
        b = q.z;
        z = 0;
        changes = 0;
        alive = true;
        failed_step = false;
        // part 0: the rest of the read after block 0; part 1: block 0 from above
        i = part == 0 ? frag : frag - 1;
        mode = kFirst;
      } else if (mode == kFirstEnd) {
        const uint32_t zt = z & 255u;
        const bool bound_before = zt <= 1u, bound_at = ((zt - 1u) & 255u) <= 1u;
        const uint32_t points = (bound_before ? changes : 0u) + (failed_step && bound_at ? 1u : 0u);
        mode = kFinish;
        if (points > o.cap) {
          o.refused = true;  // rl_next overflows: the block's branches are dropped
        } else if ((it & 1u) == 0 && alive && !emit_tail(o, ps, it, chunk, lost, 1, 0, 0, 0, 0, a, b)) {
          // the complete result of block 0 was refused (a walk that stayed alive
          // never restarted: a, b is its last interval)
        } else if (points) {
          ok_before = bound_before;
          ok_at = bound_at;
          left = points;
          const uint4 q = queue[next - stride];  // the block claimed last
          a = q.y;
          b = q.z;
          i = (it & 1u) == 0 ? frag : frag - 1;
          mode = kSecond;
        }
      } else if (mode == kExtStart) {
        if (!ext_rule_ok(it & 1u, ei, end, frag)) {
          esurv = false;
          mode = kExtDone;
        } else if ((it & 1u) == 0 ? ei > end : ei < 0) {  // nothing left to walk
          esurv = true;
          mode = kExtDone;
        } else {
          mode = kExt;
        }
      } else if (mode == kExtDone) {
        const uint32_t dir = (it & 1u) == 0 ? 1u : 0u;
        if (ekind == kExtDel) {
          if (esurv && !emit_tail(o, ps, it, chunk, lost, dir, 1, HPG_BWT_DELETION, 0xFF, bp, ea, eb)) {
            mode = kFinish;
          } else {
            c = 0;
            mode = kCNext;
          }
        } else if (ekind == kExtIns) {
          if (esurv && !emit_tail(o, ps, it, chunk, lost, dir, 1, HPG_BWT_INSERTION, c, bp, ea, eb)) {
            mode = kFinish;
          } else {
            if (esurv) {  // the mismatch starts from the interval the insertion reached
              rk = ea;
              rl = eb;
            }
            ekind = kExtMis;
            ei = bp + ((it & 1u) == 0 ? 1 : -1);
            ea = rk;
            eb = rl;
            mode = kExtStart;
          }
        } else {
          if (esurv && !emit_tail(o, ps, it, chunk, lost, dir, 1, HPG_BWT_MISMATCH, c, bp, ea, eb)) {
            mode = kFinish;
          } else {
            ++c;
            mode = kCNext;
          }
        }
      } else if (mode == kCNext) {
        while (c < 4 && c == wp) {  // the read's own base: the reference's step whose result it drops
          if (C) o.sectors += (a >> 6) == (b >> 6) ? 1u : 2u;
          ++c;
        }
        mode = c < 4 ? kCStep : kBranchDone;
      } else if (mode == kBranchDone) {
        mode = kFinish;
        if (--left != 0 && !sw_failed) {
          a = na;
          b = nb;
          i += (it & 1u) == 0 ? 1 : -1;
          if ((it & 1u) == 0 ? i <= end : i >= 0) mode = kSecond;
        }
      } else {  // kFinish
        ps.count[it] = o.n;
        ps.refused[it] = o.refused ? 1 : 0;
        ps.lost[it] = lost ? 1 : 0;
        if (C) lane_sectors += o.sectors;
        mode = kIdle;
      }
    }
    if (quit) break;
    // one step
    uint32_t sym, x, y;
    if (mode == kExt) {
      sym = W[ei];
      x = ea;
      y = eb;
    } else if (mode == kCStep) {  // a, b: the interval before the branch point's step
      sym = c;
      x = a;
      y = b;
    } else {
      sym = W[i];
      x = a;
      y = b;
    }
    const View v = (it & 1u) == 0 ? forward_view((it >> 1) & 1u) : backward_view((it >> 1) & 1u);
    step<C>(X, v, sym, x, y, o.sectors);
    const int dstep = (it & 1u) == 0 ? 1 : -1;
    if (mode == kFirst) {
      const int64_t before = (int64_t)b - (int64_t)a;
      if (alive) {
        if (x > y) {
          alive = false;
          failed_step = true;  // the step that empties the interval changes its size
        } else if ((int64_t)y - (int64_t)x != before) {
          ++changes;
        }
      }
      bool over = false;
      if (x > y) {
        a = 0;
        b = X.top;
        ++z;
        // three restarts with too few steps left for the byte count to wrap: D
        // allows no error anywhere in the range, so there is no branch point
        if (z >= 3 && z + (uint32_t)(dstep > 0 ? end - i : i) < 256) over = true;
      } else {
        a = x;
        b = y;
      }
      i += dstep;
      if (over || (dstep > 0 ? i > end : i < 0)) mode = kFirstEnd;
    } else if (mode == kSecond) {
      const bool failed = x > y;
      const bool changed = failed || (int64_t)y - (int64_t)x != (int64_t)b - (int64_t)a;
      if (changed && (failed ? ok_at : ok_before)) {  // a branch point: its extensions, then on
        na = x;
        nb = y;
        sw_failed = failed;
        bp = i;  // a, b stay the interval before the step for the branch
        wp = W[i];
        ekind = kExtDel;
        ei = i + dstep;
        ea = a;
        eb = b;
        mode = kExtStart;
      } else if (failed) {
        mode = kFinish;
      } else {
        a = x;
        b = y;
        i += dstep;
        if (dstep > 0 ? i > end : i < 0) mode = kFinish;
      }
    } else if (mode == kExt) {
      if (x > y) {
        esurv = false;
        mode = kExtDone;
      } else {
        ea = x;
        eb = y;
        ei += dstep;
        if (dstep > 0 ? ei > end : ei < 0) {
          esurv = true;
          mode = kExtDone;
        }
      }
    } else {  // kCStep
      if (x > y) {
        ++c;
        mode = kCNext;
      } else {
        rk = x;
        rl = y;
        ekind = kExtIns;
        ei = bp;
        ea = x;
        eb = y;
        mode = kExtStart;
      }
    }
  }
  if (C) atomicAdd(census, (unsigned long long)lane_sectors);
}

// Retry: block items[g] = 2 * list + part, whose results did not fit its
// slots, runs again (head and tail) into the list's final range, the last
// block after block 0's results and cut to the room they left.
__global__ void __launch_bounds__(kBlockTpb) block_retry_kernel(
    DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs, uint32_t n_items,
    const uint32_t* __restrict__ items, uint32_t max_results, PartState ps, const uint64_t* __restrict__ list_off,
    hpg_hit_t* __restrict__ hits) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_items) return;
  const uint32_t it = items[g], list = it >> 1, part = it & 1u;
  const uint32_t read = list >> 1, strand = list & 1u;
  const uint64_t b0 = offs[read];
  const int len = (int)(offs[read + 1] - b0);
  const uint32_t n0 = ps.count[2 * list];
  const uint32_t room1 = max_results - n0;
  const uint32_t m1 = ps.count[2 * list + 1] < room1 ? ps.count[2 * list + 1] : room1;
  ItemOut o;
  o.slot = hits + list_off[list] + (part ? n0 : 0u);
  o.room = part ? m1 : n0;
  o.cap = max_results;
  o.n = 0;
  o.read = read;
  o.strand = strand;
  o.refused = false;
  o.sectors = 0;
  uint32_t aflag = 0, k = 0, l = 0;
  if (block_head<false>(X, codes + b0, len, strand, (int)part, o, nullptr, aflag, k, l))
    block_tail<false>(X, codes + b0, len, strand, (int)part, o, k, l);
}

// The two blocks of each list as BWSearchCPU leaves them in one list: block
// 0's results, then the last block's up to the capacity (a full list refuses
// the rest); both anchors, except the last block's when the lists have no room
// at all and block 0 matched (BWSearchCPU returned before the last block).
// Blocks whose results do not fit their slots are appended to `retry`
// (any order: each writes a fixed range).
__global__ void block_merge_kernel(PartState ps, uint32_t n_lists, uint32_t max_results, uint32_t* __restrict__ count,
                                   uint8_t* __restrict__ refused, hpg_block_anchor_t* __restrict__ anchors,
                                   uint8_t* __restrict__ n_anchors, uint32_t* __restrict__ retry,
                                   uint32_t* __restrict__ n_retry) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_lists) return;
  const uint32_t n0 = ps.count[2 * t], n1 = ps.count[2 * t + 1];
  const uint32_t room1 = max_results - n0;
  const uint32_t m1 = n1 < room1 ? n1 : room1;
  count[t] = n0 + m1;
  if (n0 > kBlockSlots && ps.lost[2 * t]) retry[atomicAdd(n_retry, 1u)] = 2 * t;
  if (m1 > kBlockSlots && ps.lost[2 * t + 1]) retry[atomicAdd(n_retry, 1u)] = 2 * t + 1;
  refused[t] = (ps.refused[2 * t] | ps.refused[2 * t + 1] | (n1 > room1 ? 1 : 0)) ? 1 : 0;
  const uint32_t f0 = ps.aflag[2 * t], f1 = ps.aflag[2 * t + 1];
  uint32_t na = 0;
  if (f0 & 1u) anchors[2ull * t + na++] = ps.anchor[2 * t];
  if ((f1 & 1u) && !(max_results == 0 && (f0 & 2u))) anchors[2ull * t + na++] = ps.anchor[2 * t + 1];
  n_anchors[t] = (uint8_t)na;
}

// The first pass's slots of each list, packed at its scanned offset.
__global__ void block_pack_kernel(PartState ps, const uint64_t* __restrict__ off, uint32_t n_lists,
                                  uint32_t max_results, hpg_hit_t* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_lists) return;
  const uint32_t n0 = ps.count[2 * t], n1 = ps.count[2 * t + 1];
  const uint32_t room1 = max_results - n0;
  const uint32_t m1 = n1 < room1 ? n1 : room1;
  hpg_hit_t* dst = out + off[t];
  for (uint32_t part = 0; part < 2; ++part) {  // a lost block's range is written by the retry pass
    const uint32_t b = 2 * t + part, m = part ? m1 : n0;
    hpg_hit_t* d = dst + (part ? n0 : 0u);
    const uint32_t c = m < kBlockSlots ? m : kBlockSlots;
    for (uint32_t j = 0; j < c; ++j) d[j] = ps.slots[(uint64_t)b * kBlockSlots + j];
    if (m <= kBlockSlots || ps.lost[b]) continue;
    uint32_t ch = ps.ovf_head[b];
    for (uint32_t j = kBlockSlots; j < m; ++j) {
      const uint32_t o = (j - kBlockSlots) % kOvfChunk;
      if (o == 0 && j > kBlockSlots) ch = ps.ovf_next[ch];
      d[j] = ps.ovf_hits[(uint64_t)ch * kOvfChunk + o];
    }
  }
}

// Rows of each hit for the locate pass: l - k + 1, or 0 for every hit of a
// (read, strand) list whose rows pass the locate limit (that list's flag bit 1).
__global__ void block_rows_kernel(const hpg_hit_t* __restrict__ hits, const uint32_t* __restrict__ count,
                                  const uint64_t* __restrict__ off, uint32_t n_items, uint64_t limit,
                                  uint32_t* __restrict__ hit_rows, uint8_t* __restrict__ flags) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const uint64_t h0 = off[t], h1 = h0 + count[t];
  uint64_t rows = 0;
  for (uint64_t h = h0; h < h1; ++h) rows += (uint64_t)(hits[h].l - hits[h].k + 1);
  const bool over = limit && rows > limit;
  for (uint64_t h = h0; h < h1; ++h) hit_rows[h] = over ? 0u : (uint32_t)(hits[h].l - hits[h].k + 1);
  if (over) flags[t] |= 2;
}

// One locate item per row: row r belongs to the hit whose row range holds it
// (binary search over the scanned row counts; empty ranges are never chosen).
// len_calc as bwt.c:2497-2510: the read length, one less for a DELETION, one
// more for an INSERTION; the direction is dir, flipped on the '-' strand.
__global__ void block_items_kernel(const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ row_off,
                                   uint32_t n_hits, uint64_t n_rows, const uint64_t* __restrict__ offs,
                                   RowItem* __restrict__ items) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
       r += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = n_hits;  // last h with row_off[h] <= r
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (row_off[mid] <= r) lo = mid;
      else hi = mid;
    }
    const hpg_hit_t x = hits[lo];
    uint32_t len = (uint32_t)(offs[x.read + 1] - offs[x.read]);
    const uint32_t err = x.nm ? x.err_kind : 0u;
    if (err == HPG_BWT_DELETION) --len;
    else if (err == HPG_BWT_INSERTION) ++len;
    RowItem it;
    it.row = (uint32_t)(x.k + (int64_t)(r - row_off[lo]));
    it.hit = lo;
    it.out = (uint32_t)r;
    it.phys_len = ((uint32_t)(x.dir ^ x.strand) << 31) | (len & kRowLenMask);
    items[r] = it;
  }
}

unsigned grid_of(size_t n) { return (unsigned)((n + kBlockTpb - 1) / kBlockTpb); }

// The search of every (read, strand) of the uploaded batch; on return the
// device holds the packed hits (e->hits), per-list counts (e->rs_count) and
// hit offsets (e->hit_off), refused flags (e->rs_trunc), anchors (e->vecs)
// and anchor counts (e->ovf); list counts also on the host.  Per-block state
// lives in the batched form's buffers (b_arr, b_sorted, b_seg, b_res), unused
// between calls.
int block_search_device(Engine* e, size_t n, uint32_t max_results, uint64_t* total_out, std::string* err) {
  const size_t T = 2 * n, P = 4 * n;
  if (!ensure(e, e->b_res, P * kBlockSlots * sizeof(hpg_hit_t) + 16) || !ensure(e, e->b_arr, P * 4 + 16) ||
      !ensure(e, e->b_sorted, 3 * P + 16) || !ensure(e, e->b_seg, P * sizeof(hpg_block_anchor_t) + 16) ||
      !ensure(e, e->rs_count, T * 4 + 16) || !ensure(e, e->rs_trunc, T + 16) || !ensure(e, e->hit_off, (T + 1) * 8) ||
      !ensure(e, e->scan_part, scan_parts(T) * 8) || !ensure(e, e->vecs, 2 * T * sizeof(hpg_block_anchor_t) + 16) ||
      !ensure(e, e->ovf, T + 16) || !ensure(e, e->census, 16) || !ensure(e, e->rows, P * 4 + 16) ||
      !ensure(e, e->b_ctr, 64) || !ensure(e, e->b_spill, T * sizeof(uint4) + 16)) {
    *err = oom_message("block search", P * (kBlockSlots * sizeof(hpg_hit_t) + 2 * sizeof(hpg_block_anchor_t) + 16));
    return -1;
  }
  cudaStream_t s = e->stream;
  PartState ps;
  ps.slots = ptr<hpg_hit_t>(e->b_res);
  ps.count = ptr<uint32_t>(e->b_arr);
  ps.refused = ptr<uint8_t>(e->b_sorted);
  ps.aflag = ps.refused + P;
  ps.anchor = ptr<hpg_block_anchor_t>(e->b_seg);
  ps.lost = ps.refused + 2 * P;
  // overflow pool: four results a read in chunks, heads per block, a chunk chain
  const uint32_t ovf_cap = (uint32_t)std::min<size_t>(n / 8 + 1024, 0x7FFFFFFFu);
  const size_t ovf_bytes = (size_t)ovf_cap * (kOvfChunk * sizeof(hpg_hit_t) + 4) + P * 4 + T * sizeof(uint4) + 64;
  if (!ensure(e, e->b_bovf, ovf_bytes)) {
    *err = oom_message("block search overflow pool", ovf_bytes);
    return -1;
  }
  ps.ovf_hits = ptr<hpg_hit_t>(e->b_bovf);
  ps.ovf_next = reinterpret_cast<uint32_t*>(ps.ovf_hits + (size_t)ovf_cap * kOvfChunk);
  ps.ovf_head = ps.ovf_next + ovf_cap;
  // the head walks going on past their first steps (one direction at a time)
  uint4* cont = reinterpret_cast<uint4*>(
      (reinterpret_cast<uintptr_t>(ps.ovf_head + P) + 15) & ~static_cast<uintptr_t>(15));
  ps.ovf_ctr = ptr<uint32_t>(e->b_ctr) + 14;
  ps.ovf_cap = ovf_cap;
  uint32_t* n_retry = ptr<uint32_t>(e->b_ctr) + 12;
  cudaMemsetAsync(ps.count, 0, P * 4, s);
  cudaMemsetAsync(ps.refused, 0, 3 * P, s);
  cudaMemsetAsync(ps.ovf_ctr, 0, 4, s);
  cudaMemsetAsync(n_retry, 0, 4, s);
  uint32_t* d_count = ptr<uint32_t>(e->rs_count);
  uint64_t* d_off = ptr<uint64_t>(e->hit_off);
  unsigned long long* census = e->census_on ? ptr<unsigned long long>(e->census) : nullptr;
  if (census) cudaMemsetAsync(census, 0, 8, s);
  const uint8_t* codes = ptr<uint8_t>(e->codes);
  const uint64_t* offs = ptr<uint64_t>(e->offs);
  const uint8_t* ok = ptr<uint8_t>(e->ok);
  uint4* queue = ptr<uint4>(e->b_spill);
  uint32_t* n_queue = ptr<uint32_t>(e->b_ctr) + 13;
  // the tail is persistent: as many blocks as fit, at most one lane per list
  int per_sm = 0;
  if (census)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, block_tail_kernel<true>, kBlockTpb, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, block_tail_kernel<false>, kBlockTpb, 0);
  const unsigned tail_grid = std::max(1u, std::min(grid_of(T), (unsigned)(std::max(per_sm, 1) * e->num_sms)));
  cudaEventRecord(e->cev[0], s);
  uint32_t* n_cont = n_queue + 2;
  for (uint32_t phys = 0; phys < 2; ++phys) {  // per index direction: head, the heads' rest, tail
    cudaMemsetAsync(n_queue, 0, 4, s);
    cudaMemsetAsync(n_cont, 0, 4, s);
    count_launches(3);
    if (census) {
      block_head_kernel<true><<<grid_of(T), kBlockTpb, 0, s>>>(e->X, codes, offs, ok, (uint32_t)T, phys, max_results,
                                                               ps, queue, n_queue, cont, n_cont, census);
      block_head_rest_kernel<true><<<grid_of(T), kBlockTpb, 0, s>>>(e->X, codes, offs, cont, n_cont, max_results, ps,
                                                                    queue, n_queue, census);
      block_tail_kernel<true><<<tail_grid, kBlockTpb, 0, s>>>(e->X, codes, offs, queue, n_queue, max_results, ps,
                                                              census);
    } else {
      block_head_kernel<false><<<grid_of(T), kBlockTpb, 0, s>>>(e->X, codes, offs, ok, (uint32_t)T, phys,
                                                                max_results, ps, queue, n_queue, cont, n_cont,
                                                                nullptr);
      block_head_rest_kernel<false><<<grid_of(T), kBlockTpb, 0, s>>>(e->X, codes, offs, cont, n_cont, max_results,
                                                                     ps, queue, n_queue, nullptr);
      block_tail_kernel<false><<<tail_grid, kBlockTpb, 0, s>>>(e->X, codes, offs, queue, n_queue, max_results, ps,
                                                               nullptr);
    }
  }
  cudaEventRecord(e->cev[1], s);
  count_launches(1);
  block_merge_kernel<<<grid_of(T), kBlockTpb, 0, s>>>(ps, (uint32_t)T, max_results, d_count, ptr<uint8_t>(e->rs_trunc),
                                                      ptr<hpg_block_anchor_t>(e->vecs), ptr<uint8_t>(e->ovf),
                                                      ptr<uint32_t>(e->rows), n_retry);
  launch_scan(d_count, T, d_off, ptr<uint64_t>(e->scan_part), s);
  uint64_t total = 0;
  uint32_t again = 0;
  HPG_CUDA(cudaMemcpyAsync(&total, d_off + T, 8, cudaMemcpyDeviceToHost, s), "block total");
  HPG_CUDA(cudaMemcpyAsync(&again, n_retry, 4, cudaMemcpyDeviceToHost, s), "block retries");
  if (census) HPG_CUDA(cudaMemcpyAsync(&e->census_val, census, 8, cudaMemcpyDeviceToHost, s), "block census");
  HPG_CUDA(cudaStreamSynchronize(s), "block search");
  float ms = 0;
  cudaEventElapsedTime(&ms, e->cev[0], e->cev[1]);
  e->block_ms = ms;
  if (!ensure(e, e->hits, (total + 1) * sizeof(hpg_hit_t))) {
    *err = oom_message("block search results", (total + 1) * sizeof(hpg_hit_t));
    return -1;
  }
  hpg_hit_t* d_hits = ptr<hpg_hit_t>(e->hits);
  count_launches(1);
  block_pack_kernel<<<grid_of(T), kBlockTpb, 0, s>>>(ps, d_off, (uint32_t)T, max_results, d_hits);
  if (again) {  // blocks with more results than slots: the same search again, into their final ranges
    cudaEventRecord(e->cev[0], s);
    count_launches(1);
    block_retry_kernel<<<grid_of(again), kBlockTpb, 0, s>>>(e->X, codes, offs, again, ptr<uint32_t>(e->rows),
                                                            max_results, ps, d_off, d_hits);
    cudaEventRecord(e->cev[1], s);
    HPG_CUDA(cudaStreamSynchronize(s), "block search retry");
    cudaEventElapsedTime(&ms, e->cev[0], e->cev[1]);
    e->block_ms += ms;
  }
  *total_out = total;
  return 0;
}

int check_block_args(size_t n, std::string* err) {
  if (n >= (1ull << 30)) {
    *err = "too many reads in one block search";
    return -1;
  }
  return 0;
}

}  // namespace

int engine_block_search(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t max_results,
                        BlockSearchOut* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  out->hits.clear();
  out->count.assign(2 * n, 0);
  out->refused.assign(2 * n, 0);
  out->anchors.assign(4 * n, hpg_block_anchor_t{});
  out->n_anchors.assign(2 * n, 0);
  out->kernel_ms = 0;
  if (!n) return 0;
  if (check_block_args(n, err) != 0 || upload_reads(e, seqs, offs, n, err) != 0) return -1;
  uint64_t total = 0;
  if (block_search_device(e, n, max_results, &total, err) != 0) return -1;
  const size_t T = 2 * n;
  cudaStream_t s = e->stream;
  HPG_CUDA(cudaMemcpyAsync(out->count.data(), e->rs_count.p, T * 4, cudaMemcpyDeviceToHost, s), "block counts");
  out->hits.resize(total);
  if (total)
    HPG_CUDA(cudaMemcpyAsync(out->hits.data(), e->hits.p, total * sizeof(hpg_hit_t), cudaMemcpyDeviceToHost, s),
             "block results");
  HPG_CUDA(cudaMemcpyAsync(out->refused.data(), e->rs_trunc.p, T, cudaMemcpyDeviceToHost, s), "block flags");
  HPG_CUDA(cudaMemcpyAsync(out->anchors.data(), e->vecs.p, 2 * T * sizeof(hpg_block_anchor_t),
                           cudaMemcpyDeviceToHost, s),
           "block anchors");
  HPG_CUDA(cudaMemcpyAsync(out->n_anchors.data(), e->ovf.p, T, cudaMemcpyDeviceToHost, s), "block anchor counts");
  HPG_CUDA(cudaStreamSynchronize(s), "block search results");
  out->kernel_ms = e->block_ms;
  return 0;
}

int engine_block_search_result(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t max_results,
                               hpg_result_set_t* out, hpg_block_anchor_t* anchors, uint8_t* n_anchors,
                               std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  std::memset(out, 0, sizeof(*out));
  out->n_reads = n;
  const size_t T = 2 * n;
  uint64_t total = 0;
  if (n) {
    if (check_block_args(n, err) != 0 || upload_reads(e, seqs, offs, n, err) != 0) return -1;
    if (block_search_device(e, n, max_results, &total, err) != 0) return -1;
  }
  cudaStream_t s = e->stream;
  // rows of every hit (lists over the locate limit: none), their items, the locate pass
  uint64_t n_rows = 0;
  if (total) {
    if (total >= 0xFFFFFFFFull) {
      *err = "too many block search results in one call";
      return -1;
    }
    if (!ensure(e, e->ovf_count, total * 4 + 16) || !ensure(e, e->loc_off, (total + 1) * 8) ||
        !ensure(e, e->scan_part, std::max(scan_parts(total), scan_parts(T)) * 8)) {
      *err = oom_message("block search rows", total * 12);
      return -1;
    }
    count_launches(1);
    block_rows_kernel<<<grid_of(T), kBlockTpb, 0, s>>>(ptr<hpg_hit_t>(e->hits), ptr<uint32_t>(e->rs_count),
                                                       ptr<uint64_t>(e->hit_off), (uint32_t)T, e->locate_limit,
                                                       ptr<uint32_t>(e->ovf_count), ptr<uint8_t>(e->rs_trunc));
    launch_scan(ptr<uint32_t>(e->ovf_count), total, ptr<uint64_t>(e->loc_off), ptr<uint64_t>(e->scan_part), s);
    HPG_CUDA(cudaMemcpyAsync(&n_rows, ptr<uint64_t>(e->loc_off) + total, 8, cudaMemcpyDeviceToHost, s), "row total");
    HPG_CUDA(cudaStreamSynchronize(s), "block rows");
    if (n_rows > kMaxLocateRows) {
      *err = "block search: " + std::to_string(n_rows) + " rows to locate in one call (set a locate limit)";
      return -1;
    }
    if (n_rows) {
      if (!ensure(e, e->b_rowhit, n_rows * sizeof(RowItem) + 16) ||
          !ensure(e, e->locs, n_rows * sizeof(hpg_loc_t) + 16) || !ensure(e, e->b_ctr, 64)) {
        *err = oom_message("block search locate", n_rows * (sizeof(RowItem) + sizeof(hpg_loc_t)));
        return -1;
      }
      const uint64_t blocks = std::min<uint64_t>((n_rows + kBlockTpb - 1) / kBlockTpb, (uint64_t)e->num_sms * 16);
      count_launches(1);
      block_items_kernel<<<(unsigned)blocks, kBlockTpb, 0, s>>>(ptr<hpg_hit_t>(e->hits), ptr<uint64_t>(e->loc_off),
                                                               (uint32_t)total, n_rows, ptr<uint64_t>(e->offs),
                                                               static_cast<RowItem*>(e->b_rowhit.p));
      launch_locate_items(e->X, static_cast<const RowItem*>(e->b_rowhit.p), n_rows, ptr<hpg_loc_t>(e->locs),
                          ptr<unsigned int>(e->b_ctr) + 5, e->num_sms, s);
    }
  }
  out->hits = (hpg_hit_t*)host_pool_alloc((total + 1) * sizeof(hpg_hit_t));
  out->locs = (hpg_loc_t*)host_pool_alloc((n_rows + 1) * sizeof(hpg_loc_t));
  out->rs_count = (uint32_t*)host_pool_alloc((T + 1) * 4);
  out->rs_truncated = (uint8_t*)host_pool_alloc(T + 1);
  if (!out->hits || !out->locs || !out->rs_count || !out->rs_truncated) {
    *err = "out of host memory (block search results)";
    return -1;
  }
  out->n_hits = total;
  out->n_locs = n_rows;
  if (T) {
    HPG_CUDA(cudaMemcpyAsync(out->rs_count, e->rs_count.p, T * 4, cudaMemcpyDeviceToHost, s), "block counts");
    HPG_CUDA(cudaMemcpyAsync(out->rs_truncated, e->rs_trunc.p, T, cudaMemcpyDeviceToHost, s), "block flags");
    if (anchors)
      HPG_CUDA(cudaMemcpyAsync(anchors, e->vecs.p, 2 * T * sizeof(hpg_block_anchor_t), cudaMemcpyDeviceToHost, s),
               "block anchors");
    if (n_anchors) HPG_CUDA(cudaMemcpyAsync(n_anchors, e->ovf.p, T, cudaMemcpyDeviceToHost, s), "anchor counts");
  }
  if (total)
    HPG_CUDA(cudaMemcpyAsync(out->hits, e->hits.p, total * sizeof(hpg_hit_t), cudaMemcpyDeviceToHost, s),
             "block results");
  if (n_rows)
    HPG_CUDA(cudaMemcpyAsync(out->locs, e->locs.p, n_rows * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, s),
             "located rows");
  HPG_CUDA(cudaStreamSynchronize(s), "block search results");
  uint32_t derr = 0;
  HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
  if (derr) {
    cudaMemset(e->d_err, 0, 4);
    *err = "corrupt index: suffix-array walk did not reach a sampled row";
    return -1;
  }
  return 0;
}

float engine_block_ms(Engine* e) { return e->block_ms; }

}  // namespace hpgbwt
