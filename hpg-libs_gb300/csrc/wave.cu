// wave.cu -- warp-cooperative form of the batched BWSearch1 search: the
// vector searches (chains) of bwt.c:1940-1950 and the 1-error helper's
// branches (search/search.c:1491-1709).
//
// The warp, not the lane, is the unit that owns reads.  A warp claims a group
// of consecutive reads from the batch counter and stages their bases in
// shared memory as 2-bit codes, 16 to a word, with one coalesced copy; while
// staging, each lane also forms the start-table index of its read's chains.
// Its lanes then run the group's chains and the helper's branches: one
// backward-extension step per lane per loop iteration, and nothing else, so
// every lane of the warp executes the same instructions (the only branch is at
// an item's end).  A change point (a position where the interval size
// changes) goes on the warp's stack; idle lanes take it apart into its eight
// continuations (listed at wave_branch_kernel below), each a walk over the
// staged bases that is the same loop as a chain with no branching window.
// Change points that find the stack full go to the device queue for
// wave_branch_kernel; the j = 1 / j = n-1 blocks, whose results depend on one
// another, go to a list that the fused kernel's drain maps.
//
// Lanes whose item ended wait, masked, until `batch_idle` lanes of the warp
// have (or all have); then the whole warp, converged, hands out work in one
// pass: eight lanes per stacked change point, then the next chains of its
// staged groups.  Handing out a chain includes its start-table lookup, so a
// chain that fails within its first steps (a read searched on its wrong
// strand) is replaced at once, without entering the step loop.  When the
// staged chains run out, the warp stages its next group into whichever of its
// two buffers has no work left alive.
//
// A group buffer holds 4096 bases.  A claimed group that does not fit is
// staged in parts; a single read that does not fit at all (more than about
// 4064 bases) is left to the fused kernel: the launch that runs the
// backward-index chains (or all chains) appends it to a list that one launch
// of the fused kernel then maps, all four chains.
//
// The emission order keys and the chunked result slots are those of the fused
// kernel (batched.cu), so the finalize kernels are shared and the results are
// identical.
#include <cuda_runtime.h>

#include "batched.cuh"
#include "batched_dev.cuh"
#include "kernels.cuh"

namespace hpgbwt {

namespace {

using namespace bdev;

constexpr int kWBlock = 128;
constexpr int kWWarps = kWBlock / 32;
constexpr uint32_t kHalfWords = 256;              // packed words per group buffer
constexpr uint32_t kHalfBases = kHalfWords * 16;  // 4096 bases
constexpr uint32_t kWarpStack = 32;               // change points per warp stack
constexpr unsigned kFull = 0xFFFFFFFFu;

struct WarpShared {
  uint32_t words[2 * kHalfWords];  // the two group buffers; base i at bits 2(i & 15) of word i >> 4
  uint32_t slot[2][32];            // per read of a group: start of the read in its buffer | len << 16; 0 = no chains
  uint32_t kcode[2][64];           // per chain of a group: its start-table index
  uint32_t first_read[2];
  uint32_t n_chains[2];
  uint32_t handed[2];
  int live[2];                     // work items of the group alive: chains, stacked change points, walks
  uint32_t pend_first, pend_n;     // claimed reads not staged yet
  uint32_t done;                   // the batch counter is exhausted
  SpillEntry stk[kWarpStack];      // change points; jtype = J | type << 16 | (buffer << 5 | slot) << 18
  unsigned top;
};

__device__ __forceinline__ uint32_t base_at(const WarpShared& ws, uint32_t i) {
  return (ws.words[i >> 4] >> ((i & 15u) << 1)) & 3u;
}

// Codes of bases i .. i+n-1 (n <= 12) of the staged stream, base i in the low bits.
__device__ __forceinline__ uint32_t bases_at(const WarpShared& ws, uint32_t i, uint32_t n) {
  const uint32_t sh = (i & 15u) << 1;
  uint32_t x = ws.words[i >> 4] >> sh;
  if (sh + 2 * n > 32) x |= ws.words[(i >> 4) + 1] << (32 - sh);
  return x & ((1u << (2 * n)) - 1u);
}

// Reverse the order of the n 2-bit groups of x (1 <= n <= 12).
__device__ __forceinline__ uint32_t rev2(uint32_t x, uint32_t n) {
  const uint32_t r = __brev(x) >> (32 - 2 * n);
  return ((r & 0x55555555u) << 1) | ((r >> 1) & 0x55555555u);
}

// Four 8-bit codes (0..3) of a little-endian word packed into 8 bits.
__device__ __forceinline__ uint32_t pack4(uint32_t x) {
  return (x & 3u) | ((x >> 6) & 0xCu) | ((x >> 12) & 0x30u) | ((x >> 18) & 0xC0u);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(kFull, (uint32_t)v, src), hi = __shfl_sync(kFull, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// One backward-extension step (BWiteration, search/runtime.h:38-42) with the
// item's physical direction hoisted: `occ` and `dollar` of that direction and
// `cperm` the permutation of query symbols (complement on the '-' strand).
__device__ __forceinline__ void wave_step(const DevIndex& X, const OccBlock* occ, uint32_t dollar, uint32_t cperm,
                                          uint32_t b, uint32_t& k, uint32_t& l) {
  const uint32_t ph = (cperm >> (2u * b)) & 3u;
  const uint32_t q0 = k >> 6, q1 = l >> 6;
  uint32_t cnt[4];
  uint4 bits;
  load_block_m(occ + q0, X.load_mode, cnt, bits);
  uint64_t mm = match_mask(bits, ph);
  const uint32_t c0 = sel4(cnt, ph);
  uint32_t rk = c0 + (uint32_t)__popcll(mm & row_mask(k & 63));
  uint32_t rl;
  if (q1 == q0) {
    rl = c0 + (uint32_t)__popcll(mm & row_mask((l & 63) + 1));
  } else {
    load_block_m(occ + q1, X.load_mode, cnt, bits);
    mm = match_mask(bits, ph);
    rl = sel4(cnt, ph) + (uint32_t)__popcll(mm & row_mask((l & 63) + 1));
  }
  if (ph == 0) {  // the '$' row is stored as code 0 in its block
    if (k > dollar && q0 == (dollar >> 6)) rk -= 1;
    if (l >= dollar && q1 == (dollar >> 6)) rl -= 1;
  }
  const uint32_t cc = sel4(X.C, ph);  // C1 = C + 1 (checked when the index is loaded)
  k = cc + 1u + rk;
  l = cc + rl;
}

template <int MINB, bool CENSUS>
__global__ void __launch_bounds__(kWBlock, MINB) wave_search_kernel(DevIndex X, BatchedParams p) {
  __shared__ WarpShared wsh[kWWarps];
  __shared__ uint32_t c_res[kWBlock], c_spl[kWBlock], c_gs[kWBlock], c_key[kWBlock], c_meta[kWBlock];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  WarpShared& ws = wsh[tid >> 5];
  const uint32_t n_reads = p.n_reads_dev ? *p.n_reads_dev : p.n_reads;
  // part 0: the chains on the backward index ('+' backward, '-' forward), 1: those
  // on the forward index ('+' forward, '-' backward), 2: all four
  const uint32_t part = p.dir_split == 2 ? 0u : (p.dir_split == 3 ? 1u : 2u);
  const uint32_t cpr_shift = part == 2 ? 2u : 1u;  // chains per read: 4 or 2
  unsigned int* group_ctr = part == 1 ? p.chain_ctr2 : p.chain_ctr;
  const uint32_t G = p.wave_group < 1 ? 1u : (p.wave_group > 32 ? 32u : p.wave_group);
  const uint32_t L = X.kmer_len;
  // staging reads codes below both the batch's end and the buffer's size (offsets that
  // fail validation mark their reads as not ok, but may point anywhere)
  const uint64_t total_bases = min(p.offs[n_reads], p.codes_len);
  c_res[tid] = 0;
  c_spl[tid] = 0;
  c_gs[tid] = 0;
  if (lane == 0) {
    ws.pend_first = 0;
    ws.pend_n = 0;
    ws.done = 0;
    ws.top = 0;
    for (int h = 0; h < 2; ++h) {
      ws.n_chains[h] = 0;
      ws.handed[h] = 0;
      ws.live[h] = 0;
    }
  }
  __syncwarp();

  // lane state: the chain or branch walk being searched
  bool active = false;
  uint32_t rs = 0;      // 2 * read + strand
  uint32_t rbase = 0;   // position of the read's base 0 in the warp's staged stream
  int len = 0;
  uint32_t k = 0, l = 0, pk = 0, pl = 0;  // interval after / before the last step
  int pos = 0, dir = 0;                   // read position of the step's base; -1 backward, +1 forward
  uint32_t nb = 0;                        // base of the next step
  uint32_t win = 0;  // first J where the helper branches | how many J (<< 16); bit 31: a branch walk
  // the item's physical index direction, hoisted out of the step
  const OccBlock* occ = nullptr;
  uint32_t dollar = 0, cperm = 0;
  uint32_t sectors = 0;

  auto W = [&](int i) -> uint32_t { return base_at(ws, rbase + (uint32_t)i); };
  auto item_done = [&]() {
    active = false;
    atomicSub(&ws.live[c_gs[tid] >> 5], 1);
  };
  // A change point for the device queue (wave_branch_kernel), in chunks of slots.
  auto spill_cp = [&](uint32_t a, uint32_t b, uint32_t jt) {
    uint32_t cs = c_spl[tid];
    unsigned left = cs >> 28;
    if (left == 0) {
      cs = claim(p.spill_tail, kResChunk);
      left = kResChunk;
      if (cs >= (1u << 28)) {  // beyond what the packed form holds: single slots
        c_spl[tid] = 0;
        const unsigned q = claim(p.spill_tail, 1);
        if (q < p.spill_cap) p.spill[q] = SpillEntry{a, b, rs, jt};
        else atomicOr(p.status, kStatusSpillFull);
        return;
      }
    }
    const unsigned q = cs & 0x0FFFFFFFu;
    c_spl[tid] = (q + 1) | ((left - 1) << 28);
    if (q < p.spill_cap) p.spill[q] = SpillEntry{a, b, rs, jt};
    else atomicOr(p.status, kStatusSpillFull);
  };
  // A change point found by this lane's chain: blocks to the block list; the
  // others onto the warp's stack, or the device queue when the stack is full.
  auto push_cp = [&](uint32_t a, uint32_t b, uint32_t jt) {
    if ((jt >> 16) >= kBlk1) {
      const unsigned q = atomicAdd(p.block_n, 1u);
      if (q < p.block_cap) p.blocks[q] = SpillEntry{a, b, rs, jt};
      else atomicOr(p.status, kStatusSpillFull);
      return;
    }
    const uint32_t gs = c_gs[tid];
    const unsigned q = atomicAdd(&ws.top, 1u);
    if (q < kWarpStack) {
      ws.stk[q] = SpillEntry{a, b, rs, jt | (gs << 18)};
      atomicAdd(&ws.live[gs >> 5], 1);
    } else {
      spill_cp(a, b, jt);
    }
  };
  // Continuation `item` (0..7) of stacked change point e, a walk over the staged
  // bases (the eight items as listed at wave_branch_kernel).
  auto start_walk = [&](const SpillEntry& e, uint32_t item) {
    const uint32_t gs = (e.jtype >> 18) & 63u, h = gs >> 5;
    c_gs[tid] = gs;
    const uint32_t si = ws.slot[h][gs & 31u];
    rs = e.rs;
    const uint32_t strand = rs & 1u;
    len = (int)(si >> 16);
    rbase = h * kHalfBases + (si & 0xFFFFu);
    const int J = (int)(e.jtype & 0xFFFFu);
    const bool bwd = ((e.jtype >> 16) & 3u) == kCpBwd;
    dir = bwd ? -1 : 1;
    const uint32_t d = (bwd ? 0u : 1u) ^ strand;
    occ = d ? X.dir[1].occ : X.dir[0].occ;
    dollar = d ? X.dir[1].dollar : X.dir[0].dollar;
    cperm = strand ? X.comp_packed : 0xE4u;
    k = pk = e.k;
    l = pl = e.l;
    win = 1u << 31;
    uint32_t slot, kind, basev;
    if (item == 0) {  // deletion: over W[J-2..0] (forward W[J+2..n])
      pos = J + 2 * dir;
      nb = W(pos);
      slot = 0;
      kind = 1;
      basev = 0xFFu;
    } else if (item <= 4) {  // insertion of b: one step with b, then W[J-1..0]
      const uint32_t b = item - 1;
      pos = J;
      nb = b;
      slot = 1 + 2 * b;
      kind = 3;
      basev = b;
    } else {  // mismatch with b != W[J-1]: one step with b, then W[J-2..0]
      const uint32_t w = W(J + dir);
      const uint32_t b = (item - 5) + ((item - 5) >= w ? 1u : 0u);
      pos = J + dir;
      nb = b;
      slot = 2 + 2 * b;
      kind = 2;
      basev = b;
    }
    c_key[tid] = bwd ? order_key(2, (uint32_t)J, slot) : order_key(4, (uint32_t)(len - 1 - J), slot);
    c_meta[tid] = pack_meta(bwd ? 0u : 1u, 1, kind, basev, bwd ? J - 1 : J + 1);
    active = true;
  };
  // Start chain c of the group in buffer h: the start-table lookup (or the full
  // interval for short reads) and the first base; the lane stays inactive when
  // the read has no chains or the chain fails within the table's symbols.
  auto start_chain = [&](uint32_t c, uint32_t h) {
    const uint32_t sl = c >> cpr_shift, ci = c & ((1u << cpr_shift) - 1u);
    const uint32_t si = ws.slot[h][sl];
    c_gs[tid] = (h << 5) | sl;
    if (si == 0) {
      atomicSub(&ws.live[h], 1);
      return;
    }
    // 0: '+' backward, 1: '+' forward, 2: '-' backward, 3: '-' forward
    const uint32_t c4 = part == 2 ? ci : (part == 0 ? (ci ? 3u : 0u) : (ci ? 2u : 1u));
    const uint32_t strand = c4 >> 1;
    const bool fwd = (c4 & 1u) != 0;
    const uint32_t d = (fwd ? 1u : 0u) ^ strand;  // forward searches use the strand's forward view
    rs = ((ws.first_read[h] + sl) << 1) | strand;
    len = (int)(si >> 16);
    rbase = h * kHalfBases + (si & 0xFFFFu);
    dir = fwd ? 1 : -1;
    occ = d ? X.dir[1].occ : X.dir[0].occ;
    dollar = d ? X.dir[1].dollar : X.dir[0].dollar;
    cperm = strand ? X.comp_packed : 0xE4u;  // query symbols complemented on the '-' strand
    {  // branching positions of this vector search: J in [2, n/2] backward, [n/2 - 1, n - 1] forward
      const int n = len - 1;
      const int lo = fwd ? n / 2 - 1 : 2, hi = fwd ? n - 1 : n / 2;
      win = (uint32_t)lo | ((uint32_t)(hi >= lo ? hi - lo + 1 : 0) << 16);
    }
    if (L && len >= 2 * (int)L + 2) {
      // The first L steps of a chain from the full interval reach no branching
      // position: one start-table lookup stands for them.
      if (CENSUS) sectors += 1u;
      const uint2 t = __ldg((d ? X.kmer[1] : X.kmer[0]) + ws.kcode[h][c]);
      if (t.x > t.y) {  // failed within the first L steps: no change point, no hit
        atomicSub(&ws.live[h], 1);
        return;
      }
      k = pk = t.x;
      l = pl = t.y;
      pos = fwd ? (int)L : len - 1 - (int)L;
    } else {
      k = pk = 0;
      l = pl = X.top;
      pos = fwd ? 0 : len - 1;
    }
    nb = W(pos);
    active = true;
  };
  // Stage the next claimed reads into buffer h (whole warp, converged).
  auto stage = [&](uint32_t h) {
    for (;;) {
      if (ws.pend_n == 0) {
        uint32_t g0 = 0;
        if (lane == 0) g0 = atomicAdd(group_ctr, G);
        g0 = __shfl_sync(kFull, g0, 0);
        if (g0 >= n_reads) {
          if (lane == 0) ws.done = 1;
          __syncwarp();
          return;
        }
        __syncwarp();
        if (lane == 0) {
          ws.pend_first = g0;
          ws.pend_n = min(G, n_reads - g0);
        }
        __syncwarp();
      }
      // 32 lanes load np + 1 offsets; a buffer holds the start codes of 64 chains
      const uint32_t f = ws.pend_first, np = min(ws.pend_n, part == 2 ? 16u : 31u);
      const uint64_t o = (uint32_t)lane <= np ? p.offs[f + lane] : 0ull;
      const uint64_t o0 = shfl64(o, 0);
      const uint64_t bw = o0 >> 4;
      // reads 0..m-1 of the pending ones fit the buffer: lane i (1..np) checks the end of read i-1
      const bool fits = lane >= 1 && (uint32_t)lane <= np && o >= o0 && ((o + 15) >> 4) - bw <= kHalfWords;
      const unsigned fm = __ballot_sync(kFull, fits) >> 1;
      const uint32_t m = (uint32_t)__ffs(~fm) - 1u;  // leading run of reads that fit
      __syncwarp();
      if (m == 0) {  // a read longer than the buffer: left to the fused kernel
        if (lane == 0) {
          if (part != 1) {
            const unsigned q = atomicAdd(p.long_n, 1u);
            if (q < p.long_cap) p.long_list[q] = f;
            else atomicOr(p.status, kStatusBadInput);  // cannot happen: the list holds total_bases / 4000 + 2
          }
          ws.pend_first = f + 1;
          ws.pend_n -= 1;
        }
        __syncwarp();
        continue;
      }
      const uint64_t o_next = shfl64(o, (lane + 1) & 31);
      bool ok = false;
      uint32_t si = 0;
      if ((uint32_t)lane < m) {
        const uint64_t ln = o_next - o;
        ok = p.ok[f + lane] && o_next >= o && ln >= 3 && ln <= 32767;
        si = ok ? (uint32_t)(o - (bw << 4)) | ((uint32_t)ln << 16) : 0u;
        ws.slot[h][lane] = si;
      }
      const uint64_t o_end = shfl64(o, (int)m);
      const uint32_t nw = (uint32_t)(((o_end + 15) >> 4) - bw);
      for (uint32_t w = lane; w < nw; w += 32) {
        const uint64_t gb = (bw + w) << 4;
        uint32_t word = 0;
        if (gb + 16 <= total_bases) {
          const uint4 v = __ldg(reinterpret_cast<const uint4*>(p.codes + gb));
          word = pack4(v.x) | (pack4(v.y) << 8) | (pack4(v.z) << 16) | (pack4(v.w) << 24);
        } else {
          for (uint32_t i = 0; i < 16 && gb + i < total_bases; ++i) word |= (uint32_t)(p.codes[gb + i] & 3u) << (2 * i);
        }
        ws.words[h * kHalfWords + w] = word;
      }
      __syncwarp();
      // start-table indexes of this lane's read: the first symbol in search order in
      // the top bits -- a backward chain's W[len-L..len-1] in stream order, a forward
      // chain's W[0..L-1] reversed; complemented on the '-' strand
      const int ln = (int)(si >> 16);
      if (ok && L && ln >= 2 * (int)L + 2) {
        const uint32_t rb = h * kHalfBases + (si & 0xFFFFu);
        const uint32_t head = rev2(bases_at(ws, rb, L), L), tail = bases_at(ws, rb + (uint32_t)ln - L, L);
        for (uint32_t ci = 0; ci < (1u << cpr_shift); ++ci) {
          const uint32_t c4 = part == 2 ? ci : (part == 0 ? (ci ? 3u : 0u) : (ci ? 2u : 1u));
          uint32_t code = (c4 & 1u) ? head : tail;
          if (c4 >> 1) {
            if (X.comp_packed == 0x1Bu) {  // comp[b] = 3 - b
              code ^= (1u << (2 * L)) - 1u;
            } else {
              uint32_t cc = 0;
              for (uint32_t i = 0; i < L; ++i)
                cc |= ((X.comp_packed >> (2 * ((code >> (2 * i)) & 3u))) & 3u) << (2 * i);
              code = cc;
            }
          }
          ws.kcode[h][((uint32_t)lane << cpr_shift) + ci] = code;
        }
      }
      __syncwarp();
      if (lane == 0) {
        ws.first_read[h] = f;
        ws.n_chains[h] = m << cpr_shift;
        ws.handed[h] = 0;
        ws.live[h] = (int)(m << cpr_shift);
        ws.pend_first = f + m;
        ws.pend_n -= m;
      }
      __syncwarp();
      return;
    }
  };
  // Hand out work to the idle lanes (whole warp, converged).  Returns with
  // lanes still idle when nothing can be handed out right now.
  auto refill = [&]() {
    for (;;) {
      const unsigned nd = __ballot_sync(kFull, !active);
      if (!nd) return;
      const uint32_t rank = (uint32_t)__popc(nd & ((1u << lane) - 1u));
      const uint32_t n_nd = (uint32_t)__popc(nd);
      const unsigned top = min(ws.top, kWarpStack);  // pushes past the end went to the device queue
      if (top && n_nd >= 8) {  // change points first, eight lanes each: they free their group buffers
        const uint32_t take = min(n_nd >> 3, top);
        __syncwarp();
        if (!active && (rank >> 3) < take) {
          const SpillEntry e = ws.stk[top - 1 - (rank >> 3)];
          if ((rank & 7u) == 0) atomicAdd(&ws.live[(e.jtype >> 23) & 1u], 7);  // one stacked item becomes eight
          start_walk(e, rank & 7u);
        }
        __syncwarp();
        if (lane == 0) ws.top = top - take;
        __syncwarp();
        continue;
      }
      int h = -1;
      if (ws.handed[0] < ws.n_chains[0]) h = 0;
      else if (ws.handed[1] < ws.n_chains[1]) h = 1;
      if (h >= 0) {
        const uint32_t c0 = ws.handed[h];
        const uint32_t take = min(n_nd, ws.n_chains[h] - c0);
        __syncwarp();
        if (!active && rank < take) start_chain(c0 + rank, (uint32_t)h);
        __syncwarp();
        if (lane == 0) ws.handed[h] = c0 + take;
        __syncwarp();
        continue;
      }
      if (top) return;  // stacked change points wait for eight idle lanes
      if (ws.done && ws.pend_n == 0) return;
      // stage the next group into a buffer with no work left alive
      const int fh = ws.live[0] == 0 ? 0 : (ws.live[1] == 0 ? 1 : -1);
      __syncwarp();
      if (fh < 0) {
        if (nd == kFull) {
          // No lane is busy, nothing is stacked and every chain was handed out, so
          // nothing can be alive: the counts are inconsistent.  Fail the batch
          // (status) instead of waiting forever, and carry on.
          if (lane == 0) {
            atomicOr(p.status, kStatusWaveAcct);
            ws.live[0] = 0;
            ws.live[1] = 0;
          }
          __syncwarp();
          continue;
        }
        return;  // both buffers still have work running: wait for it
      }
      stage((uint32_t)fh);
    }
  };

  const uint32_t bi = p.batch_idle < 1 ? 1u : p.batch_idle;
  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !active);  // every lane, every iteration
    if (idle == kFull || (uint32_t)__popc(idle) >= bi) {
      refill();
      if (__ballot_sync(kFull, !active) == kFull && ws.done && ws.pend_n == 0 && ws.top == 0 &&
          ws.handed[0] == ws.n_chains[0] && ws.handed[1] == ws.n_chains[1]) {
        if (lane == 0 && (ws.live[0] != 0 || ws.live[1] != 0)) atomicOr(p.status, kStatusWaveAcct);
        break;  // nothing left for this warp
      }
    }
    if (!active) continue;  // waiting for more lanes to move on with

    // one step: (k,l) becomes the vector entry at pos, (pk,pl) is the entry at J = pos - dir
    if (CENSUS) sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    wave_step(X, occ, dollar, cperm, nb, k, l);
    // A chain's helper branches at J in [2, n/2] (backward, block at 1) and
    // [n/2 - 1, n - 2] (forward, block at n - 1); a walk's window is empty.
    const int J = pos - dir;
    const bool differ = (l - k) != (pl - pk);  // sizes are >= -1 here, so 32-bit differences suffice
    if (differ && (uint32_t)(J - (int)(win & 0xFFFFu)) < ((win >> 16) & 0x7FFFu))
      push_cp(pk, pl, (uint32_t)J | ((dir > 0 ? (J == len - 2 ? kBlkN : kCpFwd) : kCpBwd) << 16));
    if (k <= l && (uint32_t)(pos + dir) < (uint32_t)len) {  // a next base to match
      pk = k;
      pl = l;
      pos += dir;
      nb = W(pos);
      continue;
    }
    if (win >> 31) {  // a branch walk that reached the read end: its hit
      if (k <= l) {
        uint32_t r = c_res[tid];
        const unsigned slot = res_slot(p, r);
        c_res[tid] = r;
        write_hit(p, slot, rs, c_key[tid], k, l, c_meta[tid]);
      }
    } else if (dir < 0 && pos == 0) {  // backward vector complete: exact hit, then the j = 1 block on vec[1]
      if (k <= l) {
        uint32_t r = c_res[tid];
        const unsigned slot = res_slot(p, r);
        c_res[tid] = r;
        write_hit(p, slot, rs, order_key(0, 0, 0), k, l, pack_meta(0, 0, 0, 0, 0));
      }
      if (differ) push_cp(pk, pl, 1u | (kBlk1 << 16));
    }
    item_done();
  }
  {  // slots of this lane's last chunks that were reserved but not used
    const uint32_t r = c_res[tid];
    for (unsigned i = 0, left = r >> 28, slot = r & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.res_cap) p.res[slot + i].rs = 0xFFFFFFFFu;
    const uint32_t cs = c_spl[tid];
    for (unsigned i = 0, left = cs >> 28, q = cs & 0x0FFFFFFFu; i < left; ++i)
      if (q + i < p.spill_cap) p.spill[q + i].rs = 0xFFFFFFFFu;
  }
  if (CENSUS && p.census) atomicAdd(p.census, (unsigned long long)sectors);
}

// Branches of the 1-error helper (search/search.c:1491-1709) from queued change
// points, one work item per lane.  A change point at J with vector interval E
// (search.c:1596-1630 backward, 1674-1707 forward) has exactly eight
// continuations, each an exact search to the read end whose result, when its
// interval survives, is one hit:
//   item 0    deletion: from E over W[J-2..0] (forward: W[J+2..n]);
//   items 1-4 insertion of base b = 0..3: from E one step with b, then over W[J-1..0];
//   items 5-7 mismatch with the three bases b != W[J-1]: one step with b, then over W[J-2..0].
// An insertion and a mismatch of the same b repeat that first step (the
// helper takes it once); in exchange every item is the same loop.  A warp takes
// one change point per eight idle lanes.  The j = 1 / j = n-1 blocks, whose
// results depend on one another (search.c:1556 keeps an insertion's base as the
// position of later mismatches), are forwarded to `blocks` for the fused drain.
//
// A warp claims 32 queue slots with one atomic, keeps the change points among
// them (the queue has holes: slots reserved in chunks and not used), and
// fetches each one's read offset and the two read bases its items start from,
// so that handing out items reads shared memory only.
struct BranchShared {
  SpillEntry cp[32];
  uint64_t b0[32];      // offset of the read's first base
  uint32_t lw[32];      // read length | base at J -/+ 2 << 16 | base at J -/+ 1 << 24
  uint32_t n, next;     // change points held, next one to hand out
};

template <int MINB, bool CENSUS>
__global__ void __launch_bounds__(kWBlock, MINB) wave_branch_kernel(DevIndex X, BatchedParams p, SpillEntry* blocks,
                                                                     unsigned int* block_n, uint32_t block_cap) {
  __shared__ BranchShared bsh[kWWarps];
  __shared__ uint32_t c_res[kWBlock];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  BranchShared& bs = bsh[tid >> 5];
  const unsigned n_cp = min(*(volatile unsigned int*)p.spill_tail, p.spill_cap);
  c_res[tid] = 0;
  if (lane == 0) {
    bs.n = 0;
    bs.next = 0;
  }
  __syncwarp();
  bool active = false;
  uint32_t rs = 0, k = 0, l = 0, nb = 0, key = 0, meta = 0;
  int nxt = 0, dir = 0, end = 0;
  const uint8_t* W = nullptr;
  const OccBlock* occ = nullptr;
  uint32_t dollar = 0, cperm = 0;
  uint32_t sectors = 0;
  // refill when at least this many lanes are idle, and at least eight (one change point)
  const uint32_t bi = p.batch_idle < 8 ? 8u : p.batch_idle;
  bool exhausted = false;
  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !active);  // every lane, every iteration
    if (exhausted && bs.next == bs.n && idle == kFull) break;
    const uint32_t n_idle = (uint32_t)__popc(idle);
    if (idle == kFull || n_idle >= bi) {
      if (bs.next == bs.n && !exhausted) {  // claim the next 32 queue slots
        uint32_t c0 = 0;
        if (lane == 0) c0 = atomicAdd(p.spill_head, 32u);
        c0 = __shfl_sync(kFull, c0, 0);
        if (c0 + 32 >= n_cp) exhausted = true;
        SpillEntry e{0, 0, 0xFFFFFFFFu, 0};
        if (c0 + lane < n_cp) e = p.spill[c0 + lane];
        const uint32_t type = (e.jtype >> 16) & 3u;
        bool keep = false;
        uint64_t rb0 = 0;
        uint32_t lw = 0;
        if (e.rs != 0xFFFFFFFFu) {  // (a reserved slot nothing was written to)
          if (type >= kBlk1) {
            const unsigned q = atomicAdd(block_n, 1u);
            if (q < block_cap) blocks[q] = SpillEntry{e.k, e.l, e.rs, e.jtype & 0x3FFFFu};
            else atomicOr(p.status, kStatusSpillFull);
          } else {
            const uint32_t read = e.rs >> 1;
            rb0 = p.offs[read];
            const int len = (int)(p.offs[read + 1] - rb0);
            const int J = (int)(e.jtype & 0xFFFFu);
            const bool bwd = type == kCpBwd;
            // the queue holds only change points inside the helper's windows
            // (backward 2 <= J, forward J <= n-2); anything else is not read from
            keep = len >= 3 && (bwd ? (J >= 2 && J <= len - 1) : (J + 2 <= len - 1));
            if (keep) {
              const int dd = bwd ? -1 : 1;
              lw = (uint32_t)len | ((uint32_t)p.codes[rb0 + J + 2 * dd] << 16) |
                   ((uint32_t)p.codes[rb0 + J + dd] << 24);
            } else {
              atomicOr(p.status, kStatusBadInput);
            }
          }
        }
        const unsigned km = __ballot_sync(kFull, keep);
        if (keep) {
          const uint32_t at = (uint32_t)__popc(km & ((1u << lane) - 1u));
          bs.cp[at] = e;
          bs.b0[at] = rb0;
          bs.lw[at] = lw;
        }
        __syncwarp();
        if (lane == 0) {
          bs.n = (uint32_t)__popc(km);
          bs.next = 0;
        }
        __syncwarp();
      }
      const uint32_t first = bs.next;
      const uint32_t ncp = min(n_idle >> 3, bs.n - first);
      const uint32_t rank = (uint32_t)__popc(idle & ((1u << lane) - 1u));
      const uint32_t item = rank & 7u;
      if (!active && (rank >> 3) < ncp) {
        const uint32_t ci = first + (rank >> 3);
        const SpillEntry e = bs.cp[ci];
        const uint32_t lw = bs.lw[ci];
        const uint32_t strand = e.rs & 1u;
        const int len = (int)(lw & 0xFFFFu);
        W = p.codes + bs.b0[ci];
        end = len - 1;
        const int J = (int)(e.jtype & 0xFFFFu);
        const bool bwd = ((e.jtype >> 16) & 3u) == kCpBwd;
        dir = bwd ? -1 : 1;
        const uint32_t d = (bwd ? 0u : 1u) ^ strand;
        occ = d ? X.dir[1].occ : X.dir[0].occ;
        dollar = d ? X.dir[1].dollar : X.dir[0].dollar;
        cperm = strand ? X.comp_packed : 0xE4u;
        rs = e.rs;
        k = e.k;
        l = e.l;
        uint32_t slot, kind, basev;
        if (item == 0) {  // deletion
          nb = (lw >> 16) & 0xFFu;
          nxt = J + 3 * dir;
          slot = 0;
          kind = 1;
          basev = 0xFFu;
        } else if (item <= 4) {  // insertion of b
          const uint32_t b = item - 1;
          nb = b;
          nxt = J + dir;
          slot = 1 + 2 * b;
          kind = 3;
          basev = b;
        } else {  // mismatch with b != W[J -/+ 1]
          const uint32_t w = lw >> 24;
          const uint32_t b = (item - 5) + ((item - 5) >= w ? 1u : 0u);
          nb = b;
          nxt = J + 2 * dir;
          slot = 2 + 2 * b;
          kind = 2;
          basev = b;
        }
        key = bwd ? order_key(2, (uint32_t)J, slot) : order_key(4, (uint32_t)(len - 1 - J), slot);
        meta = pack_meta(bwd ? 0u : 1u, 1, kind, basev, bwd ? J - 1 : J + 1);
        active = true;
      }
      __syncwarp();
      if (lane == 0) bs.next = first + ncp;
      __syncwarp();
    }
    if (!active) continue;
    // the next base is fetched alongside the gather
    const uint32_t nb_next = (uint32_t)nxt <= (uint32_t)end ? W[nxt] : 0u;
    if (CENSUS) sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    wave_step(X, occ, dollar, cperm, nb, k, l);
    if (k <= l && (uint32_t)nxt <= (uint32_t)end) {  // a next base to match
      nb = nb_next;
      nxt += dir;
      continue;
    }
    if (k <= l) {  // matched to the read end: the hit
      uint32_t r = c_res[tid];
      const unsigned slot = res_slot(p, r);
      c_res[tid] = r;
      write_hit(p, slot, rs, key, k, l, meta);
    }
    active = false;
  }
  {
    const uint32_t r = c_res[tid];
    for (unsigned i = 0, left = r >> 28, slot = r & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.res_cap) p.res[slot + i].rs = 0xFFFFFFFFu;
  }
  if (CENSUS && p.census) atomicAdd(p.census, (unsigned long long)sectors);
}

template <int MINB>
int wave_occupancy(int blocks_per_sm) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wave_search_kernel<MINB, false>, kWBlock, 0);
  if (blocks_per_sm > 0 && blocks_per_sm < per_sm) per_sm = blocks_per_sm;
  return per_sm < 1 ? 1 : per_sm;
}

template <int MINB>
void launch_wave_m(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, cudaStream_t s) {
  static bool carveout = false;
  if (!carveout) {  // the group buffers need shared memory for the register-bound number of blocks
    cudaFuncSetAttribute(wave_search_kernel<MINB, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(wave_search_kernel<MINB, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    carveout = true;
  }
  const int per_sm = wave_occupancy<MINB>(t.blocks_per_sm);
  count_launches(1);
  if (p.census)
    wave_search_kernel<MINB, true><<<num_sms * per_sm, kWBlock, 0, s>>>(X, p);
  else
    wave_search_kernel<MINB, false><<<num_sms * per_sm, kWBlock, 0, s>>>(X, p);
}

int branch_occupancy() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wave_branch_kernel<10, false>, kWBlock, 0);
  return per_sm < 1 ? 1 : per_sm;
}

}  // namespace

void launch_wave_search(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms,
                        cudaStream_t s) {
  if (t.min_blocks >= 12)
    launch_wave_m<12>(X, p, t, num_sms, s);
  else if (t.min_blocks >= 8)
    launch_wave_m<8>(X, p, t, num_sms, s);
  else
    launch_wave_m<1>(X, p, t, num_sms, s);
}

void launch_wave_branches(const DevIndex& X, const BatchedParams& p, SpillEntry* blocks, unsigned int* block_n,
                          uint32_t block_cap, int num_sms, cudaStream_t s) {
  const int per_sm = branch_occupancy();
  count_launches(1);
  if (p.census)
    wave_branch_kernel<10, true><<<num_sms * per_sm, kWBlock, 0, s>>>(X, p, blocks, block_n, block_cap);
  else
    wave_branch_kernel<10, false><<<num_sms * per_sm, kWBlock, 0, s>>>(X, p, blocks, block_n, block_cap);
}

int wave_max_blocks_per_sm(const BatchedTuning& t) {
  if (t.min_blocks >= 12) return wave_occupancy<12>(t.blocks_per_sm);
  if (t.min_blocks >= 8) return wave_occupancy<8>(t.blocks_per_sm);
  return wave_occupancy<1>(t.blocks_per_sm);
}

}  // namespace hpgbwt
