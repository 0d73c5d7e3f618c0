// batched.cu -- persistent work-queue search, ordered finalize and persistent
// locate of the batched pipeline form.
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#include <cuda_runtime.h>

#include "batched.cuh"
#include "batched_dev.cuh"
#include "kernels.cuh"
#include "search_core.cuh"

namespace cg = cooperative_groups;

namespace hpgbwt {

namespace {

constexpr int kBlock = 128;

using namespace bdev;

// Next read of a chain set (part 0: the chains on the backward index, 1: those
// on the forward index, 2: all four), aggregated per warp and per set.
__device__ __forceinline__ unsigned claim_part(const BatchedParams& p, uint32_t part) {
  cg::coalesced_group g = cg::coalesced_threads();
  cg::coalesced_group sub = cg::labeled_partition(g, part);
  unsigned base = 0;
  if (sub.thread_rank() == 0) base = atomicAdd(part == 1 ? p.chain_ctr2 : p.chain_ctr, (unsigned)sub.size());
  return sub.shfl(base, 0) + sub.thread_rank();
}

__device__ __forceinline__ uint32_t sm_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

template <int D, int MINB, bool CENSUS>
__global__ void __launch_bounds__(kBlock, MINB) batched_search_kernel(DevIndex X, BatchedParams p, int drain,
                                                                      int chunk) {
  __shared__ uint32_t stk_k[D][kBlock], stk_l[D][kBlock], stk_j[D][kBlock];
  __shared__ uint32_t c_ek[kBlock], c_el[kBlock], c_meta[kBlock], c_misc[kBlock], c_res[kBlock], c_part[kBlock];
  __shared__ uint32_t c_read[kBlock];  // read whose chains this lane runs
  __shared__ uint32_t s_nreads, s_spill_end;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_nreads = p.read_list ? min(*p.read_list_n, p.long_cap) : (p.n_reads_dev ? *p.n_reads_dev : p.n_reads);
    s_spill_end = drain ? min(*(volatile unsigned int*)p.spill_tail, p.spill_cap) : 0u;
  }
  c_meta[tid] = 0;
  c_misc[tid] = 4u << 4;  // no chain of a read left
  c_res[tid] = 0;
  __syncthreads();

  // hot state
  uint32_t rs = 0;                  // 2 * read + strand
  const uint8_t* W = nullptr;
  int len = 0;
  uint32_t k = 0, l = 0;            // interval of the pending / last step
  uint32_t pk = 0, pl = 0;          // chain: previous interval; entry: aux interval
  int pos = 0, dir = 0;             // read position of the pending step; -1 backward, +1 forward
  uint32_t nb = 0;                  // base of the pending step
  uint32_t mode = kNone;
  uint32_t win = 0;                 // chain: first J where the helper branches | how many J (<< 16)
  uint32_t sectors = 0;
  // read-level work: the current read's next chain, and the next read claimed
  // and its offsets fetched ahead of time (their loads complete while the
  // current read is searched)
  // With the direction split, SMs of the first half take the two chains of a
  // read that run on the backward index ('+' backward, '-' forward) and the
  // others the two on the forward index ('+' forward, '-' backward): every
  // chain and its branches stay on one index direction, so each half's L2
  // holds one direction's blocks.  A half that runs out takes the other's reads.
  // (claim state in shared memory, touched once per read: bits 0-1 the chain
  // set being claimed, bit 2 set once it moved to the other half's reads,
  // bits 3-4 the set of the current read, bits 5-6 that of the prefetched one)
  {
    const uint32_t part0 = p.dir_split == 1 ? (sm_id() >= p.num_sms / 2 ? 1u : 0u)
                                             : (p.dir_split == 2 ? 0u : (p.dir_split == 3 ? 1u : 2u));
    c_part[tid] = part0 | (part0 << 3) | (part0 << 5);
  }
  // The claim state (read, chain of the read, chain set) lives in shared
  // memory: a lane touches it once per chain, and the registers it frees let
  // more blocks stay resident.  A read's offsets are loaded when it is claimed.
  auto next_claim = [&]() -> uint32_t {
    uint32_t st = c_part[tid];
    for (;;) {
      const uint32_t part = st & 3u;
      const uint32_t r = claim_part(p, part);
      if (r < s_nreads || part == 2u || (st & 4u) || p.dir_split != 1) {
        c_part[tid] = (st & ~(3u << 3)) | (part << 3);
        return r;
      }
      st = (st & ~3u) | (part ^ 1u) | 4u;
    }
  };
  (void)chunk;

  auto push = [&](uint32_t a, uint32_t b, uint32_t jt) {
    const uint32_t misc = c_misc[tid];
    const uint32_t sp = misc & 15u;
    if (sp < (uint32_t)D) {
      stk_k[sp][tid] = a;
      stk_l[sp][tid] = b;
      stk_j[sp][tid] = jt;
      c_misc[tid] = misc + 1;
    } else {
      const unsigned s = claim(p.spill_tail, 1);
      if (s < p.spill_cap) p.spill[s] = SpillEntry{a, b, rs, jt};
      else atomicOr(p.status, kStatusSpillFull);
    }
  };
  // Result of a continuation search that matched to the read end.
  auto emit = [&](uint32_t key, uint32_t a, uint32_t b, uint32_t meta) {
    uint32_t r = c_res[tid];
    const unsigned slot = res_slot(p, r);
    c_res[tid] = r;
    write_hit(p, slot, rs, key, a, b, meta);
  };
  auto emit_cont = [&](uint32_t m) {
    const uint32_t ej = meta_j(m), sub = meta_sub(m);
    const bool bwd = meta_type(m) == kCpBwd;
    const uint32_t b = sub == 0 ? 0u : (sub - 1) / 3;
    const bool ins = sub != 0 && (sub - 1) % 3 == 1;
    const uint32_t kind = sub == 0 ? 1u : (ins ? 3u : 2u);
    const uint32_t slot = sub == 0 ? 0u : (ins ? 1u + 2 * b : 2u + 2 * b);
    const uint32_t basev = sub == 0 ? 0xFFu : b;
    if (bwd)
      emit(order_key(2, ej, slot), k, l, pack_meta(0, 1, kind, basev, (int32_t)ej - 1));
    else
      emit(order_key(4, (uint32_t)(len - 1 - (int)ej), slot), k, l,
               pack_meta(1, 1, kind, basev, (int32_t)ej + 1));
  };

  for (;;) {
    // ---- transitions: next sub-operation, next change point, next chain ----
    // A lane out of work waits (riding along masked) until p.batch_idle lanes
    // of its converged group are out of work too, or all of them are, so the
    // transition code runs for many lanes at once instead of one at a time.
    bool go = mode == kNone;
    if (p.batch_idle > 1) {
      const unsigned grp = __activemask();
      const unsigned idle = __ballot_sync(grp, mode == kNone);
      go = go && ((uint32_t)__popc(idle) >= p.batch_idle || idle == grp);
    }
    if (go) {
    while (mode == kNone) {
      uint32_t m = c_meta[tid];
      if (meta_in(m)) {
        const uint32_t sub = meta_sub(m), etype = meta_type(m), ej = meta_j(m);
        if (sub >= kSubEnd) {
          c_meta[tid] = 0;
          continue;
        }
        const bool bwd = (etype == kCpBwd || etype == kBlk1);
        const bool blk = etype >= kBlk1;
        const int end = len - 1;
        dir = bwd ? -1 : 1;
        if (sub == 0) {
          if (blk) {  // the block's direct deletion result
            if (etype == kBlk1)
              emit(order_key(1, 0, 0), c_ek[tid], c_el[tid], pack_meta(0, 1, 1, 0xFF, 0));
            else
              emit(order_key(3, 0, 0), c_ek[tid], c_el[tid], pack_meta(1, 1, 1, 0xFF, end));
            c_meta[tid] = m + (1u << 18);
            continue;
          }
          k = c_ek[tid];
          l = c_el[tid];
          pos = bwd ? (int)ej - 2 : (int)ej + 2;
        } else {
          const uint32_t b = (sub - 1) / 3, r = (sub - 1) % 3;
          if (r == 0) {  // aux step with base b
            k = c_ek[tid];
            l = c_el[tid];
            nb = b;
            mode = kSingle;
            break;
          }
          if (blk) {
            if (r == 1) {  // block insertion: one step with the read's end base
              k = pk;
              l = pl;
              nb = etype == kBlk1 ? W[0] : W[end];
              mode = kSingle;
              break;
            }
            c_meta[tid] = m + (1u << 18);  // blocks emit their mismatch right after the aux step
            continue;
          }
          if (r == 2 && b == W[bwd ? ej - 1 : ej + 1]) {  // no mismatch with the read's own base
            c_meta[tid] = m + (1u << 18);
            continue;
          }
          k = pk;
          l = pl;
          pos = bwd ? (int)ej - (int)r : (int)ej + (int)r;
        }
        if (bwd ? pos < 0 : pos > end) {  // nothing left to match: the interval is the hit
          if (k <= l) emit_cont(m);
          c_meta[tid] = m + (1u << 18);
          continue;
        }
        nb = W[pos];
        mode = kCont;
        break;
      }
      const uint32_t misc = c_misc[tid];
      if (misc & 15u) {  // next change point of this lane's read
        const uint32_t sp = (misc & 15u) - 1;
        c_misc[tid] = misc - 1;
        c_ek[tid] = stk_k[sp][tid];
        c_el[tid] = stk_l[sp][tid];
        const uint32_t jt = stk_j[sp][tid];
        c_meta[tid] = make_meta(jt & 0xFFFFu, jt >> 16, 0, 0, true);
        continue;
      }
      if (drain) {
        const unsigned s = claim(p.spill_head, 1);
        if (s >= s_spill_end) break;
        const SpillEntry e = p.spill[s];
        if (e.rs == 0xFFFFFFFFu) continue;  // reserved but unused slot
        rs = e.rs;
        const uint32_t read = rs >> 1;
        const uint64_t b0 = p.offs[read];
        W = p.codes + b0;
        len = (int)(p.offs[read + 1] - b0);
        c_ek[tid] = e.k;
        c_el[tid] = e.l;
        c_meta[tid] = make_meta(e.jtype & 0xFFFFu, e.jtype >> 16, 0, 0, true);
        continue;
      }
      uint32_t chain = (misc >> 4) & 7u;
      if (chain >= ((((c_part[tid] >> 3) & 3u) == 2u) ? 4u : 2u)) {  // next read
        const uint32_t rc = next_claim();
        if (rc >= s_nreads) break;
        const uint32_t r = p.read_list ? p.read_list[rc] : rc;
        c_read[tid] = r;
        const uint64_t b0 = p.offs[r];
        const int L = (int)(p.offs[r + 1] - b0);
        if (!p.ok[r] || L < 3 || L > 32767) continue;  // no chains for this read (chain stays at its end)
        W = p.codes + b0;
        len = L;
        chain = 0;
      }
      c_misc[tid] = (misc & 15u) | ((chain + 1) << 4);
      const uint32_t ci = chain;
      const uint32_t cur_read = c_read[tid];
      const uint32_t cur_part = (c_part[tid] >> 3) & 3u;
      // 0: '+' backward, 1: '+' forward, 2: '-' backward, 3: '-' forward
      const uint32_t c = cur_part == 2u ? ci : (cur_part == 0u ? (ci ? 3u : 0u) : (ci ? 2u : 1u));
      rs = (cur_read << 1) | (c >> 1);
      k = 0;
      l = X.top;
      pk = 0;
      pl = X.top;
      dir = (c & 1u) ? 1 : -1;
      pos = (c & 1u) ? 0 : len - 1;
      {  // branching positions of this vector search: J in [2, n/2] backward, [n/2 - 1, n - 1] forward
        const int n = len - 1;
        const int lo = dir > 0 ? n / 2 - 1 : 2, hi = dir > 0 ? n - 1 : n / 2;
        win = (uint32_t)lo | ((uint32_t)(hi >= lo ? hi - lo + 1 : 0) << 16);
      }
      const uint32_t L = X.kmer_len;
      if (L && len >= 2 * (int)L + 2) {
        // The first L steps of a chain from the full interval never reach a
        // branching position (J stays above n/2 backward, below n/2 - 1
        // forward): one table lookup stands for them.
        const uint32_t strand = rs & 1u;
        uint32_t code = 0;
        for (uint32_t i = 0; i < L; ++i) {
          const uint32_t b = W[dir > 0 ? (int)i : len - 1 - (int)i];
          code = (code << 2) | (strand ? sel4(X.comp, b) : b);
        }
        nb = code;
        mode = kKmer;
      } else {
        nb = W[pos];
        mode = kChain;
      }
    }
    if (mode == kNone) break;  // no work left for this lane
    }
    if (mode == kNone) continue;  // waiting for more lanes to move on with

    // ---- the one gather of this iteration --------------------------------
    {
      const uint32_t strand = rs & 1u;
      const uint32_t vsel = dir > 0 ? 1u : 0u;  // forward searches use the strand's forward view
      if (mode == kKmer) {
        if (CENSUS) sectors += 1u;
        const uint2 t = __ldg(((vsel ^ strand) ? X.kmer[1] : X.kmer[0]) + nb);
        k = t.x;
        l = t.y;
      } else {
        if (CENSUS) sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
        bw_step(X, View{vsel ^ strand, strand}, nb, k, l);
      }
    }
    if (mode == kKmer) {
      if (k > l) {  // failed within the first L steps: no change point, no hit
        mode = kNone;
        continue;
      }
      pk = k;
      pl = l;
      pos = dir > 0 ? (int)X.kmer_len : len - 1 - (int)X.kmer_len;
      nb = W[pos];
      mode = kChain;
      continue;
    }
    if (mode == kChain) {
      // (k,l) = vector entry at pos, (pk,pl) = entry at J = pos - dir.  The helper
      // branches at J in [2, n/2] (backward, block at 1) and [n/2 - 1, n - 2]
      // (forward, block at n - 1).
      const int J = pos - dir;
      const bool differ = (l - k) != (pl - pk);  // sizes are >= -1 here, so 32-bit differences suffice
      if (differ && (uint32_t)(J - (int)(win & 0xFFFFu)) < (win >> 16))
        push(pk, pl, (uint32_t)J | ((dir > 0 ? (J == len - 2 ? kBlkN : kCpFwd) : kCpBwd) << 16));
      if (k <= l && (uint32_t)(pos + dir) < (uint32_t)len) {  // a next base to match
        pk = k;
        pl = l;
        pos += dir;
        nb = W[pos];
        continue;
      }
      if (dir < 0 && pos == 0) {  // backward vector complete: exact hit, then the j = 1 block on vec[1]
        if (k <= l) emit(order_key(0, 0, 0), k, l, pack_meta(0, 0, 0, 0, 0));
        if (differ) push(pk, pl, 1u | (kBlk1 << 16));
      }
      mode = kNone;
    } else if (mode == kCont) {
      if (k <= l && (uint32_t)(pos + dir) < (uint32_t)len) {
        pos += dir;
        nb = W[pos];
        continue;
      }
      const uint32_t m = c_meta[tid];
      if (k <= l) emit_cont(m);
      c_meta[tid] = m + (1u << 18);
      mode = kNone;
    } else {  // kSingle: an aux step or a block insertion step
      const uint32_t m = c_meta[tid];
      const uint32_t sub = meta_sub(m), etype = meta_type(m);
      const uint32_t b = (sub - 1) / 3;
      if ((sub - 1) % 3 == 0) {
        if (k > l) {
          c_meta[tid] = m + (3u << 18);
        } else {
          pk = k;
          pl = l;
          if (etype >= kBlk1) {
            const int end = len - 1;
            const uint32_t w = etype == kBlk1 ? W[0] : W[end];
            if (b != w) {
              if (etype == kBlk1)
                emit(order_key(1, 0, 1 + 2 * b), k, l, pack_meta(0, 1, 2, b, (int32_t)meta_bpos(m)));
              else
                emit(order_key(3, 0, 1 + 2 * b), k, l, pack_meta(1, 1, 2, b, end));
            }
          }
          c_meta[tid] = m + (1u << 18);
        }
      } else {
        uint32_t nm = m + (2u << 18);
        if (k <= l) {
          if (etype == kBlk1) {
            emit(order_key(1, 0, 2 + 2 * b), k, l, pack_meta(0, 1, 3, 3, (int32_t)b));
            nm = (nm & ~(3u << 22)) | (b << 22);
          } else {
            emit(order_key(3, 0, 2 + 2 * b), k, l, pack_meta(1, 1, 3, b, len - 1));
          }
        }
        c_meta[tid] = nm;
      }
      mode = kNone;
    }
  }
  {  // slots of this lane's last chunk that were reserved but not used
    const uint32_t r = c_res[tid];
    const unsigned left = r >> 28, slot = r & 0x0FFFFFFFu;
    for (unsigned i = 0; i < left; ++i)
      if (slot + i < p.res_cap) p.res[slot + i].rs = 0xFFFFFFFFu;
  }
  if (CENSUS && p.census) atomicAdd(p.census, (unsigned long long)sectors);
}

// Chain-only variant (the "split" form): lanes run only the vector searches,
// with the smallest possible loop, and append every change point to the
// device queue; a drain launch of batched_search_kernel then expands them.
// `phase` 0 runs only the chains on the backward index ('+' backward and '-'
// forward), 1 only those on the forward index ('+' forward, '-' backward), so
// each launch keeps one direction's occurrence blocks hot in L2; 2 runs all.
template <int MINB>
__global__ void __launch_bounds__(kBlock, MINB) chain_kernel(DevIndex X, BatchedParams p, int chunk, int phase) {
  const uint32_t n_reads_ = p.n_reads_dev ? *p.n_reads_dev : p.n_reads;
  const uint32_t n_chains = (phase == 2 ? 4u : 2u) * n_reads_;
  uint32_t rs = 0;
  const uint8_t* W = nullptr;
  int len = 0;
  uint32_t k = 0, l = 0, pk = 0, pl = 0;
  int pos = 0, dir = 0;
  uint32_t nb = 0;
  bool active = false;
  uint32_t next = 0, left = 0, sectors = 0;
  for (;;) {
    // lanes out of chains wait (masked) until p.batch_idle lanes of the
    // converged group are, or all of them are, and claim the next ones together
    bool go = !active;
    if (p.batch_idle > 1) {
      const unsigned grp = __activemask();
      const unsigned idle = __ballot_sync(grp, !active);
      go = go && ((uint32_t)__popc(idle) >= p.batch_idle || idle == grp);
    }
    if (!go && !active) continue;
    while (!active) {
      if (left == 0) {
        next = claim(p.chain_ctr, (unsigned)chunk);
        left = (unsigned)chunk;
      }
      if (next >= n_chains) break;
      const uint32_t c = next++;
      --left;
      const uint32_t read = phase == 2 ? c >> 2 : c >> 1;
      const uint64_t b0 = p.offs[read];
      const int L = (int)(p.offs[read + 1] - b0);
      if (!p.ok[read] || L < 3 || L > 32767) continue;
      const uint32_t strand = phase == 2 ? (c >> 1) & 1u : c & 1u;
      const bool fwd = phase == 2 ? (c & 1u) != 0 : ((strand ^ (uint32_t)phase) != 0);
      rs = (read << 1) | strand;
      W = p.codes + b0;
      len = L;
      k = 0;
      l = X.top;
      pk = 0;
      pl = X.top;
      dir = fwd ? 1 : -1;
      pos = fwd ? 0 : L - 1;
      const uint32_t KL = X.kmer_len;
      if (KL && L >= 2 * (int)KL + 2) {
        // start table: one lookup for the first KL steps, which reach no
        // branching position (as in the fused kernel)
        uint32_t code = 0;
        for (uint32_t i = 0; i < KL; ++i) {
          const uint32_t b = W[fwd ? (int)i : L - 1 - (int)i];
          code = (code << 2) | (strand ? sel4(X.comp, b) : b);
        }
        const uint2 t = __ldg(((((uint32_t)fwd) ^ strand) ? X.kmer[1] : X.kmer[0]) + code);
        if (p.census) sectors += 1u;
        if (t.x > t.y) continue;  // failed within the first KL steps: no change point, no hit
        k = pk = t.x;
        l = pl = t.y;
        pos = fwd ? (int)KL : L - 1 - (int)KL;
      }
      nb = W[pos];
      active = true;
    }
    if (!active) break;
    const int stop = dir > 0 ? len - 1 : 0;
    // next base, fetched alongside the gather instead of after it
    const uint32_t nb_next = pos != stop ? W[pos + dir] : 0u;
    {
      const uint32_t strand = rs & 1u;
      if (p.census) sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
      bw_step(X, View{(dir > 0 ? 1u : 0u) ^ strand, strand}, nb, k, l);
    }
    const int J = pos - dir, n = len - 1;
    const int jlo = dir > 0 ? n / 2 - 1 : 2, jhi = dir > 0 ? n - 1 : n / 2;
    const bool differ = (l - k) != (pl - pk);
    if (differ && J >= jlo && J <= jhi) {
      const uint32_t jt = (uint32_t)J | ((dir > 0 ? (J == n - 1 ? kBlkN : kCpFwd) : kCpBwd) << 16);
      const unsigned s = claim(p.spill_tail, 1);
      if (s < p.spill_cap) p.spill[s] = SpillEntry{pk, pl, rs, jt};
      else atomicOr(p.status, kStatusSpillFull);
    }
    if (k <= l && pos != stop) {
      pk = k;
      pl = l;
      pos += dir;
      nb = nb_next;
      continue;
    }
    if (dir < 0 && pos == 0) {
      if (k <= l) emit_hit(p, rs, order_key(0, 0, 0), k, l, pack_meta(0, 0, 0, 0, 0));
      if (differ) {
        const unsigned s = claim(p.spill_tail, 1);
        if (s < p.spill_cap) p.spill[s] = SpillEntry{pk, pl, rs, 1u | (kBlk1 << 16)};
        else atomicOr(p.status, kStatusSpillFull);
      }
    }
    active = false;
  }
  if (p.census) atomicAdd(p.census, (unsigned long long)sectors);
}

// Lockstep variant: one lane per read runs the read's four vector searches
// together -- '+' backward over the backward index, '-' backward over the
// forward index with complemented bases, both moving down the read, and the
// two forward searches moving up -- so every lane spends about one read length
// per read whatever the strand, and up to four independent gathers are in
// flight per lane.  Change points go to the device queue for the drain launch.
__device__ __forceinline__ void spill_push(const BatchedParams& p, uint32_t& chunk_state, uint32_t a, uint32_t b,
                                           uint32_t rs, uint32_t jt) {
  unsigned left = chunk_state >> 28;
  if (left == 0) {
    chunk_state = claim(p.spill_tail, kResChunk);
    left = kResChunk;
    if (chunk_state >= (1u << 28)) {
      chunk_state = 0;
      const unsigned s1 = claim(p.spill_tail, 1);
      if (s1 < p.spill_cap) p.spill[s1] = SpillEntry{a, b, rs, jt};
      else atomicOr(p.status, kStatusSpillFull);
      return;
    }
  }
  const unsigned slot = chunk_state & 0x0FFFFFFFu;
  chunk_state = (slot + 1) | ((left - 1) << 28);
  if (slot < p.spill_cap) p.spill[slot] = SpillEntry{a, b, rs, jt};
  else atomicOr(p.status, kStatusSpillFull);
}

template <int MINB>
__global__ void __launch_bounds__(kBlock, MINB) chain4_kernel(DevIndex X, BatchedParams p) {
  const uint32_t n_reads_ = p.n_reads_dev ? *p.n_reads_dev : p.n_reads;
  __shared__ uint32_t c_res[kBlock], c_spill[kBlock];
  const int tid = threadIdx.x;
  c_res[tid] = 0;
  c_spill[tid] = 0;
  uint32_t read = claim(p.chain_ctr, 1);
  uint32_t nxt = read < n_reads_ ? claim(p.chain_ctr, 1) : 0xFFFFFFFFu;
  uint64_t nb0 = 0, nb1 = 0;
  uint32_t nok = 0;
  if (nxt < n_reads_) {
    nb0 = p.offs[nxt];
    nb1 = p.offs[nxt + 1];
    nok = p.ok[nxt];
  }
  uint64_t b0 = 0, b1 = 0;
  uint32_t okr = 0;
  if (read < n_reads_) {
    b0 = p.offs[read];
    b1 = p.offs[read + 1];
    okr = p.ok[read];
  }
  while (read < n_reads_) {
    const int len = (int)(b1 - b0);
    if (okr && len >= 3 && len <= 32767) {
      const uint8_t* W = p.codes + b0;
      const int n = len - 1;
      // chains: 0 '+' bwd, 1 '+' fwd, 2 '-' bwd, 3 '-' fwd
      uint32_t k0 = 0, l0 = X.top, k1 = 0, l1 = X.top, k2 = 0, l2 = X.top, k3 = 0, l3 = X.top;
      uint32_t pk0 = 0, pl0 = X.top, pk1 = 0, pl1 = X.top, pk2 = 0, pl2 = X.top, pk3 = 0, pl3 = X.top;
      uint32_t alive = 0xFu;
      for (int t = 0; t <= n; ++t) {
        const int jb = n - t, jf = t;
        const uint32_t bb = W[jb], bf = W[jf];
        if (alive & 1u) bw_step(X, View{0, 0}, bb, k0, l0);
        if (alive & 2u) bw_step(X, View{1, 0}, bf, k1, l1);
        if (alive & 4u) bw_step(X, View{1, 1}, bb, k2, l2);
        if (alive & 8u) bw_step(X, View{0, 1}, bf, k3, l3);
        // backward chains: entry at jb vs entry at J = jb + 1; window [2, n/2], block at J = 1
        // forward chains:  entry at jf vs entry at J = jf - 1; window [n/2 - 1, n - 2], block at n - 1
        const int Jb = jb + 1, Jf = jf - 1;
        const bool wb = Jb >= 2 && Jb <= n / 2;
        const bool wf = Jf >= n / 2 - 1 && Jf <= n - 1 && jf >= 1;
        const uint32_t tf = (uint32_t)Jf | ((Jf == n - 1 ? kBlkN : kCpFwd) << 16);
        const uint32_t tb = (uint32_t)Jb | (kCpBwd << 16);
#define HPG_CHAIN_TAIL(I, K, L, PK, PL, WIN, JT, STRAND, BWD)                                      \
  if (alive & (1u << I)) {                                                                         \
    const bool differ = (L - K) != (PL - PK);                                                      \
    if (differ && WIN) {                                                                           \
      uint32_t cs = c_spill[tid];                                                                  \
      spill_push(p, cs, PK, PL, (read << 1) | STRAND, JT);                                         \
      c_spill[tid] = cs;                                                                           \
    }                                                                                              \
    if (K > L || (BWD ? jb == 0 : jf == n)) {                                                      \
      if (BWD && jb == 0) {                                                                        \
        const uint32_t rs_ = (read << 1) | STRAND;                                                 \
        if (K <= L) {                                                                              \
          uint32_t r = c_res[tid];                                                                 \
          const unsigned slot = res_slot(p, r);                                                    \
          c_res[tid] = r;                                                                          \
          write_hit(p, slot, rs_, order_key(0, 0, 0), K, L, pack_meta(0, 0, 0, 0, 0));             \
        }                                                                                          \
        if (differ) {                                                                              \
          uint32_t cs = c_spill[tid];                                                              \
          spill_push(p, cs, PK, PL, rs_, 1u | (kBlk1 << 16));                                      \
          c_spill[tid] = cs;                                                                       \
        }                                                                                          \
      }                                                                                            \
      alive &= ~(1u << I);                                                                         \
    } else {                                                                                       \
      PK = K;                                                                                      \
      PL = L;                                                                                      \
    }                                                                                              \
  }
        HPG_CHAIN_TAIL(0, k0, l0, pk0, pl0, wb, tb, 0u, true)
        HPG_CHAIN_TAIL(1, k1, l1, pk1, pl1, wf, tf, 0u, false)
        HPG_CHAIN_TAIL(2, k2, l2, pk2, pl2, wb, tb, 1u, true)
        HPG_CHAIN_TAIL(3, k3, l3, pk3, pl3, wf, tf, 1u, false)
#undef HPG_CHAIN_TAIL
        if (!alive) break;
      }
    }
    // next read: the prefetched one; prefetch the one after
    read = nxt;
    b0 = nb0;
    b1 = nb1;
    okr = nok;
    if (read < n_reads_) {
      nxt = claim(p.chain_ctr, 1);
      if (nxt < n_reads_) {
        nb0 = p.offs[nxt];
        nb1 = p.offs[nxt + 1];
        nok = p.ok[nxt];
      }
    }
  }
  {  // reserved but unused slots of the last chunks
    const uint32_t r = c_res[tid];
    for (unsigned i = 0, left = r >> 28, slot = r & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.res_cap) p.res[slot + i].rs = 0xFFFFFFFFu;
    const uint32_t q = c_spill[tid];
    for (unsigned i = 0, left = q >> 28, slot = q & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.spill_cap) p.spill[slot + i].rs = 0xFFFFFFFFu;
  }
}

// Phased lockstep variant: one lane per read runs the two vector searches of
// a phase together -- phase 0: '+' backward and '-' forward (both on the
// backward index), phase 1: '-' backward and '+' forward (forward index).
// Lanes then spend about one read length per read whatever the strand, the
// next read is claimed and fetched ahead, and only one direction's blocks
// are live in L2.  Change points go to the device queue for the drain launch.
template <int MINB>
__global__ void __launch_bounds__(kBlock, MINB) chain2_kernel(DevIndex X, BatchedParams p, int phase) {
  const uint32_t n_reads_ = p.n_reads_dev ? *p.n_reads_dev : p.n_reads;
  __shared__ uint32_t c_res[kBlock], c_spill[kBlock];
  const int tid = threadIdx.x;
  c_res[tid] = 0;
  c_spill[tid] = 0;
  const uint32_t sA = (uint32_t)phase, sB = 1u - (uint32_t)phase;  // strands of the backward / forward chain
  const View vA{(uint32_t)phase, sA}, vB{(uint32_t)phase, sB};
  uint32_t read = claim(p.chain_ctr, 1);
  uint32_t nxt = read < n_reads_ ? claim(p.chain_ctr, 1) : 0xFFFFFFFFu;
  uint64_t b0 = 0, b1 = 0, nb0 = 0, nb1 = 0;
  uint32_t okr = 0, nok = 0;
  if (read < n_reads_) {
    b0 = p.offs[read];
    b1 = p.offs[read + 1];
    okr = p.ok[read];
  }
  if (nxt < n_reads_) {
    nb0 = p.offs[nxt];
    nb1 = p.offs[nxt + 1];
    nok = p.ok[nxt];
  }
  uint32_t sectors = 0;
  while (read < n_reads_) {
    const int len = (int)(b1 - b0);
    if (okr && len >= 3 && len <= 32767) {
      const uint8_t* W = p.codes + b0;
      const int n = len - 1, half = n / 2;
      uint32_t kA = 0, lA = X.top, pkA = 0, plA = X.top, kB = 0, lB = X.top, pkB = 0, plB = X.top;
      bool aA = true, aB = true;
      uint32_t bA = W[n], bB = W[0];
      for (int t = 0; t <= n; ++t) {
        const int jb = n - t, jf = t;
        const uint32_t nbA = (aA && jb > 0) ? W[jb - 1] : 0u;  // next bases, fetched with this step's gathers
        const uint32_t nbB = (aB && jf < n) ? W[jf + 1] : 0u;
        if (p.census) sectors += (aA ? (((kA >> 6) == (lA >> 6)) ? 1u : 2u) : 0u) +
                                 (aB ? (((kB >> 6) == (lB >> 6)) ? 1u : 2u) : 0u);
        if (aA) bw_step(X, vA, bA, kA, lA);
        if (aB) bw_step(X, vB, bB, kB, lB);
        if (aA) {  // backward: entry at jb vs J = jb + 1; window [2, n/2], block at J = 1
          const int J = jb + 1;
          const bool differ = (lA - kA) != (plA - pkA);
          if (differ && J >= 2 && J <= half) {
            uint32_t cs = c_spill[tid];
            spill_push(p, cs, pkA, plA, (read << 1) | sA, (uint32_t)J | (kCpBwd << 16));
            c_spill[tid] = cs;
          }
          if (kA > lA || jb == 0) {
            if (jb == 0) {
              const uint32_t rs = (read << 1) | sA;
              if (kA <= lA) {
                uint32_t r = c_res[tid];
                const unsigned slot = res_slot(p, r);
                c_res[tid] = r;
                write_hit(p, slot, rs, order_key(0, 0, 0), kA, lA, pack_meta(0, 0, 0, 0, 0));
              }
              if (differ) {
                uint32_t cs = c_spill[tid];
                spill_push(p, cs, pkA, plA, rs, 1u | (kBlk1 << 16));
                c_spill[tid] = cs;
              }
            }
            aA = false;
          } else {
            pkA = kA;
            plA = lA;
            bA = nbA;
          }
        }
        if (aB) {  // forward: entry at jf vs J = jf - 1; window [n/2 - 1, n - 2], block at n - 1
          const int J = jf - 1;
          const bool differ = (lB - kB) != (plB - pkB);
          if (differ && jf >= 1 && J >= half - 1 && J <= n - 1) {
            uint32_t cs = c_spill[tid];
            spill_push(p, cs, pkB, plB, (read << 1) | sB, (uint32_t)J | ((J == n - 1 ? kBlkN : kCpFwd) << 16));
            c_spill[tid] = cs;
          }
          if (kB > lB || jf == n) {
            aB = false;
          } else {
            pkB = kB;
            plB = lB;
            bB = nbB;
          }
        }
        if (!aA && !aB) break;
      }
    }
    read = nxt;
    b0 = nb0;
    b1 = nb1;
    okr = nok;
    if (read < n_reads_) {
      nxt = claim(p.chain_ctr, 1);
      if (nxt < n_reads_) {
        nb0 = p.offs[nxt];
        nb1 = p.offs[nxt + 1];
        nok = p.ok[nxt];
      }
    }
  }
  {  // reserved but unused slots of the last chunks
    const uint32_t r = c_res[tid];
    for (unsigned i = 0, left = r >> 28, slot = r & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.res_cap) p.res[slot + i].rs = 0xFFFFFFFFu;
    const uint32_t q = c_spill[tid];
    for (unsigned i = 0, left = q >> 28, slot = q & 0x0FFFFFFFu; i < left; ++i)
      if (slot + i < p.spill_cap) p.spill[slot + i].rs = 0xFFFFFFFFu;
  }
  if (p.census) atomicAdd(p.census, (unsigned long long)sectors);
}

// ------------------------------------------------------------- finalize --

__global__ void scatter_hits_kernel(const PendingHit* __restrict__ res, const unsigned int* res_total,
                                    const uint64_t* __restrict__ seg_off, PendingHit* __restrict__ sorted,
                                    uint32_t res_cap, uint32_t* __restrict__ cursor, const unsigned* gate) {
  if (gate && *gate) return;  // a pool overflowed: the graph's host reruns the batch
  const uint32_t n = min(*res_total, res_cap);
  const uint32_t stride = gridDim.x * blockDim.x;
  // four entries a thread and round, each stage's loads and atomics issued together
  for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
    PendingHit h[4];
    uint64_t at[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t i = i0 + u * stride;
      if (i < n) h[u] = res[i];
      else h[u].rs = 0xFFFFFFFFu;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)  // 0xFFFFFFFF: past the pool, or reserved but never written (chunk tail)
      if (h[u].rs != 0xFFFFFFFFu) at[u] = seg_off[h[u].rs];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (h[u].rs != 0xFFFFFFFFu) at[u] += atomicAdd(&cursor[h[u].rs], 1u);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (h[u].rs != 0xFFFFFFFFu) sorted[at[u]] = h[u];
  }
}

constexpr uint32_t kLongList = 32;  // longer lists are sorted by a whole block (sort_long_lists_kernel)
constexpr int kRankTpb = 512, kRankTile = 2048;

__global__ void sort_truncate_kernel(PendingHit* __restrict__ sorted, const uint64_t* __restrict__ seg_off,
                                     uint32_t n_rs, uint32_t max_results, uint32_t* __restrict__ kept,
                                     uint8_t* __restrict__ trunc, const uint32_t* max_dev, const unsigned* gate,
                                     uint32_t* __restrict__ longs, unsigned* n_longs, uint32_t longs_cap) {
  const uint32_t rs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rs >= n_rs) return;
  if (gate && *gate) return;
  if (max_dev) max_results = *max_dev;
  const uint64_t b = seg_off[rs], e = seg_off[rs + 1];
  const uint64_t cnt = e - b;
  const uint32_t keep = (uint32_t)(cnt < max_results ? cnt : max_results);
  kept[rs] = keep;
  trunc[rs] = cnt > max_results ? 1 : 0;
  if (keep == 0) return;
  if (cnt > kLongList) {  // the long sort's work (the list holds enough room for every such list)
    if (longs) {
      const unsigned q = atomicAdd(n_longs, 1u);
      if (q < longs_cap) longs[q] = rs;
    }
    return;
  }
  // insertion sort by key (short list; keys are unique within a list)
  for (uint64_t i = b + 1; i < e; ++i) {
    const PendingHit x = sorted[i];
    uint64_t j = i;
    while (j > b && sorted[j - 1].key > x.key) {
      sorted[j] = sorted[j - 1];
      --j;
    }
    sorted[j] = x;
  }
}

// Lists longer than kLongList (low-complexity reads emit thousands of pending
// hits), one list at a time per block.  Up to kRankTile entries: a bitonic
// sort of the (key, position) pairs in shared memory, O(m log^2 m / 512).
// Longer: the rank of an entry is the number of entries of its list with a
// smaller pair, counted against tiles of the list's keys in shared memory,
// O(m^2 / 512).  Entries placed below the kept count are written to `scratch`
// (the unsorted pending array, dead after the scatter) and copied back.
__global__ void __launch_bounds__(kRankTpb)
    sort_long_lists_kernel(PendingHit* __restrict__ sorted, PendingHit* __restrict__ scratch,
                           const uint64_t* __restrict__ seg_off, uint32_t n_rs, const uint32_t* __restrict__ kept,
                           const unsigned* gate, const uint32_t* __restrict__ work, const unsigned* n_work,
                           uint32_t work_cap) {
  if (gate && *gate) return;
  __shared__ uint64_t tile[kRankTile];
  __shared__ uint32_t longs[kRankTpb];
  __shared__ uint32_t n_long;
  // with a work list: its entries, a block each in turn; else every list, found by a scan
  const uint64_t n_items = work ? min(*n_work, work_cap) : n_rs;
  const uint64_t per_round = work ? 1 : kRankTpb;
  for (uint64_t base = (uint64_t)blockIdx.x * per_round; base < n_items; base += (uint64_t)gridDim.x * per_round) {
    if (threadIdx.x == 0) n_long = 0;
    __syncthreads();
    if (work) {
      if (threadIdx.x == 0) {
        longs[0] = work[base];
        n_long = 1;
      }
    } else {
      const uint64_t rs = base + threadIdx.x;
      if (rs < n_rs && seg_off[rs + 1] - seg_off[rs] > kLongList && kept[rs] > 0)
        longs[atomicAdd(&n_long, 1u)] = (uint32_t)rs;
    }
    __syncthreads();
    const uint32_t nl = n_long;
    for (uint32_t q = 0; q < nl; ++q) {
      const uint32_t r = longs[q];
      const uint64_t b = seg_off[r];
      const uint32_t m = (uint32_t)(seg_off[r + 1] - b), keep = kept[r];
      if (m <= kRankTile) {
        // bitonic sort of (key, position) pairs in shared memory, padded to a power of two
        uint32_t P = 64;
        while (P < m) P <<= 1;
        __syncthreads();  // the previous list's tile is no longer read
        for (uint32_t t = threadIdx.x; t < P; t += kRankTpb)
          tile[t] = t < m ? ((uint64_t)sorted[b + t].key << 32 | t) : ~0ull;
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1) {
          for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = threadIdx.x; t < P / 2; t += kRankTpb) {
              const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), q2 = i + j;
              const uint64_t x = tile[i], y = tile[q2];
              if ((x > y) == ((i & k) == 0)) {
                tile[i] = y;
                tile[q2] = x;
              }
            }
            __syncthreads();
          }
        }
        for (uint32_t t = threadIdx.x; t < keep; t += kRankTpb) scratch[b + t] = sorted[b + (uint32_t)tile[t]];
        __syncthreads();  // every entry written before the copy back
        for (uint32_t i = threadIdx.x; i < keep; i += kRankTpb) sorted[b + i] = scratch[b + i];
        __syncthreads();  // the list is final before the next one reuses the tile
        continue;
      }
      for (uint32_t i0 = 0; i0 < m; i0 += kRankTpb) {
        const uint32_t i = i0 + threadIdx.x;
        const uint64_t mine = i < m ? ((uint64_t)sorted[b + i].key << 32 | i) : ~0ull;
        uint32_t rank = 0;
        for (uint32_t t0 = 0; t0 < m; t0 += kRankTile) {
          const uint32_t tn = min((uint32_t)kRankTile, m - t0);
          __syncthreads();  // the previous tile is no longer read
          for (uint32_t t = threadIdx.x; t < tn; t += kRankTpb)
            tile[t] = (uint64_t)sorted[b + t0 + t].key << 32 | (t0 + t);
          __syncthreads();
          for (uint32_t t = 0; t < tn; ++t) rank += tile[t] < mine ? 1u : 0u;
        }
        if (i < m && rank < keep) scratch[b + rank] = sorted[b + i];
      }
      __syncthreads();  // every rank written before the copy back
      for (uint32_t i = threadIdx.x; i < keep; i += kRankTpb) sorted[b + i] = scratch[b + i];
      __syncthreads();  // the list is final before the next one reuses the tile
    }
    __syncthreads();  // n_long and longs are read before they are reset
  }
}

__device__ __forceinline__ void write_hit_record(const PendingHit& x, uint32_t rs, hpg_hit_t* __restrict__ hits,
                                                 uint32_t* __restrict__ rows, uint64_t at) {
  hpg_hit_t h;
  h.read = rs >> 1;
  h.strand = (uint8_t)(rs & 1u);
  h.dir = (uint8_t)(x.meta & 1u);
  h.nm = (uint8_t)((x.meta >> 1) & 1u);
  h.err_kind = (uint8_t)((x.meta >> 2) & 3u);
  h.err_base = (uint8_t)((x.meta >> 4) & 0xFFu);
  h.pad0 = 0;
  h.err_pos = (int16_t)(uint16_t)(x.meta >> 16);
  h.pad1 = 0;
  h.k = (int64_t)x.k;
  h.l = (int64_t)x.l;
  hits[at] = h;
  rows[at] = x.k <= x.l ? x.l - x.k + 1 : 0u;
}

// A thread per (read, strand) list; with skip_long the lists of more than
// kLongList pending hits are left to expand_long_hits_kernel.
__global__ void expand_hits_kernel(const PendingHit* __restrict__ sorted, const uint64_t* __restrict__ seg_off,
                                   const uint64_t* __restrict__ hit_off, const uint32_t* __restrict__ kept,
                                   uint32_t n_rs, hpg_hit_t* __restrict__ hits, uint32_t* __restrict__ rows,
                                   const unsigned* gate, int skip_long) {
  const uint32_t rs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rs >= n_rs) return;
  if (gate && *gate) return;
  const uint32_t m = kept[rs];
  const uint64_t b = seg_off[rs], o = hit_off[rs];
  if (skip_long && seg_off[rs + 1] - b > kLongList) return;
  for (uint32_t i = 0; i < m; ++i) write_hit_record(sorted[b + i], rs, hits, rows, o + i);
}

// The long lists the short sort collected, a block per list.
__global__ void expand_long_hits_kernel(const PendingHit* __restrict__ sorted, const uint64_t* __restrict__ seg_off,
                                        const uint64_t* __restrict__ hit_off, const uint32_t* __restrict__ kept,
                                        hpg_hit_t* __restrict__ hits, uint32_t* __restrict__ rows,
                                        const unsigned* gate, const uint32_t* __restrict__ work,
                                        const unsigned* n_work, uint32_t work_cap) {
  if (gate && *gate) return;
  const uint32_t n = min(*n_work, work_cap);
  for (uint32_t q = blockIdx.x; q < n; q += gridDim.x) {
    const uint32_t rs = work[q];
    const uint32_t m = kept[rs];
    const uint64_t b = seg_off[rs], o = hit_off[rs];
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) write_hit_record(sorted[b + i], rs, hits, rows, o + i);
  }
}

// --------------------------------------------------------------- locate --

// Rows on the backward index fill the item array from the front, rows on the
// forward index from the back, so walks claimed in order touch one direction
// at a time.  A block takes 256 consecutive hits a round: one scan of the
// (backward, forward) row counts over the block, one atomic per direction.
constexpr int kExpandTpb = 256;

__global__ void __launch_bounds__(kExpandTpb)
    expand_rows_kernel(const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ loc_off, uint32_t n_hits,
                       uint64_t n_locs, const uint64_t* __restrict__ read_offs, RowItem* __restrict__ items,
                       unsigned int* __restrict__ side, LocateSizes z) {
  if (z.status) {  // graph form: sizes from device memory, rows checked against the item capacity
    if (*z.status) return;
    n_hits = (uint32_t)*z.n_hits;
    n_locs = *z.n_locs;
    if (n_locs > z.locs_cap) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(z.status, kStatusLocFull);
      return;
    }
  }
  __shared__ uint64_t s_warp[kExpandTpb / 32];
  __shared__ uint64_t s_base;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint64_t h0 = (uint64_t)blockIdx.x * kExpandTpb; h0 < n_hits; h0 += (uint64_t)gridDim.x * kExpandTpb) {
    const uint64_t h = h0 + threadIdx.x;
    RowItem it{0, 0, 0, 0};
    uint32_t cnt = 0, phys = 0, k = 0;
    uint64_t b = 0;
    if (h < n_hits) {
      const hpg_hit_t x = hits[h];
      b = loc_off[h];
      cnt = (uint32_t)(loc_off[h + 1] - b);
      if (cnt) {
        const uint64_t len = read_offs[x.read + 1] - read_offs[x.read];
        const uint32_t err = x.nm ? x.err_kind : 0u;
        phys = (uint32_t)x.dir ^ (uint32_t)x.strand;  // direction = type ? dir : !dir, type = !strand
        it.hit = (uint32_t)h;
        it.phys_len = (phys << 31) | (uint32_t)(len - (err == 1 ? 1 : 0) + (err == 3 ? 1 : 0));
        k = (uint32_t)x.k;
      }
    }
    // (forward << 32 | backward) row counts, scanned over the block
    const uint64_t v = phys ? (uint64_t)cnt << 32 : (uint64_t)cnt;
    uint64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t tot = 0;
      for (int w = 0; w < kExpandTpb / 32; ++w) {
        const uint64_t t = s_warp[w];
        s_warp[w] = tot;
        tot += t;
      }
      const uint32_t b0 = (uint32_t)tot ? atomicAdd(&side[0], (uint32_t)tot) : 0u;
      const uint32_t b1 = (uint32_t)(tot >> 32) ? atomicAdd(&side[1], (uint32_t)(tot >> 32)) : 0u;
      s_base = (uint64_t)b1 << 32 | b0;
    }
    __syncthreads();
    const uint64_t excl = s_base + s_warp[warp] + incl - v;
    const uint32_t at = phys ? (uint32_t)(excl >> 32) : (uint32_t)excl;
    // a hit's rows: up to 4 by its own thread; more (repeats, up to the locate
    // limit) by the whole warp, 32 rows a round, so one long hit does not hold
    // the block for thousands of serial stores
    if (cnt <= 4) {
      for (uint32_t i = 0; i < cnt; ++i) {
        it.row = k + i;
        it.out = (uint32_t)(b + i);
        items[phys ? n_locs - 1 - (at + i) : at + i] = it;
      }
    }
    unsigned big = __ballot_sync(0xFFFFFFFFu, cnt > 4);
    while (big) {
      const int j = __ffs(big) - 1;
      big &= big - 1;
      const uint32_t cj = __shfl_sync(0xFFFFFFFFu, cnt, j), aj = __shfl_sync(0xFFFFFFFFu, at, j);
      const uint32_t kj = __shfl_sync(0xFFFFFFFFu, k, j), pj = __shfl_sync(0xFFFFFFFFu, phys, j);
      const uint32_t bj = (uint32_t)__shfl_sync(0xFFFFFFFFu, b, j);
      RowItem w;
      w.hit = __shfl_sync(0xFFFFFFFFu, it.hit, j);
      w.phys_len = __shfl_sync(0xFFFFFFFFu, it.phys_len, j);
      for (uint32_t i = lane; i < cj; i += 32) {
        w.row = kj + i;
        w.out = bj + i;
        items[pj ? n_locs - 1 - (aj + i) : aj + i] = w;
      }
    }
    __syncthreads();  // s_warp and s_base are rewritten next round
  }
}

constexpr unsigned kRowsPerClaim = 4;
// Lanes whose walk reached a sampled row (or that hold no row) wait, masked,
// until this many lanes of their converged group have (or all have), and then
// finish their rows and start the next ones together: a finish makes dependent
// loads (the SA sample, the karyotype, the next row item), and a warp that
// waited for one or two finishing lanes almost every step ran at a quarter of
// the gather rate.
constexpr unsigned kLocateBatch = 8;

__global__ void __launch_bounds__(kBlock)
    locate_persistent_kernel(DevIndex X, const RowItem* __restrict__ items, uint64_t n_locs,
                             hpg_loc_t* __restrict__ out, unsigned int* row_ctr, unsigned long long* census,
                             LocateSizes z) {
  if (z.status) {
    if (*z.status) return;  // includes an item capacity overflow found by expand_rows_kernel
    n_locs = *z.n_locs;
  }
  uint32_t r = 0, left = 0;
  uint32_t i = 0, j = 0, slot = 0;
  RowItem it{0, 0, 0, 0};
  // Software pipeline: the next row item of the lane's claim is loaded while the
  // current walk runs, and a finished walk's sample is loaded then written out at
  // the lane's next refill, so a refill waits on no load.
  RowItem nx{0, 0, 0, 0};
  RowItem pit{0, 0, 0, 0};  // the finished walk whose output is pending
  uint32_t ps = 0, pj = 0;  // its sample and steps
  bool pending = false;
  bool active = false, reached = false;
  uint32_t sectors = 0;
  auto finish = [&]() {  // the pending walk's key and chromosome
    const uint32_t sa = (ps + pj) % X.walk_mod;
    const uint32_t phys = pit.phys_len >> 31;
    const uint64_t len_calc = pit.phys_len & kRowLenMask;
    uint64_t key = sa;
    if (phys && (pit.phys_len & kRowKey32))  // an int length: the SA_TYPE (32-bit) difference wraps
      key = (uint32_t)((X.top + 1u) - sa - (uint32_t)len_calc - 1u);
    else if (phys)
      key = (uint64_t)((X.top + 1u) - sa) - len_calc - 1u;
    const uint32_t id = kar_search(X, key);
    hpg_loc_t o;
    o.key = key;
    o.hit = pit.hit;
    o.pad = 0;
    if (key + len_calc <= X.kar_offset[id]) {
      o.valid = 1;
      o.chrom = id - 1;
      o.position = X.kar_start[id - 1] + (key - X.kar_offset[id - 1]);
    } else {
      o.valid = 0;
      o.chrom = 0;
      o.position = 0;
    }
    out[pit.out] = o;
    pending = false;
  };
  for (;;) {
    // one step of the walk: the row's mark entry and block are fetched together;
    // a text-sampled row ends it (at most ratio - 1 LF steps), else LF moves on
    if (active && !reached) {
      const DevDir D = dir_of(X, it.phys_len >> 31);
      uint32_t cnt[4];
      uint4 bits;
      const uint4 mk = load_mark(D, i, X.load_mode);
      load_block_m(D.occ + (i >> 6), X.load_mode, cnt, bits);
      sectors += 2;
      if (text_sampled(mk, i, slot)) {
        reached = true;
      } else {
        i = lf_from(X, D, i, cnt, bits);
        if (++j >= X.ratio) {  // only a corrupt index gets here
          atomicOr(X.err, kErrWalk);
          slot = 0;
          reached = true;
        }
      }
    }
    const bool done = !active || reached;
    const unsigned grp = __activemask();
    const unsigned ready = __ballot_sync(grp, done);
    if (!done) continue;
    if ((uint32_t)__popc(ready) < kLocateBatch && ready != grp) continue;  // wait for more lanes
    if (pending) finish();  // the previous walk of this lane: its sample has arrived by now
    if (active) {  // the walk reached a text-sampled row: load the sample, write the row next time
      ps = dir_of(X, it.phys_len >> 31).T[slot];
      ++sectors;
      pj = j;
      pit = it;
      pending = true;
      active = false;
      reached = false;
    }
    if (left == 0) {
      r = claim(row_ctr, kRowsPerClaim);
      left = kRowsPerClaim;
      if (r < n_locs) nx = items[r];
    } else {
      ++r;
    }
    --left;
    if (r >= n_locs) break;
    it = nx;
    if (left > 0 && r + 1 < n_locs) nx = items[r + 1];  // the next row, loaded during this walk
    i = it.row;
    j = 0;
    active = true;
  }
  if (pending) finish();
  if (census) atomicAdd(census, (unsigned long long)sectors);
}

template <int MINB>
void launch_chain_m(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, int phase,
                    cudaStream_t s) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain_kernel<MINB>, kBlock, 0);
  if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
  if (per_sm < 1) per_sm = 1;
  count_launches(1);
  chain_kernel<MINB><<<num_sms * per_sm, kBlock, 0, s>>>(X, p, t.chunk < 1 ? 1 : t.chunk, phase);
}

template <int D, int MINB>
void launch_search_dm(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, bool drain,
                      cudaStream_t s) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_search_kernel<D, MINB, false>, kBlock, 0);
  if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
  if (per_sm < 1) per_sm = 1;
  count_launches(1);
  const int ch = t.chunk < 1 ? 1 : t.chunk;
  if (p.census)
    batched_search_kernel<D, MINB, true><<<num_sms * per_sm, kBlock, 0, s>>>(X, p, drain ? 1 : 0, ch);
  else
    batched_search_kernel<D, MINB, false><<<num_sms * per_sm, kBlock, 0, s>>>(X, p, drain ? 1 : 0, ch);
}

template <int D>
void launch_search_d(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, bool drain,
                     cudaStream_t s) {
  if (t.min_blocks >= 16)
    launch_search_dm<D, 16>(X, p, t, num_sms, drain, s);
  else if (t.min_blocks >= 12)
    launch_search_dm<D, 12>(X, p, t, num_sms, drain, s);
  else if (t.min_blocks >= 10)
    launch_search_dm<D, 10>(X, p, t, num_sms, drain, s);
  else
    launch_search_dm<D, 1>(X, p, t, num_sms, drain, s);
}

template <int D>
int occupancy_d(const BatchedTuning& t) {
  int per_sm = 0;
  if (t.min_blocks >= 16)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_search_kernel<D, 16, false>, kBlock, 0);
  else if (t.min_blocks >= 12)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_search_kernel<D, 12, false>, kBlock, 0);
  else if (t.min_blocks >= 10)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_search_kernel<D, 10, false>, kBlock, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_search_kernel<D, 1, false>, kBlock, 0);
  if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
  return per_sm;
}

}  // namespace

int batched_max_blocks_per_sm(const BatchedTuning& t) {
  if (t.split == 3) return wave_max_blocks_per_sm(t);
  if (t.split == 2) {
    int per_sm = 0;
    if (t.min_blocks >= 16)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<16>, kBlock, 0);
    else if (t.min_blocks >= 12)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<12>, kBlock, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<1>, kBlock, 0);
    if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
    return per_sm;
  }
  if (t.split) {
    int per_sm = 0;
    if (t.split == 1) {
      if (t.min_blocks >= 16)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<16>, kBlock, 0);
      else if (t.min_blocks >= 12)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<12>, kBlock, 0);
      else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<1>, kBlock, 0);
      if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
      return per_sm;
    }
    if (t.min_blocks >= 16)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain_kernel<16>, kBlock, 0);
    else if (t.min_blocks >= 12)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain_kernel<12>, kBlock, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain_kernel<1>, kBlock, 0);
    if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
    return per_sm;
  }
  if (t.stack <= 2) return occupancy_d<2>(t);
  if (t.stack <= 4) return occupancy_d<4>(t);
  return occupancy_d<8>(t);
}

void launch_batched_search(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, bool drain,
                           cudaStream_t s) {
  if (t.split == 3 && !drain) {  // warp-cooperative chains and branches
    launch_wave_search(X, p, t, num_sms, s);
    return;
  }
  if (t.split == 2 && !drain) {  // lockstep chains, one lane per read
    int per_sm = 0;
    if (t.min_blocks >= 16) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<16>, kBlock, 0);
      count_launches(1);
      chain4_kernel<16><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p);
    } else if (t.min_blocks >= 12) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<12>, kBlock, 0);
      count_launches(1);
      chain4_kernel<12><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p);
    } else {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain4_kernel<1>, kBlock, 0);
      if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
      count_launches(1);
      chain4_kernel<1><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p);
    }
    return;
  }
  if (t.split == 1 && !drain && t.phase < 2) {  // phased lockstep: the phase's two chains per read
    int per_sm = 0;
    if (t.min_blocks >= 16) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<16>, kBlock, 0);
      count_launches(1);
      chain2_kernel<16><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p, t.phase);
    } else if (t.min_blocks >= 12) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<12>, kBlock, 0);
      count_launches(1);
      chain2_kernel<12><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p, t.phase);
    } else {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chain2_kernel<1>, kBlock, 0);
      if (t.blocks_per_sm > 0 && t.blocks_per_sm < per_sm) per_sm = t.blocks_per_sm;
      count_launches(1);
      chain2_kernel<1><<<num_sms * (per_sm > 0 ? per_sm : 1), kBlock, 0, s>>>(X, p, t.phase);
    }
    return;
  }
  if (t.split && !drain) {  // chains only; every change point goes to the queue
    const int phase = t.phase;
    if (t.min_blocks >= 16)
      launch_chain_m<16>(X, p, t, num_sms, phase, s);
    else if (t.min_blocks >= 12)
      launch_chain_m<12>(X, p, t, num_sms, phase, s);
    else
      launch_chain_m<1>(X, p, t, num_sms, phase, s);
    return;
  }
  if (t.stack <= 2)
    launch_search_d<2>(X, p, t, num_sms, drain, s);
  else if (t.stack <= 4)
    launch_search_d<4>(X, p, t, num_sms, drain, s);
  else
    launch_search_d<8>(X, p, t, num_sms, drain, s);
}

void launch_scatter_hits(const PendingHit* res, const unsigned int* res_total, const uint64_t* seg_off,
                         PendingHit* sorted, uint32_t res_cap, uint32_t* cursor, cudaStream_t s, const unsigned* gate) {
  count_launches(1);
  scatter_hits_kernel<<<1024, 256, 0, s>>>(res, res_total, seg_off, sorted, res_cap, cursor, gate);
}

size_t long_lists_cap(size_t res_cap) { return res_cap / (kLongList + 1) + 2; }

void launch_sort_truncate(PendingHit* sorted, PendingHit* scratch, const uint64_t* seg_off, uint32_t n_rs,
                          uint32_t max_results, uint32_t* kept, uint8_t* trunc, int num_sms, cudaStream_t s,
                          const uint32_t* max_dev, const unsigned* gate, uint32_t* longs, unsigned* n_longs,
                          uint32_t longs_cap) {
  if (!n_rs) return;
  const uint32_t cap = longs ? longs_cap : 0u;
  count_launches(1);
  sort_truncate_kernel<<<(n_rs + 255) / 256, 256, 0, s>>>(sorted, seg_off, n_rs, max_results, kept, trunc, max_dev,
                                                          gate, longs, n_longs, cap);
  uint64_t blocks = ((uint64_t)n_rs + kRankTpb - 1) / kRankTpb;
  if (blocks > 2ull * (uint64_t)num_sms) blocks = 2ull * (uint64_t)num_sms;
  count_launches(1);
  sort_long_lists_kernel<<<(unsigned)blocks, kRankTpb, 0, s>>>(sorted, scratch, seg_off, n_rs, kept, gate, longs,
                                                               n_longs, cap);
}

void launch_expand_hits(const PendingHit* sorted, const uint64_t* seg_off, const uint64_t* hit_off,
                        const uint32_t* kept, uint32_t n_rs, hpg_hit_t* hits, uint32_t* rows, cudaStream_t s,
                        const unsigned* gate, const uint32_t* longs, const unsigned* n_longs, uint32_t longs_cap,
                        int num_sms) {
  if (!n_rs) return;
  count_launches(1);
  expand_hits_kernel<<<(n_rs + 255) / 256, 256, 0, s>>>(sorted, seg_off, hit_off, kept, n_rs, hits, rows, gate,
                                                        longs ? 1 : 0);
  if (longs) {
    count_launches(1);
    expand_long_hits_kernel<<<2 * num_sms, 256, 0, s>>>(sorted, seg_off, hit_off, kept, hits, rows, gate, longs,
                                                        n_longs, longs_cap);
  }
}

void launch_locate_persistent(const DevIndex& X, const hpg_hit_t* hits, const uint64_t* loc_off, uint32_t n_hits,
                              uint64_t n_locs, const uint64_t* read_offs, hpg_loc_t* out, void* row_items,
                              unsigned int* row_ctr, unsigned long long* census, int num_sms, cudaStream_t s,
                              const LocateSizes& z) {
  if (!n_locs) return;
  RowItem* items = static_cast<RowItem*>(row_items);
  unsigned int* side = row_ctr + 1;  // two counters after the row claim counter
  cudaMemsetAsync(side, 0, 8, s);
  count_launches(1);
  // graph form: grid-stride over the hits, 8 blocks per SM
  const uint64_t hit_grid = z.status ? 8ull * num_sms : (n_hits + kExpandTpb - 1) / kExpandTpb;
  expand_rows_kernel<<<(unsigned)(hit_grid ? hit_grid : 1), kExpandTpb, 0, s>>>(hits, loc_off, n_hits, n_locs,
                                                                                read_offs, items, side, z);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, locate_persistent_kernel, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = (uint64_t)num_sms * per_sm;
  const uint64_t need = (n_locs + kBlock * kRowsPerClaim - 1) / (kBlock * kRowsPerClaim);
  if (need < blocks) blocks = need;
  count_launches(1);
  locate_persistent_kernel<<<(unsigned)blocks, kBlock, 0, s>>>(X, items, n_locs, out, row_ctr, census, z);
}

void launch_locate_items(const DevIndex& X, const RowItem* items, uint64_t n_items, hpg_loc_t* out,
                         unsigned int* row_ctr, int num_sms, cudaStream_t s) {
  if (!n_items) return;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, locate_persistent_kernel, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = (uint64_t)num_sms * per_sm;
  const uint64_t need = (n_items + kBlock * kRowsPerClaim - 1) / (kBlock * kRowsPerClaim);
  if (need < blocks) blocks = need;
  cudaMemsetAsync(row_ctr, 0, 4, s);
  count_launches(1);
  locate_persistent_kernel<<<(unsigned)blocks, kBlock, 0, s>>>(X, items, n_items, out, row_ctr, nullptr,
                                                               LocateSizes());
}

size_t locate_row_item_bytes() { return sizeof(RowItem); }

namespace {

// One thread per string of L symbols: the search from the full interval over
// them on physical direction d, stopped where it fails.
__global__ void build_kmer_kernel(DevIndex X, uint32_t d, uint32_t L, uint2* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (1u << (2 * L))) return;
  uint32_t k = 0, l = X.top;
  for (uint32_t i = 0; i < L; ++i) {
    bw_step(X, View{d, 0}, (c >> (2 * (L - 1 - i))) & 3u, k, l);
    if (k > l) break;
  }
  out[c] = make_uint2(k, l);
}

}  // namespace

void launch_build_kmer(const DevIndex& X, uint32_t d, uint32_t L, uint2* out, cudaStream_t s) {
  const uint32_t n = 1u << (2 * L);
  count_launches(1);
  build_kmer_kernel<<<(n + 255) / 256, 256, 0, s>>>(X, d, L, out);
}


void launch_search_stage(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms,
                         unsigned int* ctr, uint32_t* long_list, uint32_t long_cap, SpillEntry* blocks,
                         uint32_t block_cap, cudaEvent_t mid, bool external, cudaStream_t s) {
  auto mark = [&]() {
    if (!mid) return;
    if (external)
      cudaEventRecordWithFlags(mid, s, cudaEventRecordExternal);
    else
      cudaEventRecord(mid, s);
  };
  if (t.split == 1) {
    // one index direction at a time: chains on the backward index and their
    // change points, then chains on the forward index and theirs
    BatchedTuning t0 = t;
    BatchedParams p1 = p;
    p1.chain_ctr = ctr + 8;
    t0.phase = 0;
    launch_batched_search(X, p, t0, num_sms, false, s);
    launch_batched_search(X, p, t0, num_sms, true, s);
    cudaMemcpyAsync(ctr + 1, ctr + 2, 4, cudaMemcpyDeviceToDevice, s);  // drain resumes at the queue tail
    mark();
    t0.phase = 1;
    launch_batched_search(X, p1, t0, num_sms, false, s);
    launch_batched_search(X, p1, t0, num_sms, true, s);
  } else if (t.split == 3) {
    // warp-cooperative launches (one per index direction, or one for both), the
    // fused kernel over the reads too long for a warp's group buffer, then the
    // change points that did not fit the warps' stacks, and the blocks
    BatchedParams pw = p;
    pw.wave_group = (uint32_t)(t.group < 1 ? 1 : (t.group > 32 ? 32 : t.group));
    pw.long_list = long_list;
    pw.long_n = ctr + 10;
    pw.long_cap = long_cap;
    pw.blocks = blocks;
    pw.block_n = ctr + 13;
    pw.block_cap = block_cap;
    if (t.dir_split == 2) {
      pw.dir_split = 2;
      launch_wave_search(X, pw, t, num_sms, s);
      pw.dir_split = 3;
      launch_wave_search(X, pw, t, num_sms, s);
    } else {
      pw.dir_split = 0;
      launch_wave_search(X, pw, t, num_sms, s);
    }
    BatchedParams pl = p;
    BatchedTuning tl = t;
    tl.split = 0;
    tl.dir_split = 0;
    // reads above kWaveLongMin bases are at most 1/4000 of the bases: two
    // blocks per SM serve them, and an empty list costs a short launch
    tl.blocks_per_sm = 2;
    pl.dir_split = 0;
    pl.chain_ctr = ctr + 11;
    pl.read_list = long_list;
    pl.read_list_n = ctr + 10;
    pl.long_cap = long_cap;
    launch_batched_search(X, pl, tl, num_sms, false, s);
    mark();
    // queued change points' branches, eight per change point; the blocks among
    // them join the block list, which the fused kernel's drain then empties
    launch_wave_branches(X, p, blocks, ctr + 13, block_cap, num_sms, s);
    BatchedParams pb = p;
    pb.spill = blocks;
    pb.spill_head = ctr + 12;
    pb.spill_tail = ctr + 13;
    pb.spill_cap = block_cap;
    tl.blocks_per_sm = t.blocks_per_sm;
    launch_batched_search(X, pb, tl, num_sms, true, s);
  } else if (p.dir_split == 2) {  // one index direction after the other, then the queued change points
    launch_batched_search(X, p, t, num_sms, false, s);
    BatchedParams p1 = p;
    p1.dir_split = 3;
    launch_batched_search(X, p1, t, num_sms, false, s);
    mark();
    launch_batched_search(X, p, t, num_sms, true, s);
  } else {
    launch_batched_search(X, p, t, num_sms, false, s);
    mark();
    launch_batched_search(X, p, t, num_sms, true, s);
  }
}

}  // namespace hpgbwt
