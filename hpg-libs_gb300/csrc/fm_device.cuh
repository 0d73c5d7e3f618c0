// fm_device.cuh -- HBM-resident FM-index layout and the device-side rank,
// backward-extension, LF and locate primitives shared by every kernel.
//
// Layout (one per physical direction: 0 = backward index of the text,
// 1 = forward index = backward index of the reversed text):
//
//   OccBlock occ[nblk]   32-byte blocks, one per 64 BWT rows:
//       cnt[b]   number of symbol b in BWT rows [0, 64q), '$' excluded
//       bits[4]  the 2-bit codes of rows 64q..64q+63 as two bit planes:
//                bits[0..1] = low code bit of rows 0..63 (one u64),
//                bits[2..3] = high code bit; the '$' row is stored as
//                code 0 and corrected in rank_block().  A rank inside the
//                block is then two bitwise ops and one popcount.
//   uint32 S[]           sampled SA, S[i/ratio] = SA[i] (the reference's S.vec);
//                        read only to derive the two arrays below, then freed
//   uint4 mark[nblk]     text-sampled rows (SA value a multiple of the ratio),
//                        one entry per 64 rows: x = such rows before the block,
//                        y/z = their bits for rows 0..31 / 32..63
//   uint32 T[]           SA values of the text-sampled rows, in row order
//
// A locate walk (LF until a sampled row) therefore ends within ratio - 1 steps
// instead of after a geometric number of them (text_samples.cu).
//
// One rank query therefore touches exactly one 32-byte sector, against two
// separate arrays (a 4-byte desp and an 8-byte count word) per query in the
// reference's comp_matrix (search/csafm.h:51-64,166-181).
//
// Reverse-complement views (backward_rev / forward_rev, search/csafm.c:3-100)
// swap C and O rows by complement; here the query symbol is complemented
// instead, so no table is copied.
#pragma once

#include <vector_types.h>

#include <cstdint>

namespace hpgbwt {

struct __align__(32) OccBlock {
  uint32_t cnt[4];
  uint32_t bits[4];
};

struct DevDir {
  const OccBlock* occ;
  const uint32_t* S;
  const uint4* mark;
  const uint32_t* T;
  uint32_t dollar;  // BWT row holding '$'
  uint32_t nblk;
};

struct DevIndex {
  DevDir dir[2];
  uint32_t C[4], C1[4];   // C counts symbols < b without '$'; C1 = C + 1
  uint32_t comp[4];       // complement of each code
  uint32_t comp_packed;   // the same, 2 bits per code: comp[b] = (comp_packed >> 2b) & 3
  uint32_t ratio;         // SA sampling ratio
  uint32_t ratio_shift;   // log2(ratio) when ratio is a power of two, else 0xFFFFFFFF
  uint32_t walk_mod;      // O.siz - 1 = n + 1: modulus of the SA walk (csafm.h:233)
  uint32_t top;           // n = size_SA - 1: initial l of every search
  const uint64_t* kar_offset;  // kar_size + 1 entries
  const uint64_t* kar_start;
  uint32_t kar_size;
  uint32_t* err;          // device error word (bit 0: an LF walk passed its bound: a corrupt index)
  uint32_t load_mode;     // how blocks are fetched, see load_block()
  // Start table of the batched search: for every string of kmer_len symbols
  // (first symbol in the top bits, in search order) the interval the search
  // reaches from the full interval after those steps on that physical
  // direction, or the failing interval (k > l) where it stopped.  kmer_len 0:
  // no table.
  const uint2* kmer[2];
  uint32_t kmer_len;
};

constexpr uint32_t kErrWalk = 1u;

// A search view: physical direction plus whether query symbols are complemented.
struct View {
  uint32_t d;
  uint32_t comp;
};

#ifdef __CUDACC__

// Entry p (0..3) of a 4-vector by selects, so that kernel-parameter arrays
// are never indexed with a register (which would copy them to local memory).
__device__ __forceinline__ uint32_t sel4(const uint32_t (&a)[4], uint32_t p) {
  const uint32_t lo = (p & 1u) ? a[1] : a[0];
  const uint32_t hi = (p & 1u) ? a[3] : a[2];
  return (p & 2u) ? hi : lo;
}

// Block fetch.  mode 0: two 16-byte loads through L1; 1: one 32-byte load;
// 2: one 32-byte load that skips L1 and asks L2 to keep the line (evict_last),
// so the index outlives the streamed reads and outputs in L2; 3: 32-byte load
// with the L2 hint only.  The mode is uniform across a launch.
__device__ __forceinline__ void load_block_m(const OccBlock* p, uint32_t mode, uint32_t (&cnt)[4], uint4& bits) {
  if (mode == 0) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    const uint4 c = __ldg(q);
    bits = __ldg(q + 1);
    cnt[0] = c.x;
    cnt[1] = c.y;
    cnt[2] = c.z;
    cnt[3] = c.w;
  } else if (mode == 1) {
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(cnt[0]), "=r"(cnt[1]), "=r"(cnt[2]), "=r"(cnt[3]), "=r"(bits.x), "=r"(bits.y), "=r"(bits.z),
                   "=r"(bits.w)
                 : "l"(p));
  } else if (mode == 2) {
    asm("ld.global.nc.L1::no_allocate.L2::evict_last.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(cnt[0]), "=r"(cnt[1]), "=r"(cnt[2]), "=r"(cnt[3]), "=r"(bits.x), "=r"(bits.y), "=r"(bits.z),
                   "=r"(bits.w)
                 : "l"(p));
  } else {
    asm("ld.global.nc.L2::evict_last.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(cnt[0]), "=r"(cnt[1]), "=r"(cnt[2]), "=r"(cnt[3]), "=r"(bits.x), "=r"(bits.y), "=r"(bits.z),
                   "=r"(bits.w)
                 : "l"(p));
  }
}

__device__ __forceinline__ void load_block(const OccBlock* p, uint32_t (&cnt)[4], uint4& bits) {
  load_block_m(p, 0, cnt, bits);
}

// One bit per row of the block: set where the row's code is p.
__device__ __forceinline__ uint64_t match_mask(const uint4& bits, uint32_t p) {
  const uint64_t lo = ((uint64_t)bits.y << 32) | bits.x;
  const uint64_t hi = ((uint64_t)bits.w << 32) | bits.z;
  return (lo ^ ((uint64_t)(p & 1u) - 1ull)) & (hi ^ ((uint64_t)((p >> 1) & 1u) - 1ull));
}

// The first r rows (r in 0..64).
__device__ __forceinline__ uint64_t prefix_mask(uint32_t r) { return r >= 64 ? ~0ull : ((1ull << r) - 1ull); }

// Number of symbol p among the first r rows (0..64) of a block.
__device__ __forceinline__ uint32_t count_prefix(const uint4& bits, uint32_t p, uint32_t r) {
  return (uint32_t)__popcll(match_mask(bits, p) & prefix_mask(r));
}

// Occurrences of physical symbol p in BWT rows [64q, 64q + r) plus cnt, with
// the '$' row (stored as code 0) taken out.
__device__ __forceinline__ uint32_t rank_block(const DevDir& D, uint32_t q, uint32_t p, uint32_t r,
                                               const uint32_t (&cnt)[4], const uint4& bits) {
  uint32_t v = sel4(cnt, p) + count_prefix(bits, p, r);
  if (p == 0 && q == (D.dollar >> 6) && r > (D.dollar & 63)) v -= 1;
  return v;
}

// get_O(p, k): symbol p in rows [0, k).  k in [0, n+1].
__device__ __forceinline__ uint32_t rank_lo(const DevDir& D, uint32_t p, uint32_t k) {
  uint32_t cnt[4];
  uint4 bits;
  const uint32_t q = k >> 6;
  load_block(D.occ + q, cnt, bits);
  return rank_block(D, q, p, k & 63, cnt, bits);
}

// get_O(p, l + 1): symbol p in rows [0, l].  l in [0, n].
__device__ __forceinline__ uint32_t rank_hi(const DevDir& D, uint32_t p, uint32_t l) {
  uint32_t cnt[4];
  uint4 bits;
  const uint32_t q = l >> 6;
  load_block(D.occ + q, cnt, bits);
  return rank_block(D, q, p, (l & 63) + 1, cnt, bits);
}

__device__ __forceinline__ DevDir dir_of(const DevIndex& X, uint32_t d) {
  DevDir D;
  D.occ = d ? X.dir[1].occ : X.dir[0].occ;
  D.S = d ? X.dir[1].S : X.dir[0].S;
  D.mark = d ? X.dir[1].mark : X.dir[0].mark;
  D.T = d ? X.dir[1].T : X.dir[0].T;
  D.dollar = d ? X.dir[1].dollar : X.dir[0].dollar;
  D.nblk = d ? X.dir[1].nblk : X.dir[0].nblk;
  return D;
}

// The first r rows of a block (r in 0..64) as a bit mask.  PTX clamps a
// shift amount above the width to the width, so r = 64 gives all ones.
__device__ __forceinline__ uint64_t row_mask(uint32_t r) {
  uint64_t m;
  asm("shl.b64 %0, %1, %2;" : "=l"(m) : "l"(1ull), "r"(r));
  return m - 1ull;
}

// BWiteration (search/runtime.h:38-42) over a view, on 32-bit interval ends.
// k in [0, n+1], l in [0, n] always hold for the intervals the search forms.
// When k and l share a block (the common case once an interval is small)
// one 32-byte sector serves both ranks.  The '$' row (stored as code 0) is
// taken out only for symbol 0 in the one block that holds it.
__device__ __forceinline__ void bw_step(const DevIndex& X, View v, uint32_t b, uint32_t& k, uint32_t& l) {
  const uint32_t p = v.comp ? ((X.comp_packed >> (2u * b)) & 3u) : b;
  const OccBlock* occ = v.d ? X.dir[1].occ : X.dir[0].occ;
  const uint32_t q0 = k >> 6, q1 = l >> 6;
  uint32_t cnt[4];
  uint4 bits;
  load_block_m(occ + q0, X.load_mode, cnt, bits);
  uint64_t m = match_mask(bits, p);
  const uint32_t c0 = sel4(cnt, p);
  uint32_t rk = c0 + (uint32_t)__popcll(m & row_mask(k & 63));
  uint32_t rl;
  if (q1 == q0) {
    rl = c0 + (uint32_t)__popcll(m & row_mask((l & 63) + 1));
  } else {
    load_block_m(occ + q1, X.load_mode, cnt, bits);
    m = match_mask(bits, p);
    rl = sel4(cnt, p) + (uint32_t)__popcll(m & row_mask((l & 63) + 1));
  }
  if (p == 0) {
    const uint32_t dollar = v.d ? X.dir[1].dollar : X.dir[0].dollar;
    if (k > dollar && q0 == (dollar >> 6)) rk -= 1;
    if (l >= dollar && q1 == (dollar >> 6)) rl -= 1;
  }
  const uint32_t c = sel4(X.C, p);  // C1 = C + 1 (checked when the index is loaded)
  k = c + 1u + rk;
  l = c + rl;
}

// LF of row i on a physical direction from its loaded block: row 0 for the
// '$' row, else C[b] + get_O(b, i+1) with b the row's symbol (csafm.h:215-231).
__device__ __forceinline__ uint32_t lf_from(const DevIndex& X, const DevDir& D, uint32_t i, const uint32_t (&cnt)[4],
                                            const uint4& bits) {
  if (i == D.dollar) return 0;
  const uint32_t q = i >> 6, r = i & 63;
  const uint32_t lo = r < 32 ? bits.x : bits.y, hi = r < 32 ? bits.z : bits.w;
  const uint32_t b = ((lo >> (r & 31)) & 1u) | (((hi >> (r & 31)) & 1u) << 1);
  return sel4(X.C, b) + rank_block(D, q, b, r + 1, cnt, bits);
}

__device__ __forceinline__ uint32_t lf_step(const DevIndex& X, const DevDir& D, uint32_t i) {
  uint32_t cnt[4];
  uint4 bits;
  load_block_m(D.occ + (i >> 6), X.load_mode, cnt, bits);
  return lf_from(X, D, i, cnt, bits);
}

// The reference's sampled rows: row index a multiple of the ratio.
__device__ __forceinline__ bool sampled_row(const DevIndex& X, uint32_t i) {
  return X.ratio_shift != 0xFFFFFFFFu ? (i & ((1u << X.ratio_shift) - 1u)) == 0 : (i % X.ratio) == 0;
}

__device__ __forceinline__ bool ratio_multiple(const DevIndex& X, uint32_t v) {
  return X.ratio_shift != 0xFFFFFFFFu ? (v & ((1u << X.ratio_shift) - 1u)) == 0 : (v % X.ratio) == 0;
}

// Mark entry of row i, fetched like the blocks (mode 2/3: kept in L2).
__device__ __forceinline__ uint4 load_mark(const DevDir& D, uint32_t i, uint32_t mode) {
  const uint4* p = D.mark + (i >> 6);
  uint4 m;
  if (mode >= 2) {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
        : "=r"(m.x), "=r"(m.y), "=r"(m.z), "=r"(m.w)
        : "l"(p), "l"(pol));
  } else
    m = __ldg(p);
  return m;
}

// Whether row i is text-sampled, and its slot in T.
__device__ __forceinline__ bool text_sampled(const uint4& m, uint32_t i, uint32_t& slot) {
  const uint32_t r = i & 63;
  const uint32_t w = r < 32 ? m.y : m.z;
  slot = m.x + (r < 32 ? 0u : (uint32_t)__popc(m.y)) + (uint32_t)__popc(w & ((1u << (r & 31)) - 1u));
  return (w >> (r & 31)) & 1u;
}

// getScompValue (csafm.h:208-235): walk LF to a sampled row, add the steps;
// here to a text-sampled row, so at most ratio - 1 steps (a longer walk means
// a corrupt index: the error bit is set and slot 0 taken).  The row's mark
// entry and block are fetched together; `sectors` counts them and the sample.
__device__ __forceinline__ uint32_t sa_value(const DevIndex& X, const DevDir& D, uint32_t m, uint32_t* sectors) {
  uint32_t i = m, j = 0, slot = 0;
  for (;;) {
    uint32_t cnt[4];
    uint4 bits;
    const uint4 mk = load_mark(D, i, X.load_mode);
    load_block_m(D.occ + (i >> 6), X.load_mode, cnt, bits);
    if (text_sampled(mk, i, slot)) break;
    i = lf_from(X, D, i, cnt, bits);
    if (++j >= X.ratio) {
      atomicOr(X.err, kErrWalk);
      slot = 0;
      break;
    }
  }
  *sectors = 2 * (j + 1) + 1;
  return (D.T[slot] + j) % X.walk_mod;
}

// binsearch (search/io.h:43-64): first offset greater than key.
__device__ __forceinline__ uint32_t kar_search(const DevIndex& X, uint64_t key) {
  uint32_t lo = 0, size = X.kar_size;
  while (size > 0) {
    const uint32_t w = size >> 1;
    if (X.kar_offset[lo + w] <= key) {
      lo += w + 1;
      size -= w + 1;
    } else {
      size = w;
    }
  }
  return lo;
}

#endif  // __CUDACC__

}  // namespace hpgbwt
