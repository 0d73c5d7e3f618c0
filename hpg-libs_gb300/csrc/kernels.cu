// kernels.cu -- plain-form kernels of the FM-index mapping pipeline:
// read encoding, exact search, BWSearch1 (one thread per read and strand),
// device-wide scan, ordered hit gather and the locate pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "kernels.cuh"
#include "search_core.cuh"

namespace hpgbwt {

std::atomic<unsigned long long> g_launches{0};

unsigned long long launch_count() { return g_launches.load(); }
void count_launches(unsigned n) { g_launches += n; }
void uncount_launches(unsigned long long n) { g_launches -= n; }

namespace {

constexpr int kTpb = 128;

inline unsigned grid_for(size_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// Coalesced encoding: each thread translates 16 consecutive bytes; a byte
// outside the alphabet clears its read's flag (found by binary search over
// the offsets; such reads are rare).
// With `n_dev` set the read count comes from device memory and the byte count
// is offs[n] (graph replays); the grid is then sized for the capacity.
__global__ void encode_kernel(const uint8_t* __restrict__ ascii, uint64_t total, const uint64_t* __restrict__ offs,
                              uint32_t n_reads, const uint8_t* __restrict__ table, uint8_t* __restrict__ codes,
                              uint8_t* __restrict__ ok, const uint32_t* n_dev, const uint64_t* src_dev) {
  if (n_dev) {
    n_reads = *n_dev;
    const uint64_t t = offs[n_reads];
    total = t < total ? t : total;
  }
  if (src_dev && src_dev[0]) {  // the caller's device buffer, read in place (no more than it holds)
    ascii = reinterpret_cast<const uint8_t*>(src_dev[0]);
    total = src_dev[1] < total ? src_dev[1] : total;
  }
  __shared__ uint8_t tab[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tab[i] = table[i];
  __syncthreads();
  // codes mirror the bases byte for byte over [0, total), 16 a thread and round
  const bool aligned = ((reinterpret_cast<uintptr_t>(ascii) | reinterpret_cast<uintptr_t>(codes)) & 15) == 0;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c * 16 < total;
       c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = c * 16;
    uint8_t in[16], out[16];
    const uint64_t m = total - b < 16 ? total - b : 16;
    const bool full = aligned && m == 16;
    if (full) {
      *reinterpret_cast<uint4*>(in) = *reinterpret_cast<const uint4*>(ascii + b);
    } else {
      for (uint64_t i = 0; i < m; ++i) in[i] = ascii[b + i];
    }
    uint32_t bad = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      out[i] = tab[in[i]];
      if (i < (int)m && out[i] == 0xFF) bad |= 1u << i;
    }
    if (full) {
      *reinterpret_cast<uint4*>(codes + b) = *reinterpret_cast<const uint4*>(out);
    } else {
      for (uint64_t i = 0; i < m; ++i) codes[b + i] = out[i];
    }
    while (bad) {
      const int i = __ffs(bad) - 1;
      bad &= bad - 1;
      const uint64_t at = b + i;
      if (at < offs[0]) continue;
      uint32_t lo = 0, hi = n_reads;  // read r with offs[r] <= at < offs[r+1]
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offs[mid] <= at) lo = mid;
        else hi = mid;
      }
      ok[lo] = 0;
    }
  }
}

__device__ __forceinline__ View view_B(uint32_t strand) { return strand ? View{1, 1} : View{0, 0}; }
__device__ __forceinline__ View view_F(uint32_t strand) { return strand ? View{0, 1} : View{1, 0}; }

__device__ __forceinline__ void census_add(unsigned long long* census, uint32_t v) {
  if (census) atomicAdd(census, (unsigned long long)v);
}

// '+' : BWExactSearchBackward over backward; '-' : over forward_rev.
__global__ void __launch_bounds__(kTpb) exact_kernel(DevIndex X, const uint8_t* __restrict__ codes,
                                                     const uint64_t* __restrict__ offs,
                                                     const uint8_t* __restrict__ ok, uint32_t r0, uint32_t nr,
                                                     uint4* __restrict__ slots, uint32_t* __restrict__ rs_count,
                                                     uint8_t* __restrict__ rs_trunc,
                                                     unsigned long long* census) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nr) return;
  const uint32_t read = r0 + (t >> 1), strand = t & 1;
  const uint64_t b = offs[read];
  const int len = (int)(offs[read + 1] - b);
  uint32_t cnt = 0, sectors = 0;
  if (ok[read] && len >= 3 && len <= 32767) {
    uint32_t k = 0, l = X.top;
    if (exact_bwd(X, view_B(strand), codes + b, len - 1, 0, k, l, sectors)) {
      slots[(size_t)t * kSlotCap] = make_uint4(k, l, pack_meta(0, 0, 0, 0, 0), 0);
      cnt = 1;
    }
  }
  rs_count[2ull * r0 + t] = cnt;
  rs_trunc[2ull * r0 + t] = 0;
  census_add(census, sectors);
}

struct PlainEmit {
  uint4* slots;
  OvfEntry* ovf;
  uint32_t* ovf_count;
  uint32_t ovf_cap;
  uint32_t t;
  uint32_t max_results;
  uint32_t cnt;
  bool trunc;
  __device__ __forceinline__ bool operator()(const Cursor& c) {
    if (cnt >= max_results) {
      trunc = true;
      return false;
    }
    const uint32_t meta = c.meta();
    if (cnt < kSlotCap) {
      slots[(size_t)t * kSlotCap + cnt] = make_uint4(c.k, c.l, meta, 0);
    } else {
      const uint32_t pos = atomicAdd(ovf_count, 1u);
      if (pos < ovf_cap) {
        OvfEntry e;
        e.k = c.k;
        e.l = c.l;
        e.meta = meta;
        e.t = t;
        e.idx = cnt;
        e.pad0 = e.pad1 = e.pad2 = 0;
        ovf[pos] = e;
      }
    }
    ++cnt;
    return true;
  }
};

__global__ void __launch_bounds__(kTpb)
    plain_search1_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                         const uint8_t* __restrict__ ok, uint32_t r0, uint32_t nr, uint32_t max_results,
                         uint32_t max_len, uint2* __restrict__ vecs, uint4* __restrict__ slots,
                         OvfEntry* __restrict__ ovf, uint32_t ovf_cap, uint32_t* __restrict__ ovf_count,
                         uint32_t* __restrict__ rs_count, uint8_t* __restrict__ rs_trunc,
                         unsigned long long* census) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t T = 2 * nr;
  if (t >= T) return;
  const uint32_t read = r0 + (t >> 1), strand = t & 1;
  const uint64_t b = offs[read];
  const int len = (int)(offs[read + 1] - b);
  PlainEmit emit{slots, ovf, ovf_count, ovf_cap, t, max_results, 0, false};
  uint32_t sectors = 0;
  if (ok[read] && len >= 3 && (uint32_t)len <= max_len) {
    const uint8_t* W = codes + b;
    const View B = view_B(strand), F = view_F(strand);
    uint2* vB = vecs + t;
    uint2* vF = vecs + (size_t)max_len * T + t;
    vector_bwd(X, B, W, len, vB, T, sectors);
    vector_fwd(X, F, W, len, vF, T, sectors);
    search1_helper(X, W, len, vB, vF, T, B, F, emit, sectors);
  }
  rs_count[2ull * r0 + t] = emit.cnt;
  rs_trunc[2ull * r0 + t] = emit.trunc ? 1 : 0;
  census_add(census, sectors);
}

// ------------------------------------------------------------------ scan --

constexpr int kScanTpb = 512, kScanItems = 8, kScanTile = kScanTpb * kScanItems;

__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t* total) {
  __shared__ uint64_t ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const uint64_t excl = x - v + (warp > 0 ? ws[warp - 1] : 0);
  *total = ws[nw - 1];
  __syncthreads();
  return excl;
}

// The 8 values of a thread's chunk at `base` (zero past n): two 16-byte loads
// when the chunk is whole and aligned.
__device__ __forceinline__ void scan_load8(const uint32_t* __restrict__ in, size_t n, size_t base,
                                           uint32_t (&v)[kScanItems]) {
  if (base + kScanItems <= n && (reinterpret_cast<uintptr_t>(in + base) & 15) == 0) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(in + base));
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(in + base) + 1);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) v[i] = base + i < n ? in[base + i] : 0;
  }
}

__global__ void __launch_bounds__(kScanTpb) scan_reduce_kernel(const uint32_t* __restrict__ in, size_t n,
                                                               uint64_t* __restrict__ part,
                                                               const uint64_t* __restrict__ n_dev) {
  if (n_dev) n = min((uint64_t)n, *n_dev);
  if ((size_t)blockIdx.x * kScanTile > n) return;  // past the count (uniform over the block)
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  scan_load8(in, n, base, v);
  uint64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) s += v[i];
  uint64_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) scan_parts_kernel(uint64_t* part, size_t nb) {
  uint64_t carry = 0;
  for (size_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    const size_t i = b0 + threadIdx.x;
    const uint64_t v = i < nb ? part[i] : 0;
    uint64_t tot;
    const uint64_t ex = block_excl_scan(v, &tot);
    if (i < nb) part[i] = carry + ex;
    carry += tot;
  }
}

// direct: part holds the tiles' sums and each tile adds up those before it
// (few tiles); else part holds the tiles' exclusive prefixes already.
__global__ void __launch_bounds__(kScanTpb) scan_apply_kernel(const uint32_t* __restrict__ in, size_t n,
                                                              const uint64_t* __restrict__ part,
                                                              uint64_t* __restrict__ out, int direct,
                                                              const uint64_t* __restrict__ n_dev) {
  const size_t n_cap = n;
  if (n_dev) n = min((uint64_t)n, *n_dev);
  if ((size_t)blockIdx.x * kScanTile > n) return;  // past the count (uniform over the block)
  uint64_t pre;
  if (direct) {
    uint64_t own = 0;
    for (unsigned t = threadIdx.x; t < blockIdx.x; t += blockDim.x) own += part[t];
    block_excl_scan(own, &pre);
  } else {
    pre = part[blockIdx.x];
  }
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  scan_load8(in, n, base, v);
  uint64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) s += v[i];
  uint64_t tot;
  uint64_t run = pre + block_excl_scan(s, &tot);
  uint64_t o[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    o[i] = run;
    run += v[i];
  }
  if (base + kScanItems <= n && (reinterpret_cast<uintptr_t>(out + base) & 15) == 0) {
    ulonglong2* q = reinterpret_cast<ulonglong2*>(out + base);
#pragma unroll
    for (int i = 0; i < kScanItems / 2; ++i) q[i] = make_ulonglong2(o[2 * i], o[2 * i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
      if (base + i < n) out[base + i] = o[i];
  }
  if (blockIdx.x == n / kScanTile && threadIdx.x == 0) {  // the tile holding position n: the total
    out[n] = pre + tot;
    if (n_cap != n) out[n_cap] = pre + tot;
  }
}

// ---------------------------------------------------------------- gather --

__device__ __forceinline__ hpg_hit_t expand_hit(uint32_t k, uint32_t l, uint32_t meta, uint32_t read,
                                                uint32_t strand) {
  hpg_hit_t h;
  h.read = read;
  h.strand = (uint8_t)strand;
  h.dir = (uint8_t)(meta & 1u);
  h.nm = (uint8_t)((meta >> 1) & 1u);
  h.err_kind = (uint8_t)((meta >> 2) & 3u);
  h.err_base = (uint8_t)((meta >> 4) & 0xFFu);
  h.pad0 = 0;
  h.err_pos = (int16_t)(uint16_t)(meta >> 16);
  h.pad1 = 0;
  h.k = (int64_t)k;
  h.l = (int64_t)l;
  return h;
}

__global__ void gather_slots_kernel(const uint4* __restrict__ slots, const uint32_t* __restrict__ rs_count,
                                    const uint64_t* __restrict__ off, uint32_t r0, uint32_t nr,
                                    hpg_hit_t* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nr) return;
  const uint32_t c = rs_count[2ull * r0 + t];
  const uint32_t m = c < kSlotCap ? c : kSlotCap;
  const uint64_t o = off[t];
  for (uint32_t i = 0; i < m; ++i) {
    const uint4 s = slots[(size_t)t * kSlotCap + i];
    out[o + i] = expand_hit(s.x, s.y, s.z, r0 + (t >> 1), t & 1);
  }
}

__global__ void gather_ovf_kernel(const OvfEntry* __restrict__ ovf, const uint32_t* __restrict__ ovf_count,
                                  uint32_t ovf_cap, const uint32_t* __restrict__ rs_count,
                                  const uint64_t* __restrict__ off, uint32_t r0, hpg_hit_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = min(*ovf_count, ovf_cap);
  if (i >= n) return;
  const OvfEntry e = ovf[i];
  if (e.idx < rs_count[2ull * r0 + e.t]) out[off[e.t] + e.idx] = expand_hit(e.k, e.l, e.meta, r0 + (e.t >> 1), e.t & 1);
}

__global__ void hit_rows_kernel(const hpg_hit_t* __restrict__ hits, uint32_t n, uint32_t* __restrict__ rows) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t k = hits[i].k, l = hits[i].l;
  rows[i] = k <= l ? (uint32_t)(l - k + 1) : 0u;
}

__global__ void limit_rows_kernel(const uint64_t* __restrict__ list_off, uint32_t* __restrict__ rows,
                                  uint32_t n_lists, uint64_t limit, const uint64_t* limit_dev,
                                  uint8_t* __restrict__ trunc, const unsigned* gate) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_lists) return;
  if (gate && *gate) return;
  if (limit_dev) limit = *limit_dev;
  if (limit == 0) return;
  const uint64_t b = list_off[t], e = list_off[t + 1];
  uint64_t sum = 0;
  for (uint64_t h = b; h < e; ++h) sum += rows[h];
  if (sum <= limit) return;
  for (uint64_t h = b; h < e; ++h) rows[h] = 0;
  trunc[t] |= 2;
}

// ---------------------------------------------------------------- locate --

__global__ void __launch_bounds__(kTpb)
    locate_kernel(DevIndex X, const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ loc_off,
                  uint32_t n_hits, uint64_t n_locs, const uint64_t* __restrict__ read_offs, uint32_t hit_base,
                  hpg_loc_t* __restrict__ out, unsigned long long* census) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_locs) return;
  // owning hit: last h with loc_off[h] <= r
  uint32_t lo = 0, hi = n_hits;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (loc_off[mid] <= r) lo = mid;
    else hi = mid;
  }
  const hpg_hit_t h = hits[lo];
  const uint32_t row = (uint32_t)((uint64_t)h.k + (r - loc_off[lo]));
  const uint64_t len = read_offs[h.read + 1] - read_offs[h.read];
  uint64_t len_calc = len;
  const uint32_t err = h.nm ? h.err_kind : 0u;
  if (err == 1) len_calc--;
  else if (err == 3) len_calc++;
  // direction = type ? dir : !dir, with type = !strand: rows of the forward SA when set
  const uint32_t phys_fw = (uint32_t)h.dir ^ (uint32_t)h.strand;
  uint32_t steps = 0;
  uint64_t key;
  {
    const uint32_t sa = sa_value(X, dir_of(X, phys_fw), row, &steps);
    key = phys_fw ? (uint64_t)((X.top + 1u) - sa) - len_calc - 1u : (uint64_t)sa;
  }
  const uint32_t id = kar_search(X, key);
  hpg_loc_t o;
  o.key = key;
  o.hit = hit_base + lo;
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
  out[r] = o;
  census_add(census, steps);
}

}  // namespace

void launch_encode(const uint8_t* ascii, uint64_t total, const uint64_t* offs, uint32_t n_reads,
                   const uint8_t* d_table, uint8_t* codes, uint8_t* ok, cudaStream_t s) {
  if (!n_reads) return;
  cudaMemsetAsync(ok, 1, n_reads, s);
  if (!total) return;
  const uint64_t chunks = (total + 15) / 16;
  const unsigned grid = (unsigned)(chunks < 152ull * 32 * 8 ? (chunks + 255) / 256 : 152ull * 32);
  count_launches(1);
  encode_kernel<<<grid, 256, 0, s>>>(ascii, total, offs, n_reads, d_table, codes, ok, nullptr, nullptr);
}

namespace {

// Graph form: read offsets checked on the device (non-decreasing, reads at
// most 32767 bases, inside the staged bases).  A bad read is switched off so
// no kernel reads past its buffers, and the status word reports the batch.
__global__ void check_offsets_kernel(const uint64_t* __restrict__ offs, const uint32_t* __restrict__ n_dev,
                                     uint64_t bases_cap, uint8_t* __restrict__ ok, unsigned* status) {
  const uint32_t n = *n_dev;
  const uint64_t end = offs[n];
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint64_t b0 = offs[r], b1 = offs[r + 1];
    if (b1 < b0 || b1 - b0 > 32767 || b1 > end || end > bases_cap) {
      ok[r] = 0;
      atomicOr(status, 8u);
    }
  }
}

}  // namespace

void launch_check_offsets(const uint64_t* offs, const uint32_t* n_dev, uint32_t n_cap, uint64_t bases_cap,
                          uint8_t* ok, unsigned* status, cudaStream_t s) {
  const unsigned grid = (unsigned)std::min<uint64_t>((n_cap + 255) / 256, 152ull * 8);
  count_launches(1);
  check_offsets_kernel<<<grid ? grid : 1, 256, 0, s>>>(offs, n_dev, bases_cap, ok, status);
}

void launch_encode_dev(const uint8_t* ascii, uint64_t bases_cap, const uint64_t* offs, const uint32_t* n_dev,
                       uint32_t n_cap, const uint8_t* d_table, uint8_t* codes, uint8_t* ok, cudaStream_t s,
                       const uint64_t* src_dev) {
  cudaMemsetAsync(ok, 1, n_cap, s);
  const uint64_t chunks = (bases_cap + 15) / 16;
  const unsigned grid = (unsigned)(chunks < 152ull * 32 * 8 ? (chunks + 255) / 256 : 152ull * 32);
  count_launches(1);
  encode_kernel<<<grid ? grid : 1, 256, 0, s>>>(ascii, bases_cap, offs, 0, d_table, codes, ok, n_dev, src_dev);
}

void launch_exact(const DevIndex& X, const uint8_t* codes, const uint64_t* offs, const uint8_t* ok, uint32_t r0,
                  uint32_t nr, uint4* slots, uint32_t* rs_count, uint8_t* rs_trunc,
                  unsigned long long* census, cudaStream_t s) {
  if (!nr) return;
  count_launches(1);
  exact_kernel<<<grid_for(2ull * nr, kTpb), kTpb, 0, s>>>(X, codes, offs, ok, r0, nr, slots, rs_count, rs_trunc,
                                                           census);
}

void launch_plain_search1(const DevIndex& X, const uint8_t* codes, const uint64_t* offs, const uint8_t* ok,
                          uint32_t r0, uint32_t nr, uint32_t max_results, uint32_t max_len, uint2* vecs,
                          uint4* slots, OvfEntry* ovf, uint32_t ovf_cap, uint32_t* ovf_count,
                          uint32_t* rs_count, uint8_t* rs_trunc, unsigned long long* census, cudaStream_t s) {
  if (!nr) return;
  count_launches(1);
  plain_search1_kernel<<<grid_for(2ull * nr, kTpb), kTpb, 0, s>>>(X, codes, offs, ok, r0, nr, max_results, max_len,
                                                                   vecs, slots, ovf, ovf_cap, ovf_count, rs_count,
                                                                   rs_trunc, census);
}

size_t scan_parts(size_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

void launch_scan(const uint32_t* in, size_t n, uint64_t* out, uint64_t* part, cudaStream_t s,
                 const uint64_t* n_dev) {
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(uint64_t), s);
    return;
  }
  // tiles, plus one that only holds position n when n ends a tile
  const unsigned nb = (unsigned)(n / kScanTile + 1);
  // up to 4096 tiles, each tile of the apply pass sums the tile sums before it
  // (at most 8 loads a thread); more, and one block scans the tile sums first
  const int direct = nb <= 4096;
  count_launches(1);
  scan_reduce_kernel<<<nb, kScanTpb, 0, s>>>(in, n, part, n_dev);
  if (!direct) {
    count_launches(1);
    scan_parts_kernel<<<1, 1024, 0, s>>>(part, nb);
  }
  count_launches(1);
  scan_apply_kernel<<<nb, kScanTpb, 0, s>>>(in, n, part, out, direct, n_dev);
}

void launch_gather_hits(const uint4* slots, const OvfEntry* ovf, const uint32_t* ovf_count, uint32_t ovf_cap,
                        const uint32_t* rs_count, const uint64_t* off, uint32_t r0, uint32_t nr,
                        hpg_hit_t* out, cudaStream_t s) {
  if (!nr) return;
  count_launches(1);
  gather_slots_kernel<<<grid_for(2ull * nr, 256), 256, 0, s>>>(slots, rs_count, off, r0, nr, out);
  if (ovf && ovf_cap) {
    count_launches(1);
    gather_ovf_kernel<<<grid_for(ovf_cap, 256), 256, 0, s>>>(ovf, ovf_count, ovf_cap, rs_count, off, r0, out);
  }
}

void launch_hit_rows(const hpg_hit_t* hits, uint32_t n_hits, uint32_t* rows, cudaStream_t s) {
  if (!n_hits) return;
  count_launches(1);
  hit_rows_kernel<<<grid_for(n_hits, 256), 256, 0, s>>>(hits, n_hits, rows);
}

void launch_limit_rows(const uint64_t* list_off, uint32_t* rows, uint32_t n_lists, uint64_t limit,
                       const uint64_t* limit_dev, uint8_t* trunc, cudaStream_t s, const unsigned* gate) {
  if (!n_lists || (!limit_dev && limit == 0)) return;
  count_launches(1);
  limit_rows_kernel<<<grid_for(n_lists, 256), 256, 0, s>>>(list_off, rows, n_lists, limit, limit_dev, trunc, gate);
}

void launch_locate(const DevIndex& X, const hpg_hit_t* hits, const uint64_t* loc_off, uint32_t n_hits,
                   uint64_t n_locs, const uint64_t* read_offs, uint32_t hit_base, hpg_loc_t* out,
                   unsigned long long* census, cudaStream_t s) {
  if (!n_locs) return;
  count_launches(1);
  locate_kernel<<<grid_for(n_locs, kTpb), kTpb, 0, s>>>(X, hits, loc_off, n_hits, n_locs, read_offs, hit_base, out,
                                                        census);
}

}  // namespace hpgbwt
