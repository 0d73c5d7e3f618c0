// kernels.cuh -- launch wrappers of the search pipeline kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "fm_device.cuh"
#include "hpg_bwt_records.h"

namespace hpgbwt {

// Hit slot written by the search kernels: {k, l, packed meta, 0}.
// Overflow entries carry the owning (read, strand) slot id and list index.
struct OvfEntry {
  uint32_t k, l, meta, t, idx, pad0, pad1, pad2;
};

constexpr uint32_t kSlotCap = 8;  // hits kept in place per (read, strand); the rest overflow

// Kernels launched by this library since load (the benchmark's launch count).
unsigned long long launch_count();
void count_launches(unsigned n);
void uncount_launches(unsigned long long n);  // launches recorded while capturing a graph

// ASCII -> 2-bit codes (0xFF outside the alphabet) and a per-read validity flag.
void launch_encode(const uint8_t* ascii, uint64_t total, const uint64_t* offs, uint32_t n_reads,
                   const uint8_t* d_table, uint8_t* codes, uint8_t* ok, cudaStream_t s);

// Graph form of launch_encode: n_reads read from device memory, byte count
// offs[n] (at most bases_cap), flags cleared over n_cap reads.  src_dev (device
// memory: source pointer, source bytes) names where the bases are when its
// pointer is not 0 (a caller's device buffer, read in place), else `ascii`.
void launch_encode_dev(const uint8_t* ascii, uint64_t bases_cap, const uint64_t* offs, const uint32_t* n_dev,
                       uint32_t n_cap, const uint8_t* d_table, uint8_t* codes, uint8_t* ok, cudaStream_t s,
                       const uint64_t* src_dev = nullptr);

// Graph form: reads whose offsets are decreasing, longer than 32767 bases or
// past the staged bases get ok = 0 and set bit 8 of *status.
void launch_check_offsets(const uint64_t* offs, const uint32_t* n_dev, uint32_t n_cap, uint64_t bases_cap,
                          uint8_t* ok, unsigned* status, cudaStream_t s);

// Exact backward search on both strands (mode EXACT), one thread per (read, strand).
void launch_exact(const DevIndex& X, const uint8_t* codes, const uint64_t* offs, const uint8_t* ok, uint32_t r0,
                  uint32_t nr, uint4* slots, uint32_t* rs_count, uint8_t* rs_trunc,
                  unsigned long long* census, cudaStream_t s);

// Plain BWSearch1: one thread per (read, strand) runs the two vector searches
// into `vecs` and then the helper with its continuation searches.
void launch_plain_search1(const DevIndex& X, const uint8_t* codes, const uint64_t* offs, const uint8_t* ok,
                          uint32_t r0, uint32_t nr, uint32_t max_results, uint32_t max_len, uint2* vecs,
                          uint4* slots, OvfEntry* ovf, uint32_t ovf_cap, uint32_t* ovf_count,
                          uint32_t* rs_count, uint8_t* rs_trunc, unsigned long long* census, cudaStream_t s);

// Exclusive scan: out[0..n] with out[n] = total.  `part` needs scan_parts(n) entries.
// With n_dev the scan covers the first min(n, *n_dev) entries (a count found on
// the device) and writes the total at that position and at out[n].
size_t scan_parts(size_t n);
void launch_scan(const uint32_t* in, size_t n, uint64_t* out, uint64_t* part, cudaStream_t s,
                 const uint64_t* n_dev = nullptr);

// Slots + overflow pool -> ordered hpg_hit_t records, hit i of (read, strand) t at off[t] + i.
void launch_gather_hits(const uint4* slots, const OvfEntry* ovf, const uint32_t* ovf_count, uint32_t ovf_cap,
                        const uint32_t* rs_count, const uint64_t* off, uint32_t r0, uint32_t nr,
                        hpg_hit_t* out, cudaStream_t s);

// Rows per hit (l - k + 1 or 0).
void launch_hit_rows(const hpg_hit_t* hits, uint32_t n_hits, uint32_t* rows, cudaStream_t s);

// Locate limit: a list (read, strand) whose hits list_off[t]..list_off[t+1]
// cover more than `limit` rows (read from limit_dev when given; 0 = no limit)
// has its rows set to 0, so nothing of it is located, and trunc[t] |= 2.
void launch_limit_rows(const uint64_t* list_off, uint32_t* rows, uint32_t n_lists, uint64_t limit,
                       const uint64_t* limit_dev, uint8_t* trunc, cudaStream_t s, const unsigned* gate = nullptr);

// Locate every row of every hit (bwt.c:2158-2166); hit ids are offset by hit_base.
void launch_locate(const DevIndex& X, const hpg_hit_t* hits, const uint64_t* loc_off, uint32_t n_hits,
                   uint64_t n_locs, const uint64_t* read_offs, uint32_t hit_base, hpg_loc_t* out,
                   unsigned long long* census, cudaStream_t s);

}  // namespace hpgbwt
