// batched.cuh -- the batched (persistent, work-queue) form of the mapping pipeline.
//
// Search: one persistent kernel whose lanes each run a small state machine
// that issues exactly one backward-extension step per loop iteration, so the
// lanes of a warp stay converged on the gather regardless of what each lane
// is doing (a vector search, a branch continuation, a j=1 block).  Work comes
// from a global chain counter (4 chains per read: 2 strands x 2 halves) and
// from each lane's own stack of change points; a change point that does not
// fit on the stack spills to a device queue that a drain launch empties.
// Every hit carries an order key that reproduces BWSearch1VectorHelper's
// emission order (search/search.c:1491-1709); the finalize kernels sort each
// (read, strand) list by key and truncate it at max_results like add_result
// (search/results.h:93-103).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fm_device.cuh"
#include "hpg_bwt_records.h"

namespace hpgbwt {

// One emitted hit before ordering.
struct PendingHit {
  uint32_t rs;    // 2 * read + strand
  uint32_t key;   // emission order within the (read, strand) list
  uint32_t k, l;
  uint32_t meta;  // packed as pack_meta()
  uint32_t idx;   // unused (list positions are assigned by the scatter kernel)
};

// A spilled change point.
struct SpillEntry {
  uint32_t k, l;
  uint32_t rs;
  uint32_t jtype;  // J | type << 16
};

struct BatchedParams {
  // inputs
  const uint8_t* codes;
  const uint64_t* offs;
  const uint8_t* ok;
  uint32_t n_reads;
  const uint32_t* n_reads_dev;  // when set, the read count is read from device memory (graph replays)
  uint32_t max_results;
  // work queues
  unsigned int* chain_ctr;   // next chain id (next read in the fused form)
  unsigned int* chain_ctr2;  // fused form with direction split: next read for the forward-index chains
  uint32_t dir_split;        // fused form: 1 = SMs of the first half run the chains on the backward index,
                             // the others those on the forward index (each half then takes the rest);
                             // 2 / 3 = this launch runs only the backward / forward-index chains
  uint32_t num_sms;
  uint32_t batch_idle;       // fused form: lanes out of work wait until this many lanes of the
                             // converged group are (or all of them are), then move on together
  unsigned int* spill_head;  // next spill entry to drain
  unsigned int* spill_tail;  // spill entries written
  SpillEntry* spill;
  uint32_t spill_cap;
  // results
  unsigned int* res_total;
  PendingHit* res;
  uint32_t res_cap;
  uint32_t* rs_count;        // [2 * n_reads] arrivals per (read, strand)
  unsigned int* status;      // bit 0: result pool full, bit 1: spill queue full
  unsigned long long* census;
  // warp-cooperative form (wave.cu): reads claimed per warp group; reads too long for a
  // group buffer are appended to long_list (long_n of them, long_cap at most) for the
  // fused kernel; j = 1 / j = n-1 blocks go to `blocks` (block_n, block_cap) for the
  // fused drain
  uint32_t wave_group = 32;
  uint64_t codes_len = 0;  // bytes of `codes` that may be read (its allocation)
  uint32_t* long_list = nullptr;
  unsigned int* long_n = nullptr;
  uint32_t long_cap = 0;
  SpillEntry* blocks = nullptr;
  unsigned int* block_n = nullptr;
  uint32_t block_cap = 0;
  // fused form: when set, claim i runs read read_list[i], for i < *read_list_n
  const uint32_t* read_list = nullptr;
  const unsigned int* read_list_n = nullptr;
};

struct BatchedTuning {
  int block = 128;        // threads per block
  int blocks_per_sm = 0;  // 0: as many as fit
  int stack = 4;          // change points per lane kept in shared memory (2, 4 or 8)
  int chunk = 1;          // chains claimed per lane per refill (1, 2 or 4)
  int min_blocks = 1;     // register bound: 1 (compiler's choice), 12 or 16 resident blocks per SM
  int split = 0;          // 0: fused (per-lane stacks); 1: chain-only kernel + drain of every change point;
                          // 2: lockstep kernel (4 chains of a read per lane) + drain;
                          // 3: warp-cooperative kernels (wave.cu) + the fused kernel over their long reads and blocks
  int phase = 2;          // set by the engine for split launches: 0/1 one index direction, 2 both
  int dir_split = 0;      // fused form: 0 mixed, 1 direction by SM half, 2 one launch per direction
  int batch_idle = 8;     // fused form: idle lanes that move to their next work item together (1: each at once)
  int group = 32;         // warp-cooperative form (split 3): reads a warp claims at a time (32 / group lanes per read)
};

// One locate work item per SA row: the row, the owning hit (or request), the
// output index, and the physical direction with len_calc (bwt.c:2025-2036), so
// that a lane starting a walk needs a single 16-byte load.
struct RowItem {
  uint32_t row, hit, out, phys_len;  // phys_len: direction << 31 | kRowKey32 flag | len_calc
};
// The forward-direction key size_SA - SA - len_calc - 1 taken in 32 bits: the
// reference's anchor lists (bwt.c:1853-1855) subtract an int length from
// SA_TYPE (uint32_t) values, so a row whose suffix is shorter than the length
// wraps to a large 32-bit key (an invalid location), not a 64-bit one.
constexpr uint32_t kRowKey32 = 1u << 30;
constexpr uint32_t kRowLenMask = kRowKey32 - 1u;

// Located rows of one batched call: row items carry 32-bit output indices and
// rows are claimed through a 32-bit counter that may run a few claims past the
// end, so a batch stays well below 2^32 rows (the plain form has no such limit).
constexpr uint64_t kMaxLocateRows = 0xF0000000ull;

constexpr unsigned kStatusResFull = 1u, kStatusSpillFull = 2u, kStatusLocFull = 4u, kStatusBadInput = 8u;
// warp-cooperative search: a warp found live work counted for a group buffer that nothing
// held (an internal inconsistency; the batch is failed rather than trusted)
constexpr unsigned kStatusWaveAcct = 32u;
// Reads longer than this many bases may not fit a warp group buffer of the
// warp-cooperative form; a batch holds at most total_bases / kWaveLongMin + 1 such reads.
constexpr uint64_t kWaveLongMin = 4000;

// Locate sizes of the graph form: with `status` set, the hit and row counts
// are read from device memory, rows beyond `locs_cap` raise kStatusLocFull,
// and a nonzero status skips the stage.
struct LocateSizes {
  unsigned* status = nullptr;
  const uint64_t* n_hits = nullptr;
  const uint64_t* n_locs = nullptr;
  uint64_t locs_cap = 0;
};

// Search kernels: `drain` empties the spill queue instead of pulling chains.
void launch_batched_search(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms, bool drain,
                           cudaStream_t s);
int batched_max_blocks_per_sm(const BatchedTuning& t);
// The warp-cooperative search (wave.cu), one launch: p.dir_split 2 / 3 runs the
// backward- / forward-index chains, anything else all four chains of a read.
void launch_wave_search(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms,
                        cudaStream_t s);
int wave_max_blocks_per_sm(const BatchedTuning& t);
// The helper's branches of the change points queued in p.spill (from
// p.spill_head on), eight continuations per change point; j = 1 / j = n-1 block
// entries are copied to `blocks` (count in *block_n) for the fused drain.
void launch_wave_branches(const DevIndex& X, const BatchedParams& p, SpillEntry* blocks, unsigned int* block_n,
                          uint32_t block_cap, int num_sms, cudaStream_t s);
// The whole search stage of a tuning: the search launches, then (after `mid`,
// recorded when not null) the drain of queued change points.  `ctr` is the
// counter block (16 words, zeroed); the warp-cooperative form also needs
// `long_list` (room for its long reads) and `blocks` (room for the j = 1 /
// j = n-1 blocks among the change points, as many as the queue holds).
void launch_search_stage(const DevIndex& X, const BatchedParams& p, const BatchedTuning& t, int num_sms,
                         unsigned int* ctr, uint32_t* long_list, uint32_t long_cap, SpillEntry* blocks,
                         uint32_t block_cap, cudaEvent_t mid, bool external, cudaStream_t s);

// Finalize: scatter pending hits into (read, strand) segments, sort each by
// key, truncate; kept counts to `kept`, truncation flags to `trunc`.
// In the graph form `gate` (the search status word) skips the stage after a
// pool overflow and `max_dev` holds max_results.
void launch_scatter_hits(const PendingHit* res, const unsigned int* res_total, const uint64_t* seg_off,
                         PendingHit* sorted, uint32_t res_cap, uint32_t* cursor, cudaStream_t s,
                         const unsigned* gate = nullptr);
// Sorts every (read, strand) list by emission key and keeps the first max_results
// (from max_dev when given); `scratch` holds at least as many entries as
// `sorted` and its contents are overwritten (the scatter's input is dead by then).
// With `longs` (longs_cap = long_lists_cap(entries of the pool) entries) and a
// zeroed counter `n_longs`, the lists above kLongList entries are collected by
// the short sort and the long sort visits only them; without, it scans every list.
void launch_sort_truncate(PendingHit* sorted, PendingHit* scratch, const uint64_t* seg_off, uint32_t n_rs,
                          uint32_t max_results, uint32_t* kept, uint8_t* trunc, int num_sms, cudaStream_t s,
                          const uint32_t* max_dev = nullptr, const unsigned* gate = nullptr, uint32_t* longs = nullptr,
                          unsigned* n_longs = nullptr, uint32_t longs_cap = 0);
// Room for the ids of the lists longer than kLongList entries among res_cap entries.
size_t long_lists_cap(size_t res_cap);
// With the long-list work list of launch_sort_truncate, those lists' records are
// written a block per list.
void launch_expand_hits(const PendingHit* sorted, const uint64_t* seg_off, const uint64_t* hit_off,
                        const uint32_t* kept, uint32_t n_rs, hpg_hit_t* hits, uint32_t* rows, cudaStream_t s,
                        const unsigned* gate = nullptr, const uint32_t* longs = nullptr,
                        const unsigned* n_longs = nullptr, uint32_t longs_cap = 0, int num_sms = 152);

// Persistent locate: lanes pull rows from a counter and refill when their walk
// ends.  In the graph form n_hits / n_locs are capacities and `z` the sizes.
void launch_locate_persistent(const DevIndex& X, const hpg_hit_t* hits, const uint64_t* loc_off, uint32_t n_hits,
                              uint64_t n_locs, const uint64_t* read_offs, hpg_loc_t* out, void* row_items,
                              unsigned int* row_ctr, unsigned long long* census, int num_sms, cudaStream_t s,
                              const LocateSizes& z = LocateSizes());
size_t locate_row_item_bytes();
// Start table of physical direction d for strings of L symbols (4^L entries).
void launch_build_kmer(const DevIndex& X, uint32_t d, uint32_t L, uint2* out, cudaStream_t s);
// Locate caller-built rows (device array of n_items RowItem); out[item.out] per row.
void launch_locate_items(const DevIndex& X, const RowItem* items, uint64_t n_items, hpg_loc_t* out,
                         unsigned int* row_ctr, int num_sms, cudaStream_t s);

}  // namespace hpgbwt
