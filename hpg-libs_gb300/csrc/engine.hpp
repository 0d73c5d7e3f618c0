// engine.hpp -- one GPU context per loaded index: the HBM-resident index, a
// CUDA stream, a grow-only device workspace and the mapping pipeline.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "hpg_bwt_records.h"
#include "index_format.hpp"

namespace hpgbwt {

// Pipeline forms.
enum Form : int {
  kFormPlain = 0,    // one thread per (read, strand), one launch per stage
  kFormBatched = 1,  // persistent work-queue kernel replayed from a CUDA graph
};

// Device-resident output of one search call; valid until the next call.
struct DeviceResult {
  size_t n_reads = 0;
  size_t n_hits = 0;
  const hpg_hit_t* hits = nullptr;
  size_t n_locs = 0;
  const hpg_loc_t* locs = nullptr;
  const uint32_t* rs_count = nullptr;
  const uint8_t* rs_truncated = nullptr;
};

// Per-stage device times of the last call (ms), measured with CUDA events on
// the engine's stream.
enum Stage : int { kStageEncode = 0, kStageSearch, kStageFinalize, kStageLocate, kStageCount };

struct Engine;

Engine* engine_create(const HostIndex& h, int device, std::string* err);
void engine_destroy(Engine* e);
void* engine_stream(Engine* e);
int engine_device(Engine* e);

// Reads already in device memory: ASCII bytes and n_reads+1 offsets.
int engine_search_device(Engine* e, int mode, int form, const uint8_t* d_seqs, const uint64_t* d_offs, size_t n_reads,
                         uint64_t total_bases, uint32_t max_len, uint32_t max_results, DeviceResult* out,
                         std::string* err);

// Host reads in, results left on the device as engine_search_device leaves them.
int engine_search_host_keep(Engine* e, int mode, int form, const char* seqs, const uint64_t* offs, size_t n_reads,
                            uint32_t max_results, DeviceResult* out, std::string* err);

// Host reads in, host records out (malloc'ed; free with hpg_result_free).
int engine_search_host(Engine* e, int mode, int form, const char* seqs, const uint64_t* offs, size_t n_reads,
                       uint32_t max_results, hpg_result_set_t* out, std::string* err);

// Copy the last device result into caller buffers (any host memory).
int engine_copy_result(Engine* e, const DeviceResult& r, hpg_hit_t* hits, hpg_loc_t* locs, uint32_t* rs_count,
                       uint8_t* rs_truncated, std::string* err);

void engine_stage_ms(Engine* e, float* out, int n);
void engine_set_census(Engine* e, int on);
unsigned long long engine_census(Engine* e);
void engine_set_chunk(Engine* e, size_t reads_per_chunk);
size_t engine_index_bytes(Engine* e);
// Batched-form tuning (threads per block is fixed at 128): blocks per SM
// (0 = occupancy limit), change points per lane kept in shared memory, chains
// claimed per refill.
void engine_set_tuning(Engine* e, int min_blocks, int blocks_per_sm, int stack, int chunk);
void engine_get_tuning(Engine* e, int* out5);
void engine_set_load_mode(Engine* e, int mode);
// Fused form, index direction of the chains: 0 any lane any chain; 1 SMs of the
// first half the backward-index chains, the rest the forward-index ones; 2 one
// launch per direction.
void engine_set_dir_split(Engine* e, int mode);
int engine_dir_split(Engine* e);
void engine_set_wave_group(Engine* e, int reads);
int engine_wave_group(Engine* e);
void engine_set_idle_batch(Engine* e, int lanes);
int engine_idle_batch(Engine* e);
void engine_set_locate_limit(Engine* e, uint64_t max_rows);
uint64_t engine_locate_limit(Engine* e);
// Batched form from the captured CUDA graph (1, the default) or launched
// stage by stage with host-read sizes (0).
void engine_set_graph(Engine* e, int on);
// Start table of the batched search: chains of reads of 2L+2 or more bases
// begin with one lookup instead of their first L steps (0 = no table).
constexpr int kDefaultKmer = 0;
int engine_set_kmer(Engine* e, int L, std::string* err);
int engine_kmer(Engine* e);
// Host-buffer batches of at least two chunks run pipelined; reads per chunk (0 automatic, SIZE_MAX off).
void engine_set_pipeline_chunk(Engine* e, size_t reads);
int engine_graph(Engine* e);
int engine_load_mode(Engine* e);
int engine_autotune(Engine* e, const uint8_t* d_seqs, const uint64_t* d_offs, size_t n_reads, uint64_t total_bases,
                    uint32_t max_len, uint32_t max_results, int* table, int max_rows, int* rows_out,
                    std::string* err);

// ---- device passes of the alignment-list layer (map_device.cu) ----
// Host reads in (ASCII + n+1 offsets).  kl gets per read {k+, l+, k-, l-}:
// the '+' backward search over backward and the '-' forward search over
// forward_rev of bwt_map_exact_seq, where each stopped (k = l + 1 if a base failed).
int engine_exact_api(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t* kl, std::string* err);
// For the listed reads: per chain {good steps, k, l, 0} of the four vector searches.
int engine_anchor_scan(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* reads, size_t m,
                       uint32_t* out, std::string* err);
// One lock for the reference-style entry points (alignment lists, seeds,
// CALs): the engine's stream and workspace serve one call at a time.
std::mutex& map_api_mutex();

struct MapRow {
  uint32_t row, phys, len_calc;  // SA row, physical index direction (0 backward, 1 forward), located length
  uint32_t key32 = 0;  // 1: the forward key in 32-bit arithmetic, as the anchor lists (bwt.c:1853-1855)
};
// Seeds: per seed {read, first, last (included), 0}; out per seed {k, l} of the
// '+' search and {k, l} of the '-' search (k = 1, l = 0 for seeds outside
// their read or reads outside the alphabet).
int engine_seed_search(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* seeds, size_t m,
                       uint32_t* out, std::string* err);
int engine_locate_rows(Engine* e, const MapRow* rows, size_t m, hpg_loc_t* out, std::string* err);

// bwt_map_inexact_read's alignments for a batch of reads (5+ bases each),
// decided on the device: BWSearch1 with lists of capacity filter_read_mappings,
// the row filter over both strands, the located rows, the 10 bp merge and the
// list order (bwt.c:1978-2237).  Read i's records are rec[rec_off[i] ..
// rec_off[i] + n_rec[i]): {chromosome | strand << 31, position}; flags[i] bit 0:
// flag 2 (a strand passed the filter), bit 1: the list's first alignment loses
// its secondary mark (bwt.c:2234-2237), bit 2: more rows than a 32-bit count.
struct MapRec {
  uint32_t chrom_strand;  // chromosome | strand << 31
  int32_t position;
};
struct InexactRecords {
  std::vector<uint32_t> n_rec;
  std::vector<uint8_t> flags;
  std::vector<uint64_t> rec_off;
  std::vector<MapRec> rec;
};
int engine_inexact_records(Engine* e, const char* seqs, const uint64_t* offs, size_t n, int filter_read_mappings,
                           InexactRecords* out, std::string* err);
// Wall time of the last alignment-list call's device pass (search to records), seconds.
void engine_note_map_device_seconds(Engine* e, double s);
double engine_map_device_seconds(Engine* e);

// The k-error block search of bwt_map_inexact_read_2 (block_search.cu): per
// (read, strand) t = 2 * read + strand, count[t] results (hits of item t are
// contiguous, items in order), refused[t] = 1 when a list of the search was
// full, anchors[2 * t + a] for a < n_anchors[t].  Reads outside the alphabet
// or outside 3..32767 bases get nothing.
struct BlockSearchOut {
  std::vector<hpg_hit_t> hits;
  std::vector<uint32_t> count;
  std::vector<uint8_t> refused;
  std::vector<hpg_block_anchor_t> anchors;
  std::vector<uint8_t> n_anchors;
  float kernel_ms = 0;  // device time of the search kernel(s)
};
int engine_block_search(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t max_results,
                        BlockSearchOut* out, std::string* err);
// The same search with every row of every hit located on the device (the
// locate limit applies), as a result set in pooled host arrays; anchors and
// n_anchors (4 n and 2 n entries) may be null.
int engine_block_search_result(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t max_results,
                               hpg_result_set_t* out, hpg_block_anchor_t* anchors, uint8_t* n_anchors,
                               std::string* err);
float engine_block_ms(Engine* e);  // device time of the last block search's kernels
// Batched form: hits only, no located rows.
void engine_set_skip_locate(Engine* e, int on);
uint32_t engine_sa_top(Engine* e);  // last SA row (n)

}  // namespace hpgbwt
