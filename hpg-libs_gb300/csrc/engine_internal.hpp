// engine_internal.hpp -- the Engine context shared by the pipeline
// orchestration (engine.cu), the CUDA-graph form (graph.cu) and the request
// loop (serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "batched.cuh"
#include "engine.hpp"
#include "fm_device.cuh"
#include "kernels.cuh"

namespace hpgbwt {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

#define HPG_CUDA(call, msg)                                                        \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      if (err) *err = std::string(msg) + ": " + cudaGetErrorString(_e);            \
      return -1;                                                                   \
    }                                                                              \
  } while (0)

// The batched pipeline captured for one capacity class (graph.cu).
struct GraphPlan {
  // capacity class and the settings baked into the capture
  uint32_t n_cap = 0;
  uint64_t bases_cap = 0;
  uint32_t res_cap = 0, spill_cap = 0;
  uint64_t locs_cap = 0;
  BatchedTuning tuning;
  uint32_t load_mode = 0;
  bool census = false;
  bool skip_locate = false;  // hits only (the alignment-list layer locates the rows it needs)
  uint32_t kmer_len = 0;     // start table captured with the kernels (length and address)
  const void* kmer0 = nullptr;
  // device buffers
  uint8_t* seqs = nullptr;
  uint64_t* offs = nullptr;
  uint32_t* hdr = nullptr;  // [0] reads in this batch, [1] max_results, [2..3] locate limit (u64),
                            // [4..5] source of the bases (u64, 0 = seqs), [6..7] its bytes
  uint8_t* codes = nullptr;
  uint8_t* ok = nullptr;
  unsigned* ctr = nullptr;  // as the direct form: [0] chains [1] spill head [2] spill tail [3] results [4] status
                            // [5..7] locate [8] phase-1 chains [9] forward-index reads [10] long reads
                            // [11] long-read claims [12] block head [13] block tail [14] long lists
  uint32_t* arr = nullptr;  // arrivals per (read, strand)
  uint64_t* seg = nullptr;
  uint64_t* hit_off = nullptr;
  uint32_t* kept = nullptr;
  uint8_t* trunc = nullptr;
  uint64_t* part = nullptr;
  PendingHit* res = nullptr;
  PendingHit* sorted = nullptr;
  SpillEntry* spill = nullptr;
  hpg_hit_t* hits = nullptr;
  uint32_t* rows = nullptr;
  uint64_t* loc_off = nullptr;
  void* items = nullptr;
  hpg_loc_t* locs = nullptr;
  unsigned long long* census_d = nullptr;
  uint64_t* summary_d = nullptr;
  uint32_t* long_list = nullptr;  // reads too long for the warp-cooperative form's group buffers
  uint32_t* longs = nullptr;  // lists above kLongList entries, found by the sort (ctr[14] counts them)
  uint32_t long_cap = 0;
  SpillEntry* blocks = nullptr;   // j = 1 / j = n-1 blocks of the warp-cooperative form (spill_cap entries)
  // pinned host words
  uint64_t* h_summary = nullptr;  // [0] status | results << 32, [1] spill tail, [2] hits, [3] rows, [4] census
  uint32_t* h_hdr = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long kernels = 0;  // kernel nodes per replay
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<void*> allocs;
  uint64_t bytes = 0;  // device bytes held
};


struct Engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevIndex X{};
  OccBlock* d_occ[2] = {nullptr, nullptr};
  uint32_t* d_S[2] = {nullptr, nullptr};  // freed once the text-sampled arrays are built
  uint4* d_mark[2] = {nullptr, nullptr};
  uint32_t* d_T[2] = {nullptr, nullptr};
  uint64_t* d_kar_off = nullptr;
  uint64_t* d_kar_start = nullptr;
  uint8_t* d_table = nullptr;
  uint32_t* d_err = nullptr;
  uint2* d_kmer[2] = {nullptr, nullptr};  // start tables of the batched search (X.kmer_len symbols)
  uint8_t h_table[256];

  // workspace
  DevBuf seqs, offs, codes, ok, rs_count, rs_trunc, vecs, slots, ovf, ovf_count, hit_off, scan_part, hits, rows,
      loc_off, locs, census;
  // batched form
  DevBuf b_ctr, b_res, b_sorted, b_spill, b_arr, b_seg, b_rowhit, b_long, b_blocks;
  DevBuf b_bovf;  // block search: results past a block's slots, in chunks
  // alignment-list records (map_device.cu)
  DevBuf m_hitoff, m_part, m_offs, m_rows, m_pflag, m_rowoff, m_nrec, m_flags, m_rec;
  double map_device_s = 0;  // wall time of the last alignment-list call's device pass
  uint32_t b_res_cap = 0, b_spill_cap = 0;
  BatchedTuning tuning;
  int num_sms = 0;
  uint32_t ovf_cap = 0;
  size_t chunk = 0;  // reads per chunk, 0 = automatic
  bool census_on = false;
  unsigned long long census_val = 0;
  cudaEvent_t ev[kStageCount + 1];
  cudaEvent_t cev[4];
  cudaEvent_t dev_mid = nullptr;  // between the search and the drain launch
  float drain_ms = 0;
  float stage_ms[kStageCount] = {0, 0, 0, 0};
  DeviceResult last;
  // batched form replayed from a captured CUDA graph (graph.cu)
  GraphPlan** plans = nullptr;  // two per power-of-two read capacity
  cudaStream_t xs[2] = {nullptr, nullptr};  // host-to-device and device-to-host copy streams (pipelined calls)
  cudaEvent_t pev[3][2];                    // per plan slot: inputs copied, replay done, results copied
  bool pev_made = false;
  double hits_per_read = 2.0, rows_per_read = 2.0;  // result sizing of pipelined calls (running estimate)
  // Graph-plan pools per read of the capacity class, raised whenever a batch
  // overflows one: a class whose first batch comes later starts at the rates
  // earlier batches needed instead of overflowing (and rerunning) first.
  double res_per_read = 4.0, spill_per_read = 0.0, locs_per_read = 8.0;
  size_t pipe_chunk = 0;  // reads per pipelined chunk: 0 automatic, SIZE_MAX never pipelined
  bool use_graph = true;
  bool skip_locate = false;  // batched form: hits only, no located rows
  uint64_t locate_limit = 0;  // rows per (read, strand) list beyond which the list is not located; 0 = none
  float block_ms = 0;         // device time of the last block search
};

// Grow-only device buffer; `keep` preserves the old contents.
inline bool ensure(Engine* e, DevBuf& b, size_t bytes, bool keep = false) {
  if (bytes <= b.cap) return true;
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  void* p = nullptr;
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    want = bytes;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  }
  if (keep && b.p && b.cap) cudaMemcpyAsync(p, b.p, b.cap, cudaMemcpyDeviceToDevice, e->stream);
  if (b.p) {
    cudaStreamSynchronize(e->stream);
    cudaFree(b.p);
  }
  b.p = p;
  b.cap = want;
  return true;
}

// "out of device memory (<what>: <bytes> requested, <bytes> free)": the sizes
// say whether the batch or the device is the problem.
inline std::string oom_message(const char* what, size_t requested) {
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  cudaGetLastError();
  char buf[192];
  snprintf(buf, sizeof buf, "out of device memory (%s: %.2f GB requested, %.2f GB free of %.2f GB)", what,
           requested / 1e9, free_b / 1e9, total_b / 1e9);
  return buf;
}

template <typename T>
inline T* ptr(DevBuf& b) {
  return static_cast<T*>(b.p);
}


// Reads to the engine's device buffers, encoded (codes + validity flags);
// offsets may start anywhere (map_device.cu).
int upload_reads(Engine* e, const char* seqs, const uint64_t* offs, size_t n, std::string* err);

// Graph form of the batched pipeline (graph.cu).
int run_batched_graph(Engine* e, const void* seqs, const uint64_t* offs, uint32_t n, uint64_t total,
                      uint32_t max_results, DeviceResult* out, std::string* err);
void graph_plan_destroy(GraphPlan* g);
void graph_plans_destroy(Engine* e);
// Free the plans of more than max_n_cap reads (after the streams finish).
void graph_plans_drop_above(Engine* e, uint64_t max_n_cap);
// Free the grow-only workspaces of the direct, plain, block-search and
// alignment-list calls (they are allocated again on demand) and the plans of
// more than keep_n_cap reads: a server on the index keeps only what it uses.
void engine_release_workspace(Engine* e, uint64_t keep_n_cap);
// Asynchronous halves of run_batched_graph for a batch already staged in the
// plan's input buffers: launch (header + replay), then collect (synchronize,
// read the summary; returns 1 with `grow` filled when a pool overflowed, the
// batch then has to run again through run_batched_graph).
// `src` (device memory of src_bytes bases): the batch's bases are read there
// in place instead of from the plan's own buffer.
int graph_launch(Engine* e, GraphPlan* g, uint32_t n, uint32_t max_results, std::string* err,
                 const void* src = nullptr, uint64_t src_bytes = 0);
int graph_collect(Engine* e, GraphPlan* g, uint32_t n, GraphPlan* grow, DeviceResult* out, std::string* err);
// The plan serving batches of n reads and `total` bases (captured on demand).
// `pslot` (0/1) picks one of the two plans of a capacity class.
GraphPlan* graph_plan_for(Engine* e, uint32_t n, uint64_t total, const GraphPlan* grow, bool carry,
                          std::string* err, int pslot = 0);
// Recapture, at the per-read pool rates learned so far, every plan of at most
// max_n_cap reads whose pools are below them, except keep0 and keep1 (plans
// that hold a batch); for a caller that has just drained its streams after an
// overflow, so that each capacity class does not overflow (and drain) in turn.
// (Plans above max_n_cap, e.g. a large batched call's, are left alone: a
// recapture holds the old plan and the new one at once.)
int graph_plans_refresh(Engine* e, const GraphPlan* keep0, const GraphPlan* keep1, uint64_t max_n_cap,
                        std::string* err);
// Host reads in, host records out, in chunks whose copies overlap the
// neighbouring chunks' replays (graph.cu).
int run_graph_pipelined(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint64_t total,
                        uint32_t max_results, hpg_result_set_t* out, std::string* err);
// The text-sampled suffix array of both directions (mark + T), derived from the
// row samples already on the device (text_samples.cu); called once at open.
int build_text_samples(Engine* en, const uint32_t n_samples[2], std::string* err);

}  // namespace hpgbwt
