// graph.cu -- the batched pipeline captured once into a CUDA graph and
// replayed per batch.
//
// Every size the pipeline needs lives in device memory: the read count and
// max_results in a small header written before each replay, the hit and row
// totals in the scans' last elements.  Each kernel is captured at a grid sized
// for the plan's capacity (the persistent kernels at one wave) and reads its
// real extent from device memory, so one capture serves every batch of its
// capacity class.  The replay is: inputs + header to the device, one
// cudaGraphLaunch (zeroing, encode, persistent search and drain, ordered
// finalize, persistent locate, a size summary copied to pinned host memory),
// one stream synchronize.  A pool that overflows sets a status bit that the
// later stages check; the host then grows that pool, captures again and reruns
// the batch, so no result is ever dropped.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "engine_internal.hpp"

namespace hpgbwt {


namespace {

constexpr int kMaxPlans = 33;  // one per power-of-two read capacity

__global__ void graph_summary_kernel(const unsigned* __restrict__ ctr, const uint64_t* __restrict__ n_hits,
                                     const uint64_t* __restrict__ n_locs, const unsigned long long* census,
                                     uint64_t* __restrict__ out) {
  out[0] = (uint64_t)ctr[4] | ((uint64_t)ctr[3] << 32);
  out[1] = ctr[2];
  out[2] = *n_hits;
  out[3] = *n_locs;
  out[4] = census ? *census : 0ull;
}

uint64_t pow2_at_least(uint64_t v, uint64_t lo) {
  uint64_t p = lo;
  while (p < v) p <<= 1;
  return p;
}

int log2_of(uint64_t p) {
  int k = 0;
  while ((1ull << k) < p) ++k;
  return k;
}

template <typename T>
bool grab(GraphPlan* g, T** p, size_t bytes) {
  void* q = nullptr;
  if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  g->allocs.push_back(q);
  g->bytes += bytes ? bytes : 16;
  *p = static_cast<T*>(q);
  return true;
}

bool same_settings(const GraphPlan* g, const Engine* e) {
  const BatchedTuning& a = g->tuning;
  const BatchedTuning& b = e->tuning;
  return a.block == b.block && a.blocks_per_sm == b.blocks_per_sm && a.stack == b.stack && a.chunk == b.chunk &&
         a.min_blocks == b.min_blocks && a.split == b.split && g->load_mode == e->X.load_mode &&
         g->census == e->census_on && g->skip_locate == e->skip_locate;
}

void record(cudaEvent_t ev, cudaStream_t s) { cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal); }

// Allocate the plan's buffers and capture the pipeline on the engine stream.
int capture(Engine* e, GraphPlan* g, std::string* err) {
  const size_t T = 2ull * g->n_cap;
  const size_t parts = std::max(scan_parts(T), scan_parts(g->res_cap));
  if (!grab(g, &g->seqs, g->bases_cap + 64) || !grab(g, &g->offs, ((size_t)g->n_cap + 1) * 8) ||
      !grab(g, &g->hdr, 16) || !grab(g, &g->codes, g->bases_cap + 64) || !grab(g, &g->ok, (size_t)g->n_cap + 16) ||
      !grab(g, &g->ctr, 64) || !grab(g, &g->arr, T * 4 + 16) || !grab(g, &g->seg, (T + 1) * 8) ||
      !grab(g, &g->hit_off, (T + 1) * 8) || !grab(g, &g->kept, T * 4 + 16) || !grab(g, &g->trunc, T + 16) ||
      !grab(g, &g->part, parts * 8) || !grab(g, &g->res, (size_t)g->res_cap * sizeof(PendingHit)) ||
      !grab(g, &g->sorted, (size_t)g->res_cap * sizeof(PendingHit)) ||
      !grab(g, &g->spill, (size_t)g->spill_cap * sizeof(SpillEntry)) ||
      !grab(g, &g->hits, ((size_t)g->res_cap + 1) * sizeof(hpg_hit_t)) ||
      !grab(g, &g->rows, ((size_t)g->res_cap + 1) * 4) || !grab(g, &g->loc_off, ((size_t)g->res_cap + 2) * 8) ||
      !grab(g, &g->items, (g->locs_cap + 1) * locate_row_item_bytes()) ||
      !grab(g, &g->locs, (g->locs_cap + 1) * sizeof(hpg_loc_t)) || !grab(g, &g->census_d, 16) ||
      !grab(g, &g->summary_d, 64)) {
    *err = "out of device memory (graph plan)";
    return -1;
  }
  HPG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->h_summary), 64, cudaHostAllocDefault), "pinned summary");
  HPG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->h_hdr), 16, cudaHostAllocDefault), "pinned header");
  for (cudaEvent_t& ev : g->ev) HPG_CUDA(cudaEventCreate(&ev), "graph events");
  HPG_CUDA(cudaMemset(g->offs, 0, 8), "graph plan");  // an empty batch reads offs[0]

  cudaStream_t s = e->stream;
  unsigned* ctr = g->ctr;
  unsigned* status = ctr + 4;
  unsigned long long* census = g->census ? g->census_d : nullptr;
  const unsigned long long launches_before = launch_count();
  HPG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  record(g->ev[0], s);
  cudaMemsetAsync(ctr, 0, 64, s);
  cudaMemsetAsync(g->arr, 0, T * 4, s);
  cudaMemsetAsync(g->rows, 0, (size_t)g->res_cap * 4, s);
  if (census) cudaMemsetAsync(census, 0, 8, s);
  launch_encode_dev(g->seqs, g->bases_cap, g->offs, g->hdr, g->n_cap, e->d_table, g->codes, g->ok, s);
  launch_check_offsets(g->offs, g->hdr, g->n_cap, g->bases_cap, g->ok, status, s);
  record(g->ev[1], s);

  BatchedParams p;
  p.codes = g->codes;
  p.offs = g->offs;
  p.ok = g->ok;
  p.n_reads = g->n_cap;
  p.n_reads_dev = g->hdr;
  p.max_results = 0;  // truncation happens in the finalize, from the header
  p.chain_ctr = ctr + 0;
  p.spill_head = ctr + 1;
  p.spill_tail = ctr + 2;
  p.spill = g->spill;
  p.spill_cap = g->spill_cap;
  p.res_total = ctr + 3;
  p.res = g->res;
  p.res_cap = g->res_cap;
  p.rs_count = g->arr;
  p.status = status;
  p.census = census;
  if (g->tuning.split == 1) {
    BatchedTuning t = g->tuning;
    BatchedParams p1 = p;
    p1.chain_ctr = ctr + 8;
    t.phase = 0;
    launch_batched_search(e->X, p, t, e->num_sms, false, s);
    launch_batched_search(e->X, p, t, e->num_sms, true, s);
    cudaMemcpyAsync(ctr + 1, ctr + 2, 4, cudaMemcpyDeviceToDevice, s);  // drain resumes at the queue tail
    record(g->ev[2], s);
    t.phase = 1;
    launch_batched_search(e->X, p1, t, e->num_sms, false, s);
    launch_batched_search(e->X, p1, t, e->num_sms, true, s);
  } else {
    launch_batched_search(e->X, p, g->tuning, e->num_sms, false, s);
    record(g->ev[2], s);
    launch_batched_search(e->X, p, g->tuning, e->num_sms, true, s);
  }
  record(g->ev[3], s);

  // ordered finalize over the capacity (lists past the batch are empty)
  launch_scan(g->arr, T, g->seg, g->part, s);
  cudaMemsetAsync(g->hit_off, 0, T * 4, s);  // per-list cursors (hit_off is rewritten below)
  launch_scatter_hits(g->res, ctr + 3, g->seg, g->sorted, g->res_cap, reinterpret_cast<uint32_t*>(g->hit_off), s,
                      status);
  launch_sort_truncate(g->sorted, g->seg, (uint32_t)T, 0, g->kept, g->trunc, s, g->hdr + 1, status);
  launch_scan(g->kept, T, g->hit_off, g->part, s);
  launch_expand_hits(g->sorted, g->seg, g->hit_off, g->kept, (uint32_t)T, g->hits, g->rows, s, status);
  launch_scan(g->rows, g->res_cap, g->loc_off, g->part, s);
  record(g->ev[4], s);

  LocateSizes z;
  z.status = status;
  z.n_hits = g->hit_off + T;
  z.n_locs = g->loc_off + g->res_cap;
  z.locs_cap = g->locs_cap;
  if (!g->skip_locate)
    launch_locate_persistent(e->X, g->hits, g->loc_off, g->res_cap, g->locs_cap, g->offs, g->locs, g->items,
                             ctr + 5, census, e->num_sms, s, z);
  record(g->ev[5], s);
  count_launches(1);
  graph_summary_kernel<<<1, 1, 0, s>>>(ctr, z.n_hits, z.n_locs, census, g->summary_d);
  cudaMemcpyAsync(g->h_summary, g->summary_d, 40, cudaMemcpyDeviceToHost, s);
  const cudaError_t ce = cudaStreamEndCapture(s, &g->graph);
  g->kernels = launch_count() - launches_before;
  uncount_launches(g->kernels);
  if (ce != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    *err = std::string("graph capture: ") + cudaGetErrorString(ce);
    return -1;
  }
  HPG_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0), "graph instantiate");
  return 0;
}

}  // namespace

void graph_plan_destroy(GraphPlan* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (void* q : g->allocs) cudaFree(q);
  if (g->h_summary) cudaFreeHost(g->h_summary);
  if (g->h_hdr) cudaFreeHost(g->h_hdr);
  for (cudaEvent_t ev : g->ev)
    if (ev) cudaEventDestroy(ev);
  delete g;
}

void graph_plans_destroy(Engine* e) {
  if (!e->plans) return;
  cudaStreamSynchronize(e->stream);
  for (int i = 0; i < kMaxPlans; ++i) graph_plan_destroy(e->plans[i]);
  delete[] e->plans;
  e->plans = nullptr;
}

// The plan for a batch of n reads and `total` bases: one per power-of-two read
// capacity, captured again when the tuning, block-load form or census setting
// changed, or when a pool has to grow.
// With `carry` the batch already staged in the old plan's input buffers (n
// reads, `total` bases) is copied into the new plan's.
GraphPlan* graph_plan_for(Engine* e, uint32_t n, uint64_t total, const GraphPlan* grow, bool carry,
                          std::string* err) {
  if (!e->plans) {
    e->plans = new GraphPlan*[kMaxPlans];
    for (int i = 0; i < kMaxPlans; ++i) e->plans[i] = nullptr;
  }
  const uint64_t n_cap = pow2_at_least(n, 4096);
  const int slot = log2_of(n_cap);
  GraphPlan* g = e->plans[slot];
  const uint64_t bases_cap = pow2_at_least(total, n_cap * 128);
  uint32_t res_cap = (uint32_t)std::min<uint64_t>(4 * n_cap + 4096, 0xFFFFFFF0u);
  uint32_t spill_cap = (uint32_t)std::min<uint64_t>(
      e->tuning.split ? 4 * n_cap + 4096 + (uint64_t)e->num_sms * 16 * 128 * 8 : n_cap / 4 + 4096, 0xFFFFFFF0u);
  uint64_t locs_cap = 8 * n_cap + 4096;
  if (g) {  // keep what earlier batches of this class needed
    res_cap = std::max(res_cap, g->res_cap);
    spill_cap = std::max(spill_cap, g->spill_cap);
    locs_cap = std::max(locs_cap, g->locs_cap);
  }
  if (grow) {
    res_cap = std::max(res_cap, grow->res_cap);
    spill_cap = std::max(spill_cap, grow->spill_cap);
    locs_cap = std::max(locs_cap, grow->locs_cap);
  }
  if (g && same_settings(g, e) && g->bases_cap >= total && g->res_cap >= res_cap && g->spill_cap >= spill_cap &&
      g->locs_cap >= locs_cap)
    return g;
  GraphPlan* old = g;
  g = new GraphPlan();
  g->n_cap = (uint32_t)n_cap;
  g->bases_cap = old ? std::max(old->bases_cap, bases_cap) : bases_cap;
  g->res_cap = res_cap;
  g->spill_cap = spill_cap;
  g->locs_cap = locs_cap;
  g->tuning = e->tuning;
  g->load_mode = e->X.load_mode;
  g->census = e->census_on;
  g->skip_locate = e->skip_locate;
  if (old) cudaStreamSynchronize(e->stream);
  if (capture(e, g, err) != 0) {
    graph_plan_destroy(g);
    return nullptr;
  }
  if (old) {
    if (carry) {
      if (total) cudaMemcpyAsync(g->seqs, old->seqs, total, cudaMemcpyDeviceToDevice, e->stream);
      cudaMemcpyAsync(g->offs, old->offs, ((size_t)n + 1) * 8, cudaMemcpyDeviceToDevice, e->stream);
      cudaStreamSynchronize(e->stream);
    }
    graph_plan_destroy(old);
  }
  e->plans[slot] = g;
  return g;
}

int graph_launch(Engine* e, GraphPlan* g, uint32_t n, uint32_t max_results, std::string* err) {
  cudaStream_t s = e->stream;
  g->h_hdr[0] = n;
  g->h_hdr[1] = max_results;
  HPG_CUDA(cudaMemcpyAsync(g->hdr, g->h_hdr, 8, cudaMemcpyHostToDevice, s), "batch header");
  HPG_CUDA(cudaGraphLaunch(g->exec, s), "graph launch");
  count_launches((unsigned)g->kernels);
  return 0;
}

int graph_collect(Engine* e, GraphPlan* g, uint32_t n, GraphPlan* grow, DeviceResult* out, std::string* err) {
  HPG_CUDA(cudaStreamSynchronize(e->stream), "batched pipeline");
  const uint64_t* h = g->h_summary;
  const uint32_t status = (uint32_t)h[0];
  if (status & kStatusBadInput) {
    *err = "read offsets must be non-decreasing and reads at most 32767 bases";
    return -1;
  }
  if (status) {
    grow->res_cap = g->res_cap;
    grow->spill_cap = g->spill_cap;
    grow->locs_cap = g->locs_cap;
    if (status & kStatusResFull) grow->res_cap = (uint32_t)std::min<uint64_t>((h[0] >> 32) * 2 + 4096, 0xFFFFFFF0u);
    if (status & kStatusSpillFull) grow->spill_cap = (uint32_t)std::min<uint64_t>(h[1] * 2 + 4096, 0xFFFFFFF0u);
    if (status & kStatusLocFull) grow->locs_cap = h[3] + h[3] / 4 + 4096;
    return 1;
  }
  e->census_val = g->census ? h[4] : 0;
  float ms = 0;
  cudaEventElapsedTime(&e->stage_ms[kStageEncode], g->ev[0], g->ev[1]);
  cudaEventElapsedTime(&e->stage_ms[kStageSearch], g->ev[1], g->ev[3]);
  cudaEventElapsedTime(&e->drain_ms, g->ev[2], g->ev[3]);
  cudaEventElapsedTime(&ms, g->ev[3], g->ev[4]);
  e->stage_ms[kStageFinalize] = ms;
  cudaEventElapsedTime(&ms, g->ev[4], g->ev[5]);
  e->stage_ms[kStageLocate] = ms;
  DeviceResult r;
  r.n_reads = n;
  r.n_hits = h[2];
  r.hits = g->hits;
  r.n_locs = g->skip_locate ? 0 : h[3];
  r.locs = g->locs;
  r.rs_count = g->kept;
  r.rs_truncated = g->trunc;
  *out = r;
  return 0;
}

int run_batched_graph(Engine* e, const void* seqs, const uint64_t* offs, uint32_t n, uint64_t total,
                      uint32_t max_results, DeviceResult* out, std::string* err) {
  cudaStream_t s = e->stream;
  GraphPlan grow;
  const GraphPlan* staged_in = nullptr;  // plan whose own buffers hold the batch
  if (e->plans)
    for (int i = 0; i < kMaxPlans; ++i)
      if (e->plans[i] && seqs == e->plans[i]->seqs && offs == e->plans[i]->offs) staged_in = e->plans[i];
  for (int attempt = 0; attempt < 8; ++attempt) {
    GraphPlan* g = graph_plan_for(e, n, total, attempt ? &grow : nullptr, staged_in != nullptr, err);
    if (!g) return -1;
    if (staged_in) {  // follow the batch into a replacement plan
      seqs = g->seqs;
      offs = g->offs;
      staged_in = g;
    }
    if (total && seqs != g->seqs) HPG_CUDA(cudaMemcpyAsync(g->seqs, seqs, total, cudaMemcpyDefault, s), "reads");
    if (offs != g->offs)
      HPG_CUDA(cudaMemcpyAsync(g->offs, offs, ((size_t)n + 1) * 8, cudaMemcpyDefault, s), "read offsets");
    if (graph_launch(e, g, n, max_results, err) != 0) return -1;
    const int rc = graph_collect(e, g, n, &grow, out, err);
    if (rc < 0) return -1;
    if (rc == 0) return 0;
  }
  *err = "batched search pools kept overflowing";
  return -1;
}

}  // namespace hpgbwt
