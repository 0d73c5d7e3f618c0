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
#include "host_pool.hpp"

namespace hpgbwt {


namespace {

constexpr int kMaxPlans = 33;  // one per power-of-two read capacity
constexpr int kPlanSlots = 2;  // two plans per capacity: chunks of one batch alternate between them

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
         a.min_blocks == b.min_blocks && a.split == b.split && a.dir_split == b.dir_split &&
         a.batch_idle == b.batch_idle && a.group == b.group &&
         g->load_mode == e->X.load_mode &&
         g->census == e->census_on && g->skip_locate == e->skip_locate && g->kmer_len == e->X.kmer_len &&
         g->kmer0 == (const void*)e->X.kmer[0];
}

void record(cudaEvent_t ev, cudaStream_t s) { cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal); }

// Allocate the plan's buffers and capture the pipeline on the engine stream.
int capture(Engine* e, GraphPlan* g, std::string* err) {
  const size_t T = 2ull * g->n_cap;
  const size_t parts = std::max(scan_parts(T), scan_parts(g->res_cap));
  if (!grab(g, &g->seqs, g->bases_cap + 64) || !grab(g, &g->offs, ((size_t)g->n_cap + 1) * 8) ||
      !grab(g, &g->hdr, 32) || !grab(g, &g->codes, g->bases_cap + 64) || !grab(g, &g->ok, (size_t)g->n_cap + 16) ||
      !grab(g, &g->ctr, 64) || !grab(g, &g->arr, T * 4 + 16) || !grab(g, &g->seg, (T + 1) * 8) ||
      !grab(g, &g->hit_off, (T + 1) * 8) || !grab(g, &g->kept, T * 4 + 16) || !grab(g, &g->trunc, T + 16) ||
      !grab(g, &g->part, parts * 8) || !grab(g, &g->res, (size_t)g->res_cap * sizeof(PendingHit)) ||
      !grab(g, &g->sorted, (size_t)g->res_cap * sizeof(PendingHit)) ||
      !grab(g, &g->spill, (size_t)g->spill_cap * sizeof(SpillEntry)) ||
      !grab(g, &g->hits, ((size_t)g->res_cap + 1) * sizeof(hpg_hit_t)) ||
      !grab(g, &g->rows, ((size_t)g->res_cap + 1) * 4) || !grab(g, &g->loc_off, ((size_t)g->res_cap + 2) * 8) ||
      !grab(g, &g->items, (g->locs_cap + 1) * locate_row_item_bytes()) ||
      !grab(g, &g->locs, (g->locs_cap + 1) * sizeof(hpg_loc_t)) || !grab(g, &g->census_d, 16) ||
      !grab(g, &g->long_list, (size_t)g->long_cap * 4) || !grab(g, &g->longs, long_lists_cap(g->res_cap) * 4) ||
      (g->tuning.split == 3 && !grab(g, &g->blocks, (size_t)g->spill_cap * sizeof(SpillEntry))) ||
      !grab(g, &g->summary_d, 64)) {
    *err = "out of device memory (graph plan)";
    return -1;
  }
  HPG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->h_summary), 64, cudaHostAllocDefault), "pinned summary");
  HPG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->h_hdr), 32, cudaHostAllocDefault), "pinned header");
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
  if (census) cudaMemsetAsync(census, 0, 8, s);
  launch_encode_dev(g->seqs, g->bases_cap, g->offs, g->hdr, g->n_cap, e->d_table, g->codes, g->ok, s,
                    reinterpret_cast<const uint64_t*>(g->hdr + 4));
  launch_check_offsets(g->offs, g->hdr, g->n_cap, g->bases_cap, g->ok, status, s);
  record(g->ev[1], s);

  BatchedParams p;
  p.codes = g->codes;
  p.codes_len = g->bases_cap + 64;
  p.offs = g->offs;
  p.ok = g->ok;
  p.n_reads = g->n_cap;
  p.n_reads_dev = g->hdr;
  p.max_results = 0;  // truncation happens in the finalize, from the header
  p.chain_ctr = ctr + 0;
  p.chain_ctr2 = ctr + 9;
  p.dir_split = g->tuning.split == 0 ? (uint32_t)g->tuning.dir_split : 0u;
  p.num_sms = (uint32_t)e->num_sms;
  p.batch_idle = (uint32_t)(g->tuning.batch_idle < 1 ? 1 : g->tuning.batch_idle);
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
  launch_search_stage(e->X, p, g->tuning, e->num_sms, ctr, g->long_list, g->long_cap, g->blocks,
                      g->blocks ? g->spill_cap : 0u, g->ev[2], true, s);
  record(g->ev[3], s);

  // ordered finalize over the capacity (lists past the batch are empty)
  launch_scan(g->arr, T, g->seg, g->part, s);
  cudaMemsetAsync(g->hit_off, 0, T * 4, s);  // per-list cursors (hit_off is rewritten below)
  launch_scatter_hits(g->res, ctr + 3, g->seg, g->sorted, g->res_cap, reinterpret_cast<uint32_t*>(g->hit_off), s,
                      status);
  launch_sort_truncate(g->sorted, g->res, g->seg, (uint32_t)T, 0, g->kept, g->trunc, e->num_sms, s, g->hdr + 1,
                       status, g->longs, ctr + 14, (uint32_t)long_lists_cap(g->res_cap));
  launch_scan(g->kept, T, g->hit_off, g->part, s);
  launch_expand_hits(g->sorted, g->seg, g->hit_off, g->kept, (uint32_t)T, g->hits, g->rows, s, status, g->longs,
                     ctr + 14, (uint32_t)long_lists_cap(g->res_cap), e->num_sms);
  launch_limit_rows(g->hit_off, g->rows, (uint32_t)T, 0, reinterpret_cast<const uint64_t*>(g->hdr + 2), g->trunc, s,
                    status);
  launch_scan(g->rows, g->res_cap, g->loc_off, g->part, s, g->hit_off + T);  // over the hits found
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
  for (cudaStream_t x : e->xs)
    if (x) cudaStreamSynchronize(x);
  for (int i = 0; i < kMaxPlans * kPlanSlots; ++i) graph_plan_destroy(e->plans[i]);
  delete[] e->plans;
  e->plans = nullptr;
}

void graph_plans_drop_above(Engine* e, uint64_t max_n_cap) {
  if (!e->plans) return;
  cudaStreamSynchronize(e->stream);
  for (cudaStream_t x : e->xs)
    if (x) cudaStreamSynchronize(x);
  for (int i = 0; i < kMaxPlans * kPlanSlots; ++i)
    if (e->plans[i] && e->plans[i]->n_cap > max_n_cap) {
      graph_plan_destroy(e->plans[i]);
      e->plans[i] = nullptr;
    }
}

// The plan for a batch of n reads and `total` bases: one per power-of-two read
// capacity, captured again when the tuning, block-load form or census setting
// changed, or when a pool has to grow.
// With `carry` the batch already staged in the old plan's input buffers (n
// reads, `total` bases) is copied into the new plan's.
GraphPlan* graph_plan_for(Engine* e, uint32_t n, uint64_t total, const GraphPlan* grow, bool carry,
                          std::string* err, int pslot) {
  if (!e->plans) {
    e->plans = new GraphPlan*[kMaxPlans * kPlanSlots];
    for (int i = 0; i < kMaxPlans * kPlanSlots; ++i) e->plans[i] = nullptr;
  }
  if (n >= (1u << 31) || total > (1ull << 40)) {
    *err = "batch too large for one graph plan";
    return nullptr;
  }
  const uint64_t n_cap = pow2_at_least(n, 4096);
  const int slot = log2_of(n_cap) * kPlanSlots + (pslot & 1);
  GraphPlan* g = e->plans[slot];
  const uint64_t bases_cap = pow2_at_least(total, n_cap * 128);
  // a plan captured now starts at the per-read rates earlier overflows showed; a
  // plan that exists keeps its pools until a batch of its own overflows them (a
  // recapture drains every stream, which a serving pipeline should not pay for
  // a batch that fits)
  const double nc = (double)n_cap;
  const bool fresh = !g || !same_settings(g, e);
  const double res_rate = fresh ? std::max(4.0, e->res_per_read) : 4.0;
  const double locs_rate = fresh ? std::max(8.0, e->locs_per_read) : 8.0;
  const double spill_rate = fresh ? e->spill_per_read : 0.0;
  uint32_t res_cap = (uint32_t)std::min<double>(res_rate * nc + 4096, 0xFFFFFFF0u);
  uint32_t spill_cap = (uint32_t)std::min<double>(
      std::max(spill_rate * nc, e->tuning.split ? 4 * nc + 4096 + (double)e->num_sms * 16 * 128 * 8 : nc / 4 + 4096),
      0xFFFFFFF0u);
  uint64_t locs_cap = (uint64_t)std::min<double>(locs_rate * nc + 4096, kMaxLocateRows);
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
  g->long_cap = (uint32_t)std::min<uint64_t>(g->bases_cap / kWaveLongMin + 2, 0xFFFFFFF0u);
  g->res_cap = res_cap;
  g->spill_cap = spill_cap;
  g->locs_cap = locs_cap;
  g->tuning = e->tuning;
  g->load_mode = e->X.load_mode;
  g->census = e->census_on;
  g->skip_locate = e->skip_locate;
  g->kmer_len = e->X.kmer_len;
  g->kmer0 = e->X.kmer[0];
  if (old) {  // no stream may still read the old plan's buffers
    cudaStreamSynchronize(e->stream);
    for (cudaStream_t x : e->xs)
      if (x) cudaStreamSynchronize(x);
  }
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

int graph_plans_refresh(Engine* e, const GraphPlan* keep0, const GraphPlan* keep1, uint64_t max_n_cap,
                        std::string* err) {
  if (!e->plans) return 0;
  for (int i = 0; i < kMaxPlans * kPlanSlots; ++i) {
    GraphPlan* g = e->plans[i];
    if (!g || g == keep0 || g == keep1 || g->n_cap > max_n_cap || !same_settings(g, e)) continue;
    const double nc = (double)g->n_cap;
    GraphPlan grow;
    grow.res_cap = (uint32_t)std::min<double>(std::max(4.0, e->res_per_read) * nc + 4096, 0xFFFFFFF0u);
    grow.spill_cap = (uint32_t)std::min<double>(e->spill_per_read * nc, 0xFFFFFFF0u);
    grow.locs_cap = (uint64_t)std::min<double>(std::max(8.0, e->locs_per_read) * nc + 4096, kMaxLocateRows);
    if (g->res_cap >= grow.res_cap && g->spill_cap >= grow.spill_cap && g->locs_cap >= grow.locs_cap) continue;
    if (!graph_plan_for(e, g->n_cap, g->bases_cap, &grow, false, err, i % kPlanSlots)) return -1;
  }
  return 0;
}

int graph_launch(Engine* e, GraphPlan* g, uint32_t n, uint32_t max_results, std::string* err, const void* src,
                 uint64_t src_bytes) {
  cudaStream_t s = e->stream;
  g->h_hdr[0] = n;
  g->h_hdr[1] = max_results;
  const uint64_t limit = e->skip_locate ? 0 : e->locate_limit;  // hits-only calls locate nothing anyway
  std::memcpy(g->h_hdr + 2, &limit, 8);
  const uint64_t src_hdr[2] = {reinterpret_cast<uint64_t>(src), src ? src_bytes : 0};
  std::memcpy(g->h_hdr + 4, src_hdr, 16);
  HPG_CUDA(cudaMemcpyAsync(g->hdr, g->h_hdr, 32, cudaMemcpyHostToDevice, s), "batch header");
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
  if (status & kStatusWaveAcct) {
    *err = "internal error: inconsistent work counts in the warp-cooperative search";
    return -1;
  }
  if (status) {
    // the rates this batch needed, with room, for every capacity class from now on
    const double nr = std::max<double>(n, 1.0);
    if (status & kStatusResFull) e->res_per_read = std::max(e->res_per_read, 1.5 * (double)(h[0] >> 32) / nr);
    if (status & kStatusSpillFull) e->spill_per_read = std::max(e->spill_per_read, 1.5 * (double)h[1] / nr);
    if (status & kStatusLocFull) e->locs_per_read = std::max(e->locs_per_read, 1.25 * (double)h[3] / nr);
    grow->res_cap = g->res_cap;
    grow->spill_cap = g->spill_cap;
    grow->locs_cap = g->locs_cap;
    if (status & kStatusResFull) grow->res_cap = (uint32_t)std::min<uint64_t>((h[0] >> 32) * 2 + 4096, 0xFFFFFFF0u);
    if (status & kStatusSpillFull) grow->spill_cap = (uint32_t)std::min<uint64_t>(h[1] * 2 + 4096, 0xFFFFFFF0u);
    if (status & kStatusLocFull) {
      if (h[3] > kMaxLocateRows) {
        *err = "too many located rows in one batched call (" + std::to_string(h[3]) + ", limit " +
               std::to_string(kMaxLocateRows) + "): split the batch or use the plain form";
        return -1;
      }
      grow->locs_cap = std::min<uint64_t>(h[3] + h[3] / 4 + 4096, kMaxLocateRows);
    }
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

namespace {

// Read and hit ids of one chunk made batch-wide.
__global__ void chunk_rebase_kernel(hpg_hit_t* __restrict__ hits, uint64_t n_hits, uint32_t r0,
                                    hpg_loc_t* __restrict__ locs, uint64_t n_locs, uint32_t h0) {
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = tid; i < n_hits; i += stride) hits[i].read += r0;
  for (uint64_t j = tid; j < n_locs; j += stride) locs[j].hit += h0;
}

// A result array that grows (page-locked blocks) while chunks land in it.
template <typename T>
bool reserve(T** p, size_t* cap, size_t used, size_t want, cudaStream_t copies) {
  if (want <= *cap) return true;
  const size_t n = std::max(want, *cap + *cap / 2);
  T* q = static_cast<T*>(host_pool_alloc(n * sizeof(T)));
  if (!q) return false;
  if (*p) {
    cudaStreamSynchronize(copies);  // earlier chunks must have landed
    if (used) std::memcpy(q, *p, used * sizeof(T));
    host_pool_free(*p);
  }
  *p = q;
  *cap = n;
  return true;
}

}  // namespace

int run_graph_pipelined(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint64_t total,
                        uint32_t max_results, hpg_result_set_t* out, std::string* err) {
  (void)total;
  const size_t chunk = e->pipe_chunk ? e->pipe_chunk : std::max<size_t>(262144, (n + 3) / 4);
  if (chunk == 0 || n == 0) return -1;
  const size_t K = (n + chunk - 1) / chunk;
  if (!e->xs[0]) {
    HPG_CUDA(cudaStreamCreateWithFlags(&e->xs[0], cudaStreamNonBlocking), "copy stream");
    HPG_CUDA(cudaStreamCreateWithFlags(&e->xs[1], cudaStreamNonBlocking), "copy stream");
  }
  if (!e->pev_made) {
    for (auto& row : e->pev)
      for (cudaEvent_t& ev : row) HPG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "pipeline events");
    e->pev_made = true;
  }
  cudaStream_t cs = e->stream, h2d = e->xs[0], d2h = e->xs[1];
  cudaEvent_t* ev_in = e->pev[0];
  cudaEvent_t* ev_run = e->pev[1];
  cudaEvent_t* ev_out = e->pev[2];
  // page-locked staging of each slot's chunk offsets
  std::vector<uint64_t*> stage(2, nullptr);
  for (int s = 0; s < 2; ++s) {
    stage[s] = static_cast<uint64_t*>(host_pool_alloc((chunk + 1) * 8));
    if (!stage[s]) {
      *err = "out of host memory (chunk offsets)";
      return -1;
    }
  }
  auto release = [&]() {
    for (uint64_t* p : stage) host_pool_free(p);
  };
  // result arrays, sized from the hit and row rates of the previous call
  std::memset(out, 0, sizeof(*out));
  out->n_reads = n;
  out->rs_count = static_cast<uint32_t*>(host_pool_alloc((2 * n + 1) * 4));
  out->rs_truncated = static_cast<uint8_t*>(host_pool_alloc(2 * n + 1));
  size_t hcap = 0, lcap = 0;
  const size_t hguess = (size_t)(e->hits_per_read * 1.25 * (double)n) + 1024;
  const size_t lguess = (size_t)(e->rows_per_read * 1.25 * (double)n) + 1024;
  if (!out->rs_count || !out->rs_truncated || !reserve(&out->hits, &hcap, 0, hguess, d2h) ||
      !reserve(&out->locs, &lcap, 0, lguess, d2h)) {
    release();
    *err = "out of host memory (results)";
    return -1;
  }
  std::vector<GraphPlan*> plan(K, nullptr);
  std::vector<uint32_t> nr(K);
  float st[kStageCount + 1] = {0, 0, 0, 0, 0};
  auto issue = [&](size_t i) -> int {
    const int s = (int)(i & 1);
    const size_t r0 = i * chunk, r1 = std::min(n, r0 + chunk);
    nr[i] = (uint32_t)(r1 - r0);
    if (offs[r1] < offs[r0]) {
      *err = "read offsets must be non-decreasing and reads at most 32767 bases";
      return -1;
    }
    const uint64_t b0 = offs[r0], bases = offs[r1] - b0;
    GraphPlan* g = graph_plan_for(e, nr[i], bases, nullptr, false, err, s);
    if (!g) return -1;
    plan[i] = g;
    HPG_CUDA(cudaEventSynchronize(ev_in[s]), "chunk staging");  // the slot's previous offsets were sent
    for (size_t r = r0; r <= r1; ++r) stage[s][r - r0] = offs[r] - b0;
    // inputs once the slot's previous replay has finished with them
    HPG_CUDA(cudaStreamWaitEvent(h2d, ev_run[s], 0), "pipeline order");
    if (bases) HPG_CUDA(cudaMemcpyAsync(g->seqs, seqs + b0, bases, cudaMemcpyDefault, h2d), "chunk reads");
    HPG_CUDA(cudaMemcpyAsync(g->offs, stage[s], (nr[i] + 1) * 8, cudaMemcpyHostToDevice, h2d), "chunk offsets");
    HPG_CUDA(cudaEventRecord(ev_in[s], h2d), "pipeline order");
    // replay once the inputs are in and the slot's previous results are out
    HPG_CUDA(cudaStreamWaitEvent(cs, ev_in[s], 0), "pipeline order");
    HPG_CUDA(cudaStreamWaitEvent(cs, ev_out[s], 0), "pipeline order");
    if (graph_launch(e, g, nr[i], max_results, err) != 0) return -1;
    HPG_CUDA(cudaEventRecord(ev_run[s], cs), "pipeline order");
    return 0;
  };
  size_t h0 = 0, l0 = 0;
  auto collect = [&](size_t i) -> int {
    const int s = (int)(i & 1);
    GraphPlan* g = plan[i];
    HPG_CUDA(cudaEventSynchronize(ev_run[s]), "chunk replay");
    const uint64_t* h = g->h_summary;
    if ((uint32_t)h[0] & kStatusBadInput) {
      *err = "read offsets must be non-decreasing and reads at most 32767 bases";
      return -1;
    }
    if ((uint32_t)h[0]) {  // a pool overflowed: grow it and rerun this chunk alone
      HPG_CUDA(cudaStreamSynchronize(h2d), "pipeline drain");
      HPG_CUDA(cudaStreamSynchronize(d2h), "pipeline drain");
      HPG_CUDA(cudaStreamSynchronize(cs), "pipeline drain");
      const size_t r0 = i * chunk;
      DeviceResult r;
      if (run_batched_graph(e, g->seqs, g->offs, nr[i], offs[r0 + nr[i]] - offs[r0], max_results, &r, err) != 0)
        return -1;
      g = plan[i] = graph_plan_for(e, nr[i], offs[r0 + nr[i]] - offs[r0], nullptr, false, err, s);
      if (!g) return -1;
      h = g->h_summary;  // the rerun's summary, in the grown plan
      HPG_CUDA(cudaEventRecord(ev_run[s], cs), "pipeline order");
    }
    const uint64_t nh = h[2], nl = g->skip_locate ? 0 : h[3];
    if (!reserve(&out->hits, &hcap, h0, h0 + nh + 1, d2h) || !reserve(&out->locs, &lcap, l0, l0 + nl + 1, d2h)) {
      *err = "out of host memory (results)";
      return -1;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]);
    st[kStageEncode] += ms;
    cudaEventElapsedTime(&ms, g->ev[1], g->ev[3]);
    st[kStageSearch] += ms;
    cudaEventElapsedTime(&ms, g->ev[2], g->ev[3]);
    st[kStageCount] += ms;
    cudaEventElapsedTime(&ms, g->ev[3], g->ev[4]);
    st[kStageFinalize] += ms;
    cudaEventElapsedTime(&ms, g->ev[4], g->ev[5]);
    st[kStageLocate] += ms;
    const size_t r0 = i * chunk;
    HPG_CUDA(cudaStreamWaitEvent(d2h, ev_run[s], 0), "pipeline order");
    if ((r0 || h0) && (nh || nl)) {
      const uint64_t work = std::max<uint64_t>(nh, nl);
      count_launches(1);
      chunk_rebase_kernel<<<(unsigned)std::min<uint64_t>((work + 255) / 256, 1216), 256, 0, d2h>>>(
          g->hits, nh, (uint32_t)r0, g->locs, nl, (uint32_t)h0);
    }
    if (nh) HPG_CUDA(cudaMemcpyAsync(out->hits + h0, g->hits, nh * sizeof(hpg_hit_t), cudaMemcpyDeviceToHost, d2h),
                     "copy hits");
    if (nl) HPG_CUDA(cudaMemcpyAsync(out->locs + l0, g->locs, nl * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, d2h),
                     "copy rows");
    HPG_CUDA(cudaMemcpyAsync(out->rs_count + 2 * r0, g->kept, 2ull * nr[i] * 4, cudaMemcpyDeviceToHost, d2h),
             "copy counts");
    HPG_CUDA(cudaMemcpyAsync(out->rs_truncated + 2 * r0, g->trunc, 2ull * nr[i], cudaMemcpyDeviceToHost, d2h),
             "copy flags");
    HPG_CUDA(cudaEventRecord(ev_out[s], d2h), "pipeline order");
    h0 += nh;
    l0 += nl;
    return 0;
  };
  int rc = 0;
  for (size_t i = 0; i < K && rc == 0; ++i) {
    rc = issue(i);
    if (rc == 0 && i >= 1) rc = collect(i - 1);
  }
  if (rc == 0) rc = collect(K - 1);
  cudaError_t ce = cudaStreamSynchronize(d2h);
  release();
  if (rc != 0) return -1;
  if (ce != cudaSuccess) {
    *err = std::string("result copies: ") + cudaGetErrorString(ce);
    return -1;
  }
  out->n_hits = h0;
  out->n_locs = l0;
  for (int k = 0; k < kStageCount; ++k) e->stage_ms[k] = st[k];
  e->drain_ms = st[kStageCount];
  if (n >= 1024) {
    e->hits_per_read = 0.5 * e->hits_per_read + 0.5 * (double)h0 / n;
    e->rows_per_read = 0.5 * e->rows_per_read + 0.5 * (double)l0 / n;
  }
  return 0;
}

int run_batched_graph(Engine* e, const void* seqs, const uint64_t* offs, uint32_t n, uint64_t total,
                      uint32_t max_results, DeviceResult* out, std::string* err) {
  cudaStream_t s = e->stream;
  GraphPlan grow;
  const GraphPlan* staged_in = nullptr;  // plan whose own buffers hold the batch
  int pslot = 0;
  if (e->plans)
    for (int i = 0; i < kMaxPlans * kPlanSlots; ++i)
      if (e->plans[i] && seqs == e->plans[i]->seqs && offs == e->plans[i]->offs) {
        staged_in = e->plans[i];
        pslot = i % kPlanSlots;
      }
  // bases already in this device's memory are encoded where they are; host
  // (or other devices') bases are copied into the plan's buffer
  bool in_place = false;
  if (!staged_in && total) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, seqs) == cudaSuccess)
      in_place = at.type == cudaMemoryTypeDevice && at.device == e->device;
    cudaGetLastError();
  }
  // a batch staged in a plan stays in that plan's capacity class (a server may
  // run small batches in a larger class's plan)
  const uint32_t n_plan = staged_in ? std::max<uint32_t>(n, staged_in->n_cap) : n;
  for (int attempt = 0; attempt < 8; ++attempt) {
    GraphPlan* g = graph_plan_for(e, n_plan, total, attempt ? &grow : nullptr, staged_in != nullptr, err, pslot);
    if (!g) return -1;
    if (staged_in) {  // follow the batch into a replacement plan
      seqs = g->seqs;
      offs = g->offs;
      staged_in = g;
    }
    if (total && seqs != g->seqs && !in_place)
      HPG_CUDA(cudaMemcpyAsync(g->seqs, seqs, total, cudaMemcpyDefault, s), "reads");
    if (offs != g->offs)
      HPG_CUDA(cudaMemcpyAsync(g->offs, offs, ((size_t)n + 1) * 8, cudaMemcpyDefault, s), "read offsets");
    if (graph_launch(e, g, n, max_results, err, in_place ? seqs : nullptr, total) != 0) return -1;
    const int rc = graph_collect(e, g, n, &grow, out, err);
    if (rc < 0) return -1;
    if (rc == 0) return 0;
  }
  *err = "batched search pools kept overflowing";
  return -1;
}

}  // namespace hpgbwt
