// serve.cu -- the serving form: a request loop with continuous batching over
// the graph-replayed batched pipeline.
//
// Clients submit read sets of any size (up to the batch capacity) at any
// time.  One worker thread owns the index's stream.  Each iteration it admits,
// in arrival order, every waiting request that fits the batch's read, base and
// HBM budgets (frontier pools and hit lists estimated from the hit and row
// rates of earlier batches), stages them side by side in the capacity plan's
// device buffers (one copy per request straight from the client's memory), and
// replays the captured pipeline once for all of them: the requests' reads share
// the persistent search and locate kernels.  Two batches are in flight, in the
// two plans of their capacity class: while one replays on the index's stream,
// the next one's reads go in on a copy stream and the previous one's results,
// rebased to each request's own read and hit numbering on the device, come out
// on another, so the replays run back to back.  Results land in pinned host
// buffers, which clients read in place until they release the request.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine_internal.hpp"
#include "serve.hpp"

namespace hpgbwt {

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Per batch: segment s holds the reads [seg_read0[s], seg_read0[s+1]).  Hit
// read ids and located-row hit ids become segment-relative; bounds[2s] and
// bounds[2s+1] get the first hit and first row of each segment (s = n_seg is
// the end).  With a summary (the replay's device summary: status, -, hits,
// rows) the counts are read from it, n_hits and n_locs being their caps, and
// a batch whose pools overflowed is left alone (it runs again and is rebased
// after its rerun); so the kernel can follow the replay in stream order.
__global__ void serve_rebase_kernel(hpg_hit_t* __restrict__ hits, uint64_t n_hits, hpg_loc_t* __restrict__ locs,
                                    uint64_t n_locs, const uint64_t* __restrict__ hit_off,
                                    const uint64_t* __restrict__ loc_off, const uint32_t* __restrict__ seg_read0,
                                    uint32_t n_seg, uint64_t* __restrict__ bounds,
                                    const uint64_t* __restrict__ summary) {
  if (summary) {
    if ((uint32_t)summary[0] != 0) return;
    n_hits = min(summary[2], n_hits);
    n_locs = min(summary[3], n_locs);
  }
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t s = tid; s <= n_seg; s += stride) {
    const uint64_t h0 = hit_off[2ull * seg_read0[s]];
    bounds[2 * s] = h0;
    bounds[2 * s + 1] = loc_off[h0];
  }
  for (uint64_t i = tid; i < n_hits; i += stride) {
    const uint32_t r = hits[i].read;
    uint32_t lo = 0, hi = n_seg;  // last segment starting at or before r
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (seg_read0[mid] <= r) lo = mid;
      else hi = mid;
    }
    hits[i].read = r - seg_read0[lo];
  }
  for (uint64_t j = tid; j < n_locs; j += stride) {
    const uint64_t h = locs[j].hit;
    uint32_t lo = 0, hi = n_seg;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (hit_off[2ull * seg_read0[mid]] <= h) lo = mid;
      else hi = mid;
    }
    locs[j].hit = (uint32_t)(h - hit_off[2ull * seg_read0[lo]]);
  }
}

struct ServeReq {
  uint64_t ticket = 0;
  const char* seqs = nullptr;  // client memory, read when the request's batch is staged
  const uint64_t* offs = nullptr;
  uint32_t n = 0;
  uint64_t bases = 0;
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 in a batch, 2 done, 3 failed
  std::string err;
  int set = -1;
  uint64_t hit0 = 0, nh = 0, loc0 = 0, nl = 0, read0 = 0;
};

// Pinned host buffers one batch's results land in; requests point into them.
struct ResultBuf {
  hpg_hit_t* hits = nullptr;
  size_t hits_cap = 0;
  hpg_loc_t* locs = nullptr;
  size_t locs_cap = 0;
  uint32_t* cnt = nullptr;
  uint8_t* trunc = nullptr;
  size_t rs_cap = 0;
  uint64_t* bounds = nullptr;
  size_t seg_cap = 0;
  int refs = 0;
  cudaEvent_t done = nullptr;
};

struct Batch {
  std::vector<ServeReq*> reqs;
  uint32_t n = 0;
  uint64_t bases = 0;
  int slot = 0;  // staging slot of its offsets and segment table
  GraphPlan* g = nullptr;
  ResultBuf* rb = nullptr;  // result set its copies go to, once they are queued
  double t_launch = 0;
};

constexpr int kSets = 3;

template <typename T>
bool pinned_grow(T** p, size_t* cap, size_t want) {
  if (want <= *cap) return true;
  const size_t n = std::max(want, *cap + *cap / 2);
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaHostAlloc(reinterpret_cast<void**>(p), n * sizeof(T) + 64, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return false;
  }
  *cap = n;
  return true;
}

}  // namespace

struct Server {
  Engine* e = nullptr;
  size_t max_reads = 0;
  uint64_t max_bases = 0;
  uint64_t budget = 0;
  uint32_t max_results = 0;
  size_t max_segs = 4096;
  uint32_t floor_n = 4096;  // smallest capacity class a batch runs in (plans captured at start)

  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_sets;
  std::deque<ServeReq*> queue;
  std::unordered_map<uint64_t, ServeReq*> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;

  ResultBuf sets[kSets];
  int next_set = 0;
  uint64_t* h_offs[2] = {nullptr, nullptr};
  uint32_t* h_seg[2] = {nullptr, nullptr};
  uint32_t* d_seg[2] = {nullptr, nullptr};
  uint64_t* d_bounds[2] = {nullptr, nullptr};
  uint32_t* h_err = nullptr;  // pinned copy of the index's error word, per slot
  // per pipeline slot: inputs sent, replay done, results out
  cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_run[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
  // time split, printed when the server is freed if HPG_BWT_TIMING is set: replay device
  // time (events around each replay), host time blocked on replays and on result copies
  bool timing = std::getenv("HPG_BWT_TIMING") != nullptr;
  cudaEvent_t tv0[2] = {nullptr, nullptr}, tv1[2] = {nullptr, nullptr};
  double t_replay = 0, t_wait_run = 0, t_wait_out = 0, t_issue = 0, t_plan = 0, t_prep = 0, t_copies = 0,
         t_take = 0, t_publish = 0, t_form = 0;
  // the longest single instance of each, the replay's and the host's parts
  double m_replay = 0, m_wait_run = 0, m_wait_out = 0, m_plan = 0, m_take = 0, m_cycle = 0, last_cycle = 0;
  static void note(double& sum, double& mx, double v) {
    sum += v;
    mx = v > mx ? v : mx;
  }

  // admission estimates, updated from finished batches
  double hits_per_read = 4.0, rows_per_read = 16.0;

  // statistics
  uint64_t batches = 0, requests = 0, reads = 0, regrows = 0, max_batch_reads = 0, max_batch_reqs = 0;
  uint64_t plan_bytes = 0;
  double gpu_ms = 0;
  std::string fatal;

  // HBM bytes a batch of n reads and `bases` bases is expected to hold.
  double est_bytes(uint64_t n, uint64_t bases) const {
    const double per_read = 9.0 + 2 * 25.0 + hits_per_read * 1.25 * (2 * 24 + 32 + 4 + 8) +
                            rows_per_read * 1.25 * (16 + 32) + 4.0;
    return 2.0 * (double)bases + per_read * (double)n;
  }

  // Take waiting requests in arrival order while they fit (called with mu held).
  void form(Batch* b) {
    b->reqs.clear();
    b->n = 0;
    b->bases = 0;
    double bytes = 0;
    while (!queue.empty() && b->reqs.size() < max_segs) {
      ServeReq* q = queue.front();
      const double add = est_bytes(q->n, q->bases);
      if (!b->reqs.empty() && ((size_t)b->n + q->n > max_reads || b->bases + q->bases > max_bases ||
                               bytes + add > (double)budget))
        break;
      queue.pop_front();
      q->state = 1;
      b->reqs.push_back(q);
      b->n += q->n;
      b->bases += q->bases;
      bytes += add;
    }
  }

  // Offsets and segment table of a batch into its pinned staging slot.
  void prepare(Batch* b) {
    uint64_t* o = h_offs[b->slot];
    uint32_t* sg = h_seg[b->slot];
    uint64_t base = 0;
    uint32_t r = 0;
    for (size_t s = 0; s < b->reqs.size(); ++s) {
      const ServeReq* q = b->reqs[s];
      sg[s] = r;
      const uint64_t o0 = q->offs[0];
      for (uint32_t i = 0; i < q->n; ++i) o[r + i] = base + (q->offs[i] - o0);
      r += q->n;
      base += q->bases;
    }
    o[r] = base;
    sg[b->reqs.size()] = r;
  }

  // Send a batch's reads, offsets and segment table on the input stream and
  // queue its replay behind them, in the batch's pipeline slot.
  int issue(Batch* b, std::string* err) {
    cudaStream_t cs = e->stream, h2d = e->xs[0];
    const int k = b->slot;
    const double p0 = now_ms();
    b->g = graph_plan_for(e, std::max<uint32_t>(b->n, floor_n), b->bases, nullptr, false, err, k);
    if (!b->g) return -1;
    HPG_CUDA(cudaEventSynchronize(ev_in[k]), "serving staging");  // the slot's previous tables were sent
    const double p1 = now_ms();
    prepare(b);
    const double p2 = now_ms();
    if (timing) {
      note(t_plan, m_plan, p1 - p0);
      t_prep += p2 - p1;
    }
    // inputs once the slot's previous replay has read its own, the segment table once
    // the slot's previous rebase has read it
    HPG_CUDA(cudaStreamWaitEvent(h2d, ev_run[k], 0), "serving order");
    uint64_t at = 0;
    for (const ServeReq* q : b->reqs) {
      if (q->bases)
        HPG_CUDA(cudaMemcpyAsync(b->g->seqs + at, q->seqs + q->offs[0], q->bases, cudaMemcpyDefault, h2d),
                 "stage reads");
      at += q->bases;
    }
    HPG_CUDA(cudaMemcpyAsync(b->g->offs, h_offs[k], ((size_t)b->n + 1) * 8, cudaMemcpyHostToDevice, h2d),
             "stage offsets");
    HPG_CUDA(cudaStreamWaitEvent(h2d, ev_out[k], 0), "serving order");
    HPG_CUDA(cudaMemcpyAsync(d_seg[k], h_seg[k], (b->reqs.size() + 1) * 4, cudaMemcpyHostToDevice, h2d),
             "segments");
    HPG_CUDA(cudaEventRecord(ev_in[k], h2d), "serving order");
    if (timing) t_copies += now_ms() - p2;
    // the replay once its inputs are in and the slot's previous results are out
    HPG_CUDA(cudaStreamWaitEvent(cs, ev_in[k], 0), "serving order");
    HPG_CUDA(cudaStreamWaitEvent(cs, ev_out[k], 0), "serving order");
    b->t_launch = now_ms();
    if (timing) cudaEventRecord(tv0[k], cs);
    if (graph_launch(e, b->g, b->n, max_results, err) != 0) return -1;
    // the rebase follows the replay on its stream: no wait for SMs that the next
    // replay's persistent kernels hold, and the copies out need only this event
    GraphPlan* g = b->g;
    count_launches(1);
    serve_rebase_kernel<<<e->num_sms * 2, 256, 0, cs>>>(g->hits, g->res_cap, g->locs, g->skip_locate ? 0 : g->locs_cap,
                                                       g->hit_off, g->loc_off, d_seg[k], (uint32_t)b->reqs.size(),
                                                       d_bounds[k], g->summary_d);
    if (timing) cudaEventRecord(tv1[k], cs);
    HPG_CUDA(cudaEventRecord(ev_run[k], cs), "serving order");
    if (timing) t_issue += now_ms() - b->t_launch;
    return 0;
  }

  ResultBuf* take_set(size_t hits, size_t locs, size_t rs, size_t segs, std::string* err) {
    int pick = -1;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_sets.wait(lk, [&] {
        for (int k = 0; k < kSets; ++k)
          if (sets[(next_set + k) % kSets].refs == 0) return true;
        return false;
      });
      for (int k = 0; k < kSets && pick < 0; ++k)
        if (sets[(next_set + k) % kSets].refs == 0) pick = (next_set + k) % kSets;
      next_set = (pick + 1) % kSets;
    }
    ResultBuf& rb = sets[pick];
    if (!pinned_grow(&rb.hits, &rb.hits_cap, hits + 1) || !pinned_grow(&rb.locs, &rb.locs_cap, locs + 1) ||
        !pinned_grow(&rb.bounds, &rb.seg_cap, 2 * segs + 2)) {
      *err = "out of pinned host memory (serving results)";
      return nullptr;
    }
    if (rs > rb.rs_cap) {
      size_t c1 = rb.rs_cap, c2 = rb.rs_cap;
      if (!pinned_grow(&rb.cnt, &c1, rs + 1) || !pinned_grow(&rb.trunc, &c2, rs + 1)) {
        *err = "out of pinned host memory (serving results)";
        return nullptr;
      }
      rb.rs_cap = std::min(c1, c2);
    }
    return &rb;
  }

  void fail(Batch* b, const std::string& why) {
    std::lock_guard<std::mutex> lk(mu);
    for (ServeReq* q : b->reqs) {
      q->state = 3;
      q->err = why;
      q->t_done = now_ms();
    }
    b->reqs.clear();
    cv_done.notify_all();
  }

  // Wait for a batch's replay, then queue its rebase and result copies on the
  // output stream (the other slot's batch keeps the GPU busy meanwhile).  The
  // slot's inputs are free from here on: the next batch of the slot is sent
  // before these results are waited for.
  int collect_start(Batch* b, const GraphPlan* other, std::string* err) {
    cudaStream_t cs = e->stream, h2d = e->xs[0], d2h = e->xs[1];
    const int k = b->slot;
    const double w0 = now_ms();
    HPG_CUDA(cudaEventSynchronize(ev_run[k]), "batched pipeline");
    if (timing) {
      note(t_wait_run, m_wait_run, now_ms() - w0);
      float ms = 0;
      cudaEventElapsedTime(&ms, tv0[k], tv1[k]);
      note(t_replay, m_replay, ms);
    }
    GraphPlan* g = b->g;
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
    const bool rerun = status != 0;
    if (rerun) {  // a pool overflowed: drain the pipeline, grow the pool and run the batch again
      ++regrows;
      HPG_CUDA(cudaStreamSynchronize(h2d), "serving drain");
      HPG_CUDA(cudaStreamSynchronize(d2h), "serving drain");
      HPG_CUDA(cudaStreamSynchronize(cs), "serving drain");
      DeviceResult r;
      if (run_batched_graph(e, g->seqs, g->offs, b->n, b->bases, max_results, &r, err) != 0) return -1;
      g = b->g = graph_plan_for(e, std::max<uint32_t>(b->n, floor_n), b->bases, nullptr, false, err, k);
      if (!g) return -1;
      // the streams are drained: bring the other classes' plans to the rates this
      // overflow showed now, rather than one overflow (and drain) per class
      uint64_t top = 4096;
      while (top < max_reads) top <<= 1;
      if (graph_plans_refresh(e, g, other, top, err) != 0) return -1;
      h = g->h_summary;
      HPG_CUDA(cudaEventRecord(ev_run[k], cs), "serving order");
    }
    gpu_ms += now_ms() - b->t_launch;
    const uint64_t nh = h[2], nl = g->skip_locate ? 0 : h[3];
    const size_t nseg = b->reqs.size();
    const double k0 = now_ms();
    ResultBuf* rb = take_set(nh, nl, 2ull * b->n, nseg, err);
    if (!rb) return -1;
    if (timing) note(t_take, m_take, now_ms() - k0);
    HPG_CUDA(cudaStreamWaitEvent(d2h, ev_run[k], 0), "serving order");
    if (rerun) {  // the rebase that followed the replay left the overflowed batch alone
      const uint64_t work = std::max<uint64_t>(std::max<uint64_t>(nh, nl), nseg + 1);
      const unsigned grid = (unsigned)std::min<uint64_t>((work + 255) / 256, (uint64_t)e->num_sms * 8);
      count_launches(1);
      serve_rebase_kernel<<<grid, 256, 0, d2h>>>(g->hits, nh, g->locs, nl, g->hit_off, g->loc_off, d_seg[k],
                                                 (uint32_t)nseg, d_bounds[k], nullptr);
    }
    if (nh)
      HPG_CUDA(cudaMemcpyAsync(rb->hits, g->hits, nh * sizeof(hpg_hit_t), cudaMemcpyDeviceToHost, d2h), "copy hits");
    if (nl)
      HPG_CUDA(cudaMemcpyAsync(rb->locs, g->locs, nl * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, d2h), "copy rows");
    if (b->n) {
      HPG_CUDA(cudaMemcpyAsync(rb->cnt, g->kept, 2ull * b->n * 4, cudaMemcpyDeviceToHost, d2h), "copy counts");
      HPG_CUDA(cudaMemcpyAsync(rb->trunc, g->trunc, 2ull * b->n, cudaMemcpyDeviceToHost, d2h), "copy flags");
    }
    HPG_CUDA(cudaMemcpyAsync(rb->bounds, d_bounds[k], (nseg + 1) * 16, cudaMemcpyDeviceToHost, d2h),
             "copy bounds");
    HPG_CUDA(cudaMemcpyAsync(h_err + k, e->d_err, 4, cudaMemcpyDeviceToHost, d2h), "error word");
    HPG_CUDA(cudaEventRecord(rb->done, d2h), "result event");
    HPG_CUDA(cudaEventRecord(ev_out[k], d2h), "serving order");
    b->rb = rb;
    return 0;
  }

  // Wait for a batch's result copies and publish them to its requests.
  int collect_finish(Batch* b, std::string* err) {
    const int k = b->slot;
    ResultBuf* rb = b->rb;
    const size_t nseg = b->reqs.size();
    const double w1 = now_ms();
    HPG_CUDA(cudaEventSynchronize(rb->done), "result copies");
    if (timing) note(t_wait_out, m_wait_out, now_ms() - w1);
    HPG_CUDA(cudaGetLastError(), "rebase kernel");
    if (h_err[k]) {
      cudaMemsetAsync(e->d_err, 0, 4, e->xs[1]);
      *err = "corrupt index: suffix-array walk did not reach a sampled row";
      return -1;
    }
    const double t = now_ms();
    std::lock_guard<std::mutex> lk(mu);
    uint32_t read0 = 0;  // the slot's staged segment table may already hold the next batch's
    for (size_t q = 0; q < nseg; ++q) {
      ServeReq* r = b->reqs[q];
      r->set = (int)(rb - sets);
      r->read0 = read0;
      read0 += r->n;
      r->hit0 = rb->bounds[2 * q];
      r->nh = rb->bounds[2 * q + 2] - r->hit0;
      r->loc0 = rb->bounds[2 * q + 1];
      r->nl = rb->bounds[2 * q + 3] - r->loc0;
      r->state = 2;
      r->t_done = t;
      rb->refs++;
    }
    ++batches;
    requests += nseg;
    reads += b->n;
    max_batch_reads = std::max<uint64_t>(max_batch_reads, b->n);
    max_batch_reqs = std::max<uint64_t>(max_batch_reqs, nseg);
    if (b->n >= 1024) {  // smoothed, biased up: admission must not undershoot
      const double hpr = (double)(rb->bounds[2 * nseg] - rb->bounds[0]) / b->n,
                   rpr = (double)(rb->bounds[2 * nseg + 1] - rb->bounds[1]) / b->n;
      hits_per_read = std::max(hpr, 0.8 * hits_per_read + 0.2 * hpr);
      rows_per_read = std::max(rpr, 0.8 * rows_per_read + 0.2 * rpr);
    }
    plan_bytes = 0;
    for (int i = 0; i < 66; ++i)
      if (e->plans && e->plans[i]) plan_bytes += e->plans[i]->bytes;
    b->reqs.clear();
    cv_done.notify_all();
    if (timing) {
      t_publish += now_ms() - t;
      const double c = now_ms();  // one batch published to the next
      if (last_cycle > 0) m_cycle = std::max(m_cycle, c - last_cycle);
      last_cycle = c;
    }
    return 0;
  }

  void run() {
    cudaSetDevice(e->device);
    // two batches replaying or queued, plus one whose results are being copied out;
    // batches finish in the order they were issued, so a batch object comes back
    // into use three issues later, after it was published
    Batch batch[3];
    std::deque<Batch*> inflight;
    int slot = 0, next_obj = 0;
    auto fill = [&](bool may_wait) {  // keep two batches in flight while requests wait
      while (inflight.size() < 2) {
        Batch* b = &batch[next_obj];
        {
          std::unique_lock<std::mutex> lk(mu);
          if (may_wait && inflight.empty()) cv_work.wait(lk, [&] { return stop || !queue.empty(); });
          if (queue.empty()) return;
          b->slot = slot;
          const double f0 = now_ms();
          form(b);
          if (timing) t_form += now_ms() - f0;
        }
        if (b->reqs.empty()) return;
        next_obj = (next_obj + 1) % 3;
        std::string err;
        if (issue(b, &err) != 0) {
          fail(b, err);
          continue;
        }
        inflight.push_back(b);
        slot ^= 1;
      }
    };
    for (;;) {
      fill(true);
      if (inflight.empty()) {
        std::lock_guard<std::mutex> lk(mu);
        if (stop && queue.empty()) return;  // stopping with nothing left
        continue;
      }
      Batch* b = inflight.front();
      inflight.pop_front();
      std::string err;
      int rc = collect_start(b, inflight.empty() ? nullptr : inflight.front()->g, &err);
      if (rc == 0) {
        fill(false);  // the freed slot's next inputs travel while its results come out
        rc = collect_finish(b, &err);
      }
      if (rc != 0) {
        fail(b, err);
        std::lock_guard<std::mutex> lk(mu);
        fatal = err;
      }
    }
  }
};

Server* server_create(Engine* e, size_t max_batch_reads, uint64_t max_batch_bases, uint64_t hbm_budget,
                      uint32_t max_results, std::string* err) {
  if (max_batch_reads == 0 || max_batch_reads >= (1ull << 30)) {
    *err = "batch capacity must be 1 .. 2^30-1 reads";
    return nullptr;
  }
  if (cudaSetDevice(e->device) != cudaSuccess) {
    *err = "cudaSetDevice failed";
    return nullptr;
  }
  Server* S = new Server();
  S->e = e;
  S->max_reads = max_batch_reads;
  S->max_bases = max_batch_bases ? max_batch_bases : (uint64_t)max_batch_reads * 320;
  S->max_results = max_results;
  if (hbm_budget == 0) {  // a quarter of what is free now
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    hbm_budget = fr / 4;
  }
  S->budget = hbm_budget;
  bool ok = true;
  for (int k = 0; k < 2 && ok; ++k) {
    ok = cudaHostAlloc(reinterpret_cast<void**>(&S->h_offs[k]), (max_batch_reads + 1) * 8, 0) == cudaSuccess &&
         cudaHostAlloc(reinterpret_cast<void**>(&S->h_seg[k]), (S->max_segs + 1) * 4, 0) == cudaSuccess;
  }
  for (int k = 0; k < 2 && ok; ++k)
    ok = cudaMalloc(&S->d_seg[k], (S->max_segs + 1) * 4) == cudaSuccess &&
         cudaMalloc(&S->d_bounds[k], (S->max_segs + 1) * 16) == cudaSuccess &&
         cudaEventCreateWithFlags(&S->ev_in[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&S->ev_run[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&S->ev_out[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreate(&S->tv0[k]) == cudaSuccess && cudaEventCreate(&S->tv1[k]) == cudaSuccess;
  ok = ok && cudaHostAlloc(reinterpret_cast<void**>(&S->h_err), 16, 0) == cudaSuccess;
  if (ok && !e->xs[0])
    ok = cudaStreamCreateWithFlags(&e->xs[0], cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&e->xs[1], cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; k < kSets && ok; ++k) ok = cudaEventCreateWithFlags(&S->sets[k].done, cudaEventDisableTiming) ==
                                            cudaSuccess;
  // result sets sized for two hits and two located rows per read of a full batch up
  // front (they grow past that when a batch needs it), so that pinning host memory
  // stays out of the first batches' latency
  for (int k = 0; k < kSets && ok; ++k) {
    ResultBuf& rb = S->sets[k];
    size_t c1 = 0, c2 = 0;
    ok = pinned_grow(&rb.hits, &rb.hits_cap, 2 * max_batch_reads + 1) &&
         pinned_grow(&rb.locs, &rb.locs_cap, 2 * max_batch_reads + 1) &&
         pinned_grow(&rb.bounds, &rb.seg_cap, 2 * S->max_segs + 2) &&
         pinned_grow(&rb.cnt, &c1, 2 * max_batch_reads + 1) && pinned_grow(&rb.trunc, &c2, 2 * max_batch_reads + 1);
    rb.rs_cap = std::min(c1, c2);
  }
  if (!ok) {
    cudaGetLastError();
    *err = "out of memory (serving buffers)";
    server_destroy(S);
    return nullptr;
  }
  // the graph plans of every capacity class a batch can run in, both slots,
  // captured now: a capture (allocations that wait for the device, then the
  // capture itself) in the middle of serving stalled the pipeline for tens of
  // ms.  Batches below 1/64 of the capacity run in that smallest class.
  {
    // the index's batch-call workspaces and larger plans go first (a device
    // result of an earlier call on the index is valid until the next call)
    uint64_t top = 4096;
    while (top < max_batch_reads) top <<= 1;
    engine_release_workspace(e, top);
    uint64_t cls = 4096;
    while (cls < max_batch_reads / 64) cls <<= 1;
    S->floor_n = (uint32_t)cls;
    const uint64_t bases_per_read = std::max<uint64_t>(1, S->max_bases / max_batch_reads);
    for (;; cls <<= 1) {
      for (int k = 0; k < 2; ++k) {
        std::string perr;
        if (!graph_plan_for(e, (uint32_t)cls, std::min<uint64_t>(cls * bases_per_read, S->max_bases), nullptr, false,
                            &perr, k)) {
          *err = "serving plans: " + perr;
          server_destroy(S);
          return nullptr;
        }
      }
      if (cls >= max_batch_reads) break;
    }
  }
  S->worker = std::thread([S] { S->run(); });
  return S;
}

void server_destroy(Server* S) {
  if (!S) return;
  if (S->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
    }
    S->cv_work.notify_all();
    S->worker.join();
  }
  cudaStreamSynchronize(S->e->stream);
  for (cudaStream_t x : S->e->xs)
    if (x) cudaStreamSynchronize(x);
  if (S->timing && S->batches)
    std::fprintf(stderr,
                 "[hpgbwt] server: %llu batches, %.0f reads per batch; per batch: replay %.3f ms on the device, "
                 "host blocked %.3f ms on replays and %.3f ms on result copies; host work: form %.3f, plan %.3f, "
                 "tables %.3f, copy calls %.3f, launch %.3f, result set %.3f, publish %.3f ms\n",
                 (unsigned long long)S->batches, (double)S->reads / S->batches, S->t_replay / S->batches,
                 S->t_wait_run / S->batches, S->t_wait_out / S->batches, S->t_form / S->batches,
                 S->t_plan / S->batches, S->t_prep / S->batches, S->t_copies / S->batches, S->t_issue / S->batches,
                 S->t_take / S->batches, S->t_publish / S->batches);
  if (S->timing && S->batches)
    std::fprintf(stderr,
                 "[hpgbwt] server: longest: replay %.3f ms, host blocked on a replay %.3f and on result copies %.3f, "
                 "plan %.3f, result set %.3f; publish to publish %.3f ms\n",
                 S->m_replay, S->m_wait_run, S->m_wait_out, S->m_plan, S->m_take, S->m_cycle);
  for (ResultBuf& rb : S->sets) {
    cudaFreeHost(rb.hits);
    cudaFreeHost(rb.locs);
    cudaFreeHost(rb.cnt);
    cudaFreeHost(rb.trunc);
    cudaFreeHost(rb.bounds);
    if (rb.done) cudaEventDestroy(rb.done);
  }
  for (int k = 0; k < 2; ++k) {
    cudaFreeHost(S->h_offs[k]);
    cudaFreeHost(S->h_seg[k]);
  }
  for (int k = 0; k < 2; ++k) {
    cudaFree(S->d_seg[k]);
    cudaFree(S->d_bounds[k]);
    if (S->ev_in[k]) cudaEventDestroy(S->ev_in[k]);
    if (S->ev_run[k]) cudaEventDestroy(S->ev_run[k]);
    if (S->ev_out[k]) cudaEventDestroy(S->ev_out[k]);
    if (S->tv0[k]) cudaEventDestroy(S->tv0[k]);
    if (S->tv1[k]) cudaEventDestroy(S->tv1[k]);
  }
  if (S->h_err) cudaFreeHost(S->h_err);
  for (auto& kv : S->reqs) delete kv.second;
  delete S;
}

int server_submit(Server* S, const char* seqs, const uint64_t* offs, size_t n, uint64_t* ticket, std::string* err) {
  if (n > S->max_reads) {
    *err = "request has more reads than the batch capacity";
    return -1;
  }
  if (n && (!seqs || !offs)) {
    *err = "null reads";
    return -1;
  }
  for (size_t i = 0; i < n; ++i) {
    if (offs[i + 1] < offs[i] || offs[i + 1] - offs[i] > 32767) {
      *err = "read offsets must be non-decreasing and reads at most 32767 bases";
      return -1;
    }
  }
  const uint64_t bases = n ? offs[n] - offs[0] : 0;
  if (bases > S->max_bases) {
    *err = "request has more bases than the batch capacity";
    return -1;
  }
  ServeReq* q = new ServeReq();
  static const uint64_t zero = 0;
  q->seqs = seqs;
  q->offs = n ? offs : &zero;
  q->n = (uint32_t)n;
  q->bases = bases;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      delete q;
      *err = "server is stopping";
      return -1;
    }
    q->ticket = S->next_ticket++;
    q->t_submit = now_ms();
    S->reqs[q->ticket] = q;
    S->queue.push_back(q);
  }
  S->cv_work.notify_one();
  *ticket = q->ticket;
  return 0;
}

int server_wait(Server* S, uint64_t ticket, hpg_result_set_t* view, double* latency_ms, int timeout_ms,
                std::string* err) {
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) {
    *err = "unknown or released ticket";
    return -1;
  }
  ServeReq* q = it->second;
  auto done = [&] { return q->state >= 2; };
  if (timeout_ms < 0) {
    S->cv_done.wait(lk, done);
  } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    return 1;
  }
  if (q->state == 3) {
    *err = q->err;
    return -1;
  }
  const ResultBuf& rb = S->sets[q->set];
  if (view) {
    view->n_reads = q->n;
    view->n_hits = q->nh;
    view->hits = rb.hits + q->hit0;
    view->n_locs = q->nl;
    view->locs = rb.locs + q->loc0;
    view->rs_count = rb.cnt + 2 * q->read0;
    view->rs_truncated = rb.trunc + 2 * q->read0;
  }
  if (latency_ms) *latency_ms = q->t_done - q->t_submit;
  return 0;
}

int server_release(Server* S, uint64_t ticket, std::string* err) {
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) {
    *err = "unknown or released ticket";
    return -1;
  }
  ServeReq* q = it->second;
  if (q->state < 2) {
    *err = "request still in flight";
    return -1;
  }
  if (q->state == 2) S->sets[q->set].refs--;
  S->reqs.erase(it);
  delete q;
  S->cv_sets.notify_all();
  return 0;
}

void server_stats(Server* S, double* out, int n) {
  std::lock_guard<std::mutex> lk(S->mu);
  const uint64_t plan_bytes = S->plan_bytes;
  const double v[] = {(double)S->batches,
                      (double)S->requests,
                      (double)S->reads,
                      S->batches ? (double)S->reads / S->batches : 0.0,
                      S->gpu_ms,
                      (double)S->regrows,
                      (double)plan_bytes,
                      (double)S->budget,
                      (double)S->max_batch_reads,
                      (double)S->max_batch_reqs,
                      (double)S->queue.size(),
                      S->hits_per_read,
                      S->rows_per_read};
  for (int i = 0; i < n && i < (int)(sizeof(v) / sizeof(v[0])); ++i) out[i] = v[i];
}

}  // namespace hpgbwt
