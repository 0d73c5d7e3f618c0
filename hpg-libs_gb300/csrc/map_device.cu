// map_device.cu -- device passes of the alignment-list layer (map_api.cpp):
// the exact search pair of bwt_map_exact_seq, the vector-search endpoints the
// anchor lists start from, and locating caller-chosen SA rows.
#include <cuda_runtime.h>

#include <vector>

#include "engine_internal.hpp"

namespace hpgbwt {

namespace {

// bwt_map_exact_seq (bwt.c:919-940): '+' BWExactSearchBackward over backward
// from the last base, '-' BWExactSearchForward over forward_rev from the
// first, both from the full interval; the interval where the search stopped
// (k = l + 1 when a base failed), as the reference's result keeps it.
__global__ void exact_api_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                 const uint8_t* __restrict__ ok, uint32_t n, uint4* __restrict__ out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint64_t b = offs[r];
  const int len = (int)(offs[r + 1] - b);
  uint4 o = make_uint4(1, 0, 1, 0);  // reads outside the alphabet: nothing to locate
  if (ok[r] && len >= 0 && len <= 32767) {
    const uint8_t* W = codes + b;
    uint32_t k = 0, l = X.top;
    for (int i = len - 1; i >= 0; --i) {
      bw_step(X, View{0, 0}, W[i], k, l);
      if (k > l) break;
    }
    o.x = k;
    o.y = l;
    k = 0;
    l = X.top;
    for (int i = 0; i < len; ++i) {
      bw_step(X, View{1, 1}, W[i], k, l);
      if (k > l) break;
    }
    o.z = k;
    o.w = l;
  }
  out[r] = o;
}

// The four vector searches of bwt.c:1940-1950, reduced to what the anchor
// lists use (bwt.c:2249-2271): good steps and the last good interval of each.
//   c 0: backward over backward ('+' BACKWARD)   c 1: forward over forward ('+' FORWARD)
//   c 2: forward over backward_rev ('-' BACKWARD) c 3: backward over forward_rev ('-' FORWARD)
__global__ void anchor_scan_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                   const uint8_t* __restrict__ ok, const uint32_t* __restrict__ reads, uint32_t m,
                                   uint4* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * m) return;
  const uint32_t r = reads[t >> 2], c = t & 3u;
  const uint64_t b = offs[r];
  const int len = (int)(offs[r + 1] - b);
  uint4 o = make_uint4(0, 1, 0, 0);  // no good step: no interval
  if (ok[r] && len > 0 && len <= 32767) {
    const uint8_t* W = codes + b;
    const View v = c == 0 ? View{0, 0} : c == 1 ? View{1, 0} : c == 2 ? View{0, 1} : View{1, 1};
    const bool backward = (c == 0 || c == 3);
    uint32_t k = 0, l = X.top, nt = 0, gk = 1, gl = 0;
    for (int s = 0; s < len; ++s) {
      bw_step(X, v, W[backward ? len - 1 - s : s], k, l);
      if (k > l) break;
      ++nt;
      gk = k;
      gl = l;
    }
    o = make_uint4(nt, gk, gl, 0);
  }
  out[t] = o;
}

// bwt_map_exact_seed (bwt.c:1232-1252): the seed W[first .. last] of a read,
// '+' BWExactSearchBackward over backward from `last`, '-' BWExactSearchForward
// over backward_rev (the backward index with complemented symbols) from
// `first`, both from the full interval; the interval where the search stopped.
__global__ void seed_search_kernel(DevIndex X, const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs,
                                   const uint8_t* __restrict__ ok, const uint4* __restrict__ seeds, uint32_t m,
                                   uint4* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const uint4 sd = seeds[t];
  const uint64_t b = offs[sd.x];
  const uint64_t len = offs[sd.x + 1] - b;
  uint4 o = make_uint4(1, 0, 1, 0);  // nothing to locate
  if (ok[sd.x] && sd.y <= sd.z && sd.z < len) {
    const uint8_t* W = codes + b;
    uint32_t k = 0, l = X.top;
    for (int64_t i = sd.z; i >= (int64_t)sd.y; --i) {
      bw_step(X, View{0, 0}, W[i], k, l);
      if (k > l) break;
    }
    o.x = k;
    o.y = l;
    k = 0;
    l = X.top;
    for (uint32_t i = sd.y; i <= sd.z; ++i) {
      bw_step(X, View{0, 1}, W[i], k, l);
      if (k > l) break;
    }
    o.z = k;
    o.w = l;
  }
  out[t] = o;
}

// ---- bwt_map_inexact_read's records (bwt.c:1978-2289) on the device ----

// Per read: the exact hits the reference locates.  Rows are counted as l - k
// over '+' then '-' (bwt.c:1978, 2148-2149); the strand whose count passes
// filter_read_mappings loses its alignments and the read gets flag 2.
// pflag: bit 0 the '+' strand passed the filter, bit 1 the '-' strand.
__global__ void inexact_plan_kernel(const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ hit_off,
                                    uint32_t n, uint64_t filter, uint32_t* __restrict__ rows,
                                    uint8_t* __restrict__ pflag) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  uint64_t tot = 0, rt[2] = {0, 0};
  uint8_t ex = 0;
  for (int type = 1; type >= 0 && !ex; --type) {
    const uint64_t t = 2ull * g + (type ? 0 : 1);
    for (uint64_t h = hit_off[t]; h < hit_off[t + 1]; ++h) {
      const hpg_hit_t x = hits[h];
      if (x.nm) continue;
      tot += (uint64_t)(x.l - x.k);
      if (tot > filter) {
        ex = type ? 1 : 2;
        rt[type] = 0;
        break;
      }
      rt[type] += (uint64_t)(x.l - x.k) + 1;
    }
  }
  const uint64_t r = rt[0] + rt[1];
  rows[g] = r > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)r;
  pflag[g] = ex | (r > 0xFFFFFFFFull ? 4 : 0);
}

// Per read: one locate item per SA row of every planned hit ('+' hits first, in
// list order), physical direction = result direction, flipped on the '-' strand.
__global__ void inexact_rows_kernel(const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ hit_off,
                                    const uint64_t* __restrict__ read_offs, const uint64_t* __restrict__ row_off,
                                    const uint8_t* __restrict__ pflag, uint32_t n, RowItem* __restrict__ items) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const uint32_t len = (uint32_t)(read_offs[g + 1] - read_offs[g]);
  uint64_t at = row_off[g];
  const uint8_t ex = pflag[g];
  for (int type = 1; type >= 0; --type) {
    if (ex & (type ? 1 : 2)) break;
    const uint64_t t = 2ull * g + (type ? 0 : 1);
    for (uint64_t h = hit_off[t]; h < hit_off[t + 1]; ++h) {
      const hpg_hit_t x = hits[h];
      if (x.nm) continue;
      const uint32_t phys = (uint32_t)x.dir ^ (uint32_t)(type ? 0 : 1);
      for (int64_t j = x.k; j <= x.l; ++j, ++at)
        items[at] = RowItem{(uint32_t)j, g, (uint32_t)at, (phys << 31) | (len & kRowLenMask)};
    }
  }
}

// Per read: the alignments in the reference's list order.  Per strand, the
// valid located rows in row order are the candidates; a candidate within 10 bp
// of an earlier candidate on its chromosome is merged away (all have the one
// cigar operation of an exact match, bwt.c:2190-2221); the survivors are taken
// from the back (bwt.c:2223-2235).  rec: chromosome | strand << 31, position.
// flags: bit 0 flag 2 (a strand passed the filter), bit 1 a candidate that
// would have been the list's primary alignment was merged away.
__global__ void inexact_records_kernel(const hpg_hit_t* __restrict__ hits, const uint64_t* __restrict__ hit_off,
                                       const uint64_t* __restrict__ row_off, const uint8_t* __restrict__ pflag,
                                       const hpg_loc_t* __restrict__ locs, uint32_t n, MapRec* __restrict__ rec,
                                       uint32_t* __restrict__ n_rec, uint8_t* __restrict__ flags) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const uint64_t base = row_off[g];
  uint64_t at = base, out = base;
  uint32_t num = 0;
  uint8_t fl = 0;
  const uint8_t ex = pflag[g];
  for (int type = 1; type >= 0; --type) {
    if (ex & (type ? 1 : 2)) {
      fl |= 1;
      break;
    }
    const uint64_t t = 2ull * g + (type ? 0 : 1);
    uint64_t nr = 0;
    for (uint64_t h = hit_off[t]; h < hit_off[t + 1]; ++h) {
      const hpg_hit_t x = hits[h];
      if (!x.nm) nr += (uint64_t)(x.l - x.k) + 1;
    }
    const uint32_t before = num;
    for (uint64_t a = nr; a-- > 0;) {
      const hpg_loc_t& q = locs[at + a];
      if (!q.valid) continue;
      const int pos = (int)q.position;
      bool merged = false;
      for (uint64_t b = 0; b < a && !merged; ++b) {
        const hpg_loc_t& o = locs[at + b];
        merged = o.valid && o.chrom == q.chrom && abs(pos - (int)o.position) < 10;
      }
      if (merged) {
        if (before == 0) fl |= 2;
        continue;
      }
      rec[out++] = MapRec{q.chrom | ((uint32_t)(type ? 0 : 1) << 31), pos};
      ++num;
    }
    at += nr;
  }
  n_rec[g] = num;
  flags[g] = fl;
}

}  // namespace


int upload_reads(Engine* e, const char* seqs, const uint64_t* offs, size_t n, std::string* err) {
  cudaStream_t s = e->stream;
  const uint64_t total = n ? offs[n] - offs[0] : 0;
  if (!ensure(e, e->seqs, total + 16) || !ensure(e, e->offs, (n + 1) * 8) || !ensure(e, e->codes, total + 16) ||
      !ensure(e, e->ok, n + 16)) {
    *err = "out of device memory (reads)";
    return -1;
  }
  std::vector<uint64_t> rel(n + 1);
  for (size_t i = 0; i <= n; ++i) rel[i] = n ? offs[i] - offs[0] : 0;
  if (total) HPG_CUDA(cudaMemcpyAsync(e->seqs.p, seqs + offs[0], total, cudaMemcpyHostToDevice, s), "upload reads");
  HPG_CUDA(cudaMemcpyAsync(e->offs.p, rel.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s), "upload offsets");
  launch_encode(ptr<uint8_t>(e->seqs), total, ptr<uint64_t>(e->offs), (uint32_t)n, e->d_table, ptr<uint8_t>(e->codes),
                ptr<uint8_t>(e->ok), s);
  HPG_CUDA(cudaStreamSynchronize(s), "encode");  // `rel` is pageable and local
  return 0;
}

namespace {

int check_walk(Engine* e, std::string* err) {
  uint32_t derr = 0;
  HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
  if (derr) {
    cudaMemset(e->d_err, 0, 4);
    *err = "corrupt index: suffix-array walk did not reach a sampled row";
    return -1;
  }
  return 0;
}

}  // namespace

int engine_exact_api(Engine* e, const char* seqs, const uint64_t* offs, size_t n, uint32_t* kl, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (n >= (1ull << 31)) {
    *err = "too many reads in one batch";
    return -1;
  }
  if (!n) return 0;
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, n * sizeof(uint4) + 16)) {
    *err = "out of device memory (exact intervals)";
    return -1;
  }
  cudaStream_t s = e->stream;
  count_launches(1);
  exact_api_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes), ptr<uint64_t>(e->offs),
                                                                ptr<uint8_t>(e->ok), (uint32_t)n, ptr<uint4>(e->slots));
  HPG_CUDA(cudaMemcpyAsync(kl, e->slots.p, n * sizeof(uint4), cudaMemcpyDeviceToHost, s), "exact intervals");
  HPG_CUDA(cudaStreamSynchronize(s), "exact search");
  return 0;
}

int engine_anchor_scan(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* reads, size_t m,
                       uint32_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, 4 * m * sizeof(uint4) + 16) || !ensure(e, e->rows, m * 4 + 16)) {
    *err = "out of device memory (anchor scan)";
    return -1;
  }
  cudaStream_t s = e->stream;
  HPG_CUDA(cudaMemcpyAsync(e->rows.p, reads, m * 4, cudaMemcpyHostToDevice, s), "anchor reads");
  count_launches(1);
  anchor_scan_kernel<<<(unsigned)((4 * m + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes),
                                                                      ptr<uint64_t>(e->offs), ptr<uint8_t>(e->ok),
                                                                      ptr<uint32_t>(e->rows), (uint32_t)m,
                                                                      ptr<uint4>(e->slots));
  HPG_CUDA(cudaMemcpyAsync(out, e->slots.p, 4 * m * sizeof(uint4), cudaMemcpyDeviceToHost, s), "anchor scan");
  HPG_CUDA(cudaStreamSynchronize(s), "anchor scan");
  return 0;
}

int engine_seed_search(Engine* e, const char* seqs, const uint64_t* offs, size_t n, const uint32_t* seeds, size_t m,
                       uint32_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (m >= (1ull << 31)) {
    *err = "too many seeds in one call";
    return -1;
  }
  for (size_t i = 0; i < m; ++i)
    if (seeds[4 * i] >= n) {
      *err = "seed of a read outside the batch";
      return -1;
    }
  if (upload_reads(e, seqs, offs, n, err) != 0) return -1;
  if (!ensure(e, e->slots, 2 * m * sizeof(uint4) + 16)) {
    *err = "out of device memory (seeds)";
    return -1;
  }
  cudaStream_t s = e->stream;
  uint4* d_seeds = ptr<uint4>(e->slots);
  uint4* d_out = d_seeds + m;
  HPG_CUDA(cudaMemcpyAsync(d_seeds, seeds, m * sizeof(uint4), cudaMemcpyHostToDevice, s), "seeds");
  count_launches(1);
  seed_search_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(e->X, ptr<uint8_t>(e->codes), ptr<uint64_t>(e->offs),
                                                                  ptr<uint8_t>(e->ok), d_seeds, (uint32_t)m, d_out);
  HPG_CUDA(cudaMemcpyAsync(out, d_out, m * sizeof(uint4), cudaMemcpyDeviceToHost, s), "seed intervals");
  HPG_CUDA(cudaStreamSynchronize(s), "seed search");
  return 0;
}

int engine_locate_rows(Engine* e, const MapRow* rows, size_t m, hpg_loc_t* out, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (!m) return 0;
  if (m >= (1ull << 32)) {
    *err = "too many rows to locate in one call";
    return -1;
  }
  std::vector<RowItem> items(m);
  for (size_t i = 0; i < m; ++i) {
    if (rows[i].row > e->X.top) {
      *err = "row outside the suffix array";
      return -1;
    }
    items[i].row = rows[i].row;
    items[i].hit = (uint32_t)i;
    items[i].out = (uint32_t)i;
    items[i].phys_len = (rows[i].phys << 31) | (rows[i].key32 ? kRowKey32 : 0u) | (rows[i].len_calc & kRowLenMask);
  }
  if (!ensure(e, e->b_rowhit, m * sizeof(RowItem) + 16) || !ensure(e, e->locs, m * sizeof(hpg_loc_t) + 16) ||
      !ensure(e, e->b_ctr, 64)) {
    *err = "out of device memory (locate rows)";
    return -1;
  }
  cudaStream_t s = e->stream;
  HPG_CUDA(cudaMemcpyAsync(e->b_rowhit.p, items.data(), m * sizeof(RowItem), cudaMemcpyHostToDevice, s), "rows");
  launch_locate_items(e->X, static_cast<const RowItem*>(e->b_rowhit.p), m, ptr<hpg_loc_t>(e->locs),
                      ptr<unsigned int>(e->b_ctr) + 5, e->num_sms, s);
  HPG_CUDA(cudaMemcpyAsync(out, e->locs.p, m * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, s), "located rows");
  HPG_CUDA(cudaStreamSynchronize(s), "locate rows");
  return check_walk(e, err);
}

void engine_set_skip_locate(Engine* e, int on) { e->skip_locate = on != 0; }

std::mutex& map_api_mutex() {
  static std::mutex mu;
  return mu;
}
uint32_t engine_sa_top(Engine* e) { return e->X.top; }

int engine_inexact_records(Engine* e, const char* seqs, const uint64_t* offs, size_t n, int filter_read_mappings,
                           InexactRecords* out, std::string* err) {
  out->n_rec.assign(n, 0);
  out->flags.assign(n, 0);
  out->rec_off.assign(n + 1, 0);
  out->rec.clear();
  if (!n) return 0;
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  const int fr = filter_read_mappings;
  // the search: BWSearch1 with result lists of capacity filter_read_mappings, hits only
  DeviceResult r;
  engine_set_skip_locate(e, 1);
  const int rc = engine_search_host_keep(e, HPG_BWT_MODE_SEARCH1, kFormBatched, seqs, offs, n,
                                         fr > 0 ? (uint32_t)fr : 0u, &r, err);
  engine_set_skip_locate(e, 0);
  if (rc != 0) return -1;
  cudaStream_t s = e->stream;
  const size_t T = 2 * n;
  if (!ensure(e, e->m_hitoff, (T + 1) * 8) || !ensure(e, e->m_part, scan_parts(std::max(T, n)) * 8) ||
      !ensure(e, e->m_offs, (n + 1) * 8) || !ensure(e, e->m_rows, n * 4 + 16) || !ensure(e, e->m_pflag, n + 16) ||
      !ensure(e, e->m_rowoff, (n + 1) * 8) || !ensure(e, e->m_nrec, n * 4 + 16) || !ensure(e, e->m_flags, n + 16)) {
    *err = "out of device memory (alignment records)";
    return -1;
  }
  std::vector<uint64_t> rel(n + 1);
  for (size_t i = 0; i <= n; ++i) rel[i] = offs[i] - offs[0];
  HPG_CUDA(cudaMemcpyAsync(e->m_offs.p, rel.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s), "record offsets");
  launch_scan(r.rs_count, T, ptr<uint64_t>(e->m_hitoff), ptr<uint64_t>(e->m_part), s);
  const unsigned grid = (unsigned)((n + 127) / 128);
  count_launches(1);
  inexact_plan_kernel<<<grid, 128, 0, s>>>(r.hits, ptr<uint64_t>(e->m_hitoff), (uint32_t)n,
                                           (uint64_t)(int64_t)(long)fr, ptr<uint32_t>(e->m_rows),
                                           ptr<uint8_t>(e->m_pflag));
  launch_scan(ptr<uint32_t>(e->m_rows), n, ptr<uint64_t>(e->m_rowoff), ptr<uint64_t>(e->m_part), s);
  uint64_t rows = 0;
  HPG_CUDA(cudaMemcpyAsync(&rows, ptr<uint64_t>(e->m_rowoff) + n, 8, cudaMemcpyDeviceToHost, s), "row total");
  HPG_CUDA(cudaStreamSynchronize(s), "record plan");
  if (rows >= (1ull << 32)) {
    *err = "too many rows to locate in one call";
    return -1;
  }
  if (!ensure(e, e->b_rowhit, rows * sizeof(RowItem) + 16) || !ensure(e, e->locs, rows * sizeof(hpg_loc_t) + 16) ||
      !ensure(e, e->m_rec, rows * sizeof(MapRec) + 16) || !ensure(e, e->b_ctr, 64)) {
    *err = "out of device memory (alignment records)";
    return -1;
  }
  count_launches(1);
  inexact_rows_kernel<<<grid, 128, 0, s>>>(r.hits, ptr<uint64_t>(e->m_hitoff), ptr<uint64_t>(e->m_offs),
                                           ptr<uint64_t>(e->m_rowoff), ptr<uint8_t>(e->m_pflag), (uint32_t)n,
                                           static_cast<RowItem*>(e->b_rowhit.p));
  launch_locate_items(e->X, static_cast<const RowItem*>(e->b_rowhit.p), rows, ptr<hpg_loc_t>(e->locs),
                      ptr<unsigned int>(e->b_ctr) + 5, e->num_sms, s);
  count_launches(1);
  inexact_records_kernel<<<grid, 128, 0, s>>>(r.hits, ptr<uint64_t>(e->m_hitoff), ptr<uint64_t>(e->m_rowoff),
                                              ptr<uint8_t>(e->m_pflag), ptr<hpg_loc_t>(e->locs), (uint32_t)n,
                                              ptr<MapRec>(e->m_rec), ptr<uint32_t>(e->m_nrec),
                                              ptr<uint8_t>(e->m_flags));
  out->rec.resize(rows);
  HPG_CUDA(cudaMemcpyAsync(out->n_rec.data(), e->m_nrec.p, n * 4, cudaMemcpyDeviceToHost, s), "record counts");
  HPG_CUDA(cudaMemcpyAsync(out->flags.data(), e->m_flags.p, n, cudaMemcpyDeviceToHost, s), "record flags");
  HPG_CUDA(cudaMemcpyAsync(out->rec_off.data(), e->m_rowoff.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s),
           "record offsets");
  if (rows)
    HPG_CUDA(cudaMemcpyAsync(out->rec.data(), e->m_rec.p, rows * sizeof(MapRec), cudaMemcpyDeviceToHost, s),
             "records");
  HPG_CUDA(cudaStreamSynchronize(s), "alignment records");
  return check_walk(e, err);
}

void engine_note_map_device_seconds(Engine* e, double s) { e->map_device_s = s; }
double engine_map_device_seconds(Engine* e) { return e->map_device_s; }

}  // namespace hpgbwt
