// engine.cu -- GPU context: index upload, workspace and pipeline orchestration.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "engine_internal.hpp"
#include "host_pool.hpp"
#include "hpg_bwt.h"

namespace hpgbwt {

namespace {

// Code of row t (0..63) of a block (bit-plane layout).
uint32_t block_code(const OccBlock& B, int t) {
  const uint32_t lo = t < 32 ? B.bits[0] : B.bits[1], hi = t < 32 ? B.bits[2] : B.bits[3];
  return ((lo >> (t & 31)) & 1u) | (((hi >> (t & 31)) & 1u) << 1);
}

// Repack the reference's O/count tables (column c = row c-1) into 32-byte
// blocks of 64 rows with 2-bit codes and block-start counts.
std::string pack_occ(const OccTable& o, std::vector<OccBlock>* out, uint32_t* dollar) {
  const uint64_t rows = (uint64_t)o.siz - 1;  // n + 1
  const uint64_t nblk = (rows >> 6) + 1;
  out->assign(nblk, OccBlock{});
  int64_t dollar_row = -1;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t q = 0; q < (int64_t)nblk; ++q) {
    OccBlock& B = (*out)[(size_t)q];
    for (int b = 0; b < 4; ++b) {
      const size_t idx = (size_t)b * o.m + (size_t)q;
      B.cnt[b] = q < (int64_t)o.m ? o.desp[idx] + (uint32_t)(o.count[idx] & 1u) : 0u;
    }
    uint64_t plane0 = 0, plane1 = 0;  // low and high code bit of each row
    for (int t = 0; t < 64; ++t) {
      const uint64_t row = (uint64_t)q * 64 + t;
      if (row >= rows) break;
      const uint64_t col = row + 1, cq = col >> 6, cb = col & 63;
      int sym = -1, nset = 0;
      for (int b = 0; b < 4; ++b)
        if (cq < o.m && ((o.count[(size_t)b * o.m + cq] >> cb) & 1u)) {
          sym = b;
          ++nset;
        }
      if (nset > 1) bad = 1;
      if (sym < 0) {
#pragma omp critical
        {
          if (dollar_row >= 0) bad = 1;
          dollar_row = (int64_t)row;
        }
        sym = 0;
      }
      plane0 |= (uint64_t)(sym & 1) << t;
      plane1 |= (uint64_t)((sym >> 1) & 1) << t;
    }
    B.bits[0] = (uint32_t)plane0;
    B.bits[1] = (uint32_t)(plane0 >> 32);
    B.bits[2] = (uint32_t)plane1;
    B.bits[3] = (uint32_t)(plane1 >> 32);
  }
  if (bad || dollar_row < 0) return "occurrence table is not a valid BWT";
  // Block counts must equal the running counts of the codes (so every rank,
  // and with a consistent C every LF step, stays inside [0, n]).
  uint64_t run[4] = {0, 0, 0, 0};
  for (uint64_t q = 0; q < nblk; ++q) {
    const OccBlock& B = (*out)[q];
    for (int b = 0; b < 4; ++b)
      if (B.cnt[b] != run[b]) return "occurrence counts disagree with the BWT";
    for (int t = 0; t < 64; ++t) {
      const uint64_t row = q * 64 + t;
      if (row >= rows) break;
      if ((int64_t)row == dollar_row) continue;
      run[block_code(B, t)]++;
    }
  }
  *dollar = (uint32_t)dollar_row;
  return "";
}

// C must be the cumulative symbol counts (C1 = C + 1) for LF to stay in range.
std::string check_C(const HostIndex& h, const std::vector<OccBlock>& blk, uint32_t dollar) {
  uint64_t tot[4] = {0, 0, 0, 0};
  const uint64_t rows = (uint64_t)h.O.siz - 1;
  const OccBlock& last = blk.back();
  const uint64_t q = blk.size() - 1;
  for (int b = 0; b < 4; ++b) {
    tot[b] = last.cnt[b];
    for (int t = 0; t < 64; ++t) {
      const uint64_t row = q * 64 + t;
      if (row >= rows) break;
      if (row == dollar) continue;
      if (block_code(last, t) == (uint32_t)b) tot[b]++;
    }
  }
  uint64_t acc = 0;
  for (int b = 0; b < 4; ++b) {
    if (h.C[b] != acc || h.C1[b] != acc + 1) return "C/C1 vectors disagree with the occurrence table";
    acc += tot[b];
  }
  if (acc + 1 != rows) return "occurrence table size disagrees with its counts";
  return "";
}

}  // namespace

Engine* engine_create(const HostIndex& h, int device, std::string* err) {
  Alphabet a;
  std::string e = make_alphabet(h.alphabet, &a);
  if (!e.empty()) {
    *err = e;
    return nullptr;
  }
  if (h.S.ratio != h.Si.ratio || h.S.ratio == 0) {
    *err = "S and Si sampling ratios differ";
    return nullptr;
  }
  std::vector<OccBlock> blk[2];
  uint32_t dollar[2] = {0, 0};
  if (!(e = pack_occ(h.O, &blk[0], &dollar[0])).empty() || !(e = pack_occ(h.Oi, &blk[1], &dollar[1])).empty() ||
      !(e = check_C(h, blk[0], dollar[0])).empty() || !(e = check_C(h, blk[1], dollar[1])).empty()) {
    *err = e;
    return nullptr;
  }
  for (int d = 0; d < 2; ++d) {
    const SampledVec& S = d ? h.Si : h.S;
    if ((uint64_t)S.n * S.ratio < (uint64_t)h.O.siz - 1 || S.siz + 1 != h.O.siz) {
      *err = "sampled suffix array does not cover every row";
      return nullptr;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    *err = "no CUDA device available: the GB300 mapping path has no CPU fallback";
    return nullptr;
  }
  Engine* en = new Engine();
  en->device = device;
  auto fail = [&](const char* what, cudaError_t ce) {
    *err = std::string(what) + ": " + cudaGetErrorString(ce);
    engine_destroy(en);
    return (Engine*)nullptr;
  };
  cudaError_t ce;
  if ((ce = cudaSetDevice(device)) != cudaSuccess) return fail("cudaSetDevice", ce);
  if ((ce = cudaStreamCreateWithFlags(&en->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail("cudaStreamCreate", ce);
  for (int i = 0; i <= kStageCount; ++i) cudaEventCreate(&en->ev[i]);
  for (int i = 0; i < 4; ++i) cudaEventCreate(&en->cev[i]);
  cudaEventCreate(&en->dev_mid);
  const SampledVec* S[2] = {&h.S, &h.Si};
  for (int d = 0; d < 2; ++d) {
    if ((ce = cudaMalloc(&en->d_occ[d], blk[d].size() * sizeof(OccBlock))) != cudaSuccess)
      return fail("cudaMalloc(occ)", ce);
    if ((ce = cudaMemcpy(en->d_occ[d], blk[d].data(), blk[d].size() * sizeof(OccBlock), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return fail("upload occ", ce);
    if ((ce = cudaMalloc(&en->d_S[d], (size_t)S[d]->n * 4 + 4)) != cudaSuccess) return fail("cudaMalloc(S)", ce);
    if ((ce = cudaMemcpy(en->d_S[d], S[d]->v.data(), (size_t)S[d]->n * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail("upload S", ce);
    en->X.dir[d].occ = en->d_occ[d];
    en->X.dir[d].S = en->d_S[d];
    en->X.dir[d].dollar = dollar[d];
    en->X.dir[d].nblk = (uint32_t)blk[d].size();
  }
  const size_t nk = h.kar.start.size();
  if ((ce = cudaMalloc(&en->d_kar_off, (nk + 1) * 8)) != cudaSuccess) return fail("cudaMalloc(karyotype)", ce);
  if ((ce = cudaMalloc(&en->d_kar_start, (nk + 1) * 8)) != cudaSuccess) return fail("cudaMalloc(karyotype)", ce);
  cudaMemcpy(en->d_kar_off, h.kar.offset.data(), (nk + 1) * 8, cudaMemcpyHostToDevice);
  if (nk) cudaMemcpy(en->d_kar_start, h.kar.start.data(), nk * 8, cudaMemcpyHostToDevice);
  std::memcpy(en->h_table, a.code_of, 256);
  if ((ce = cudaMalloc(&en->d_table, 256)) != cudaSuccess) return fail("cudaMalloc(table)", ce);
  cudaMemcpy(en->d_table, en->h_table, 256, cudaMemcpyHostToDevice);
  if ((ce = cudaMalloc(&en->d_err, 4)) != cudaSuccess) return fail("cudaMalloc(err)", ce);
  cudaMemset(en->d_err, 0, 4);
  en->X.err = en->d_err;
  en->X.load_mode = 2;
  // default batched form: warp-cooperative, 16 reads per warp group, one launch
  // per index direction, 12 resident blocks per SM (the autotuner may pick another)
  en->tuning.split = 3;
  en->tuning.group = 16;
  en->tuning.dir_split = 2;
  en->tuning.min_blocks = 12;
  en->X.kmer_len = 0;
  en->X.kmer[0] = en->X.kmer[1] = nullptr;

  for (int b = 0; b < 4; ++b) {
    en->X.C[b] = h.C[b];
    en->X.C1[b] = h.C1[b];
    en->X.comp[b] = a.comp[b];
    en->X.comp_packed |= (a.comp[b] & 3u) << (2 * b);
  }
  en->X.ratio = h.S.ratio;
  en->X.ratio_shift = 0xFFFFFFFFu;
  for (uint32_t s = 0; s < 32; ++s)
    if ((1u << s) == h.S.ratio) en->X.ratio_shift = s;
  en->X.walk_mod = h.O.siz - 1;
  en->X.top = h.S.siz - 1;
  en->X.kar_offset = en->d_kar_off;
  en->X.kar_start = en->d_kar_start;
  en->X.kar_size = (uint32_t)nk;
  cudaDeviceGetAttribute(&en->num_sms, cudaDevAttrMultiProcessorCount, device);
  if ((ce = cudaDeviceSynchronize()) != cudaSuccess) return fail("index upload", ce);
  {
    const uint32_t n_samples[2] = {(uint32_t)S[0]->n, (uint32_t)S[1]->n};
    std::string terr;
    if (build_text_samples(en, n_samples, &terr) != 0) {
      *err = terr;
      engine_destroy(en);
      return nullptr;
    }
    for (int d = 0; d < 2; ++d) {  // the row samples served only the derivation
      cudaFree(en->d_S[d]);
      en->d_S[d] = nullptr;
      en->X.dir[d].S = nullptr;
    }
  }
  {
    std::string kerr;
    if (engine_set_kmer(en, kDefaultKmer, &kerr) != 0) {
      *err = kerr;
      engine_destroy(en);
      return nullptr;
    }
  }
  return en;
}

void engine_release_workspace(Engine* e, uint64_t keep_n_cap) {
  graph_plans_drop_above(e, keep_n_cap);
  cudaStreamSynchronize(e->stream);
  DevBuf* bufs[] = {&e->seqs, &e->offs, &e->codes, &e->ok, &e->rs_count, &e->rs_trunc, &e->vecs, &e->slots,
                    &e->ovf, &e->ovf_count, &e->hit_off, &e->scan_part, &e->hits, &e->rows, &e->loc_off, &e->locs,
                    &e->b_res, &e->b_sorted, &e->b_spill, &e->b_arr, &e->b_seg, &e->b_rowhit, &e->b_long,
                    &e->b_blocks, &e->b_bovf, &e->m_hitoff, &e->m_part, &e->m_offs, &e->m_rows, &e->m_pflag,
                    &e->m_rowoff, &e->m_nrec, &e->m_flags, &e->m_rec};
  for (DevBuf* b : bufs) {
    cudaFree(b->p);
    b->p = nullptr;
    b->cap = 0;
  }
  e->b_res_cap = e->b_spill_cap = 0;
  e->last = DeviceResult();
}

void engine_destroy(Engine* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  graph_plans_destroy(e);
  for (cudaStream_t& x : e->xs)
    if (x) cudaStreamDestroy(x);
  if (e->pev_made)
    for (auto& row : e->pev)
      for (cudaEvent_t ev : row) cudaEventDestroy(ev);
  for (int d = 0; d < 2; ++d) {
    cudaFree(e->d_occ[d]);
    cudaFree(e->d_S[d]);
    cudaFree(e->d_mark[d]);
    cudaFree(e->d_T[d]);
  }
  cudaFree(e->d_kar_off);
  cudaFree(e->d_kar_start);
  cudaFree(e->d_table);
  cudaFree(e->d_err);
  cudaFree(e->d_kmer[0]);
  cudaFree(e->d_kmer[1]);
  DevBuf* bufs[] = {&e->seqs, &e->offs, &e->codes, &e->ok, &e->rs_count, &e->rs_trunc, &e->vecs, &e->slots,
                    &e->ovf, &e->ovf_count, &e->hit_off, &e->scan_part, &e->hits, &e->rows, &e->loc_off, &e->locs,
                    &e->census, &e->b_ctr, &e->b_res, &e->b_sorted, &e->b_spill, &e->b_arr, &e->b_seg,
                    &e->b_rowhit, &e->b_long, &e->b_blocks, &e->b_bovf, &e->m_hitoff, &e->m_part, &e->m_offs,
                    &e->m_rows, &e->m_pflag, &e->m_rowoff, &e->m_nrec, &e->m_flags, &e->m_rec};
  for (DevBuf* b : bufs) cudaFree(b->p);
  for (int i = 0; i <= kStageCount; ++i)
    if (e->ev[i]) cudaEventDestroy(e->ev[i]);
  for (int i = 0; i < 4; ++i)
    if (e->cev[i]) cudaEventDestroy(e->cev[i]);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

void* engine_stream(Engine* e) { return (void*)e->stream; }

// Accessors for the allocation-free entry point (noalloc.cu).
DevIndex engine_dev_index(void* e) { return static_cast<Engine*>(e)->X; }
const uint8_t* engine_code_table(void* e) { return static_cast<Engine*>(e)->d_table; }
int engine_device_of(void* e) { return static_cast<Engine*>(e)->device; }
void* engine_stream_of(void* e) { return (void*)static_cast<Engine*>(e)->stream; }
int engine_device(Engine* e) { return e->device; }
void engine_set_census(Engine* e, int on) { e->census_on = on != 0; }
unsigned long long engine_census(Engine* e) { return e->census_val; }
void engine_set_chunk(Engine* e, size_t reads) { e->chunk = reads; }
size_t engine_index_bytes(Engine* e) {
  return ((size_t)e->X.dir[0].nblk + e->X.dir[1].nblk) * sizeof(OccBlock);
}

void engine_stage_ms(Engine* e, float* out, int n) {
  for (int i = 0; i < n && i < kStageCount; ++i) out[i] = e->stage_ms[i];
  if (n > kStageCount) out[kStageCount] = e->drain_ms;  // of the search stage: time in the drain launch
}

namespace {

// Batched form: persistent search (+ drain of spilled change points), ordered
// finalize, persistent locate.  Grows its pools and reruns on overflow.
int run_batched(Engine* e, const uint8_t* d_offs_u8, const uint64_t* d_offs, uint32_t n, uint32_t max_results,
                unsigned long long* census, size_t* n_hits_out, size_t* n_locs_out, float* t_search, float* t_final,
                float* t_loc, std::string* err) {
  (void)d_offs_u8;
  cudaStream_t s = e->stream;
  const size_t T = 2ull * n;
  // reads too long for a warp group buffer of the warp-cooperative form (at most one per kWaveLongMin bases)
  const uint32_t long_cap = (uint32_t)std::min<size_t>(e->codes.cap / kWaveLongMin + 2, 0xFFFFFFF0u);
  if (!ensure(e, e->b_ctr, 64) || !ensure(e, e->b_arr, T * 4 + 16) || !ensure(e, e->b_seg, (T + 1) * 8) ||
      !ensure(e, e->hit_off, (T + 1) * 8) || !ensure(e, e->scan_part, scan_parts(T) * 8) ||
      !ensure(e, e->b_long, (size_t)long_cap * 4)) {
    *err = "out of device memory (batched counters)";
    return -1;
  }
  if (e->b_res_cap < 4 * (size_t)n + 4096) e->b_res_cap = (uint32_t)std::min<size_t>(4 * (size_t)n + 4096, 0xFFFFFFF0u);
  const size_t spill_want = e->tuning.split ? 4 * (size_t)n + 4096 + (size_t)e->num_sms * 16 * 128 * 8
                                            : (size_t)n / 4 + 4096;
  if (e->b_spill_cap < spill_want) e->b_spill_cap = (uint32_t)std::min<size_t>(spill_want, 0xFFFFFFF0u);
  unsigned int* ctr = ptr<unsigned int>(e->b_ctr);  // [0] chains [1] spill head [2] spill tail [3] results [4] status [5..7] locate [8] phase-1 chains
  uint32_t status = 0, res_total = 0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    const bool wave = e->tuning.split == 3;
    if (!ensure(e, e->b_res, (size_t)e->b_res_cap * sizeof(PendingHit)) ||
        !ensure(e, e->b_sorted, (size_t)e->b_res_cap * sizeof(PendingHit)) ||
        !ensure(e, e->b_spill, (size_t)e->b_spill_cap * sizeof(SpillEntry)) ||
        (wave && !ensure(e, e->b_blocks, (size_t)e->b_spill_cap * sizeof(SpillEntry)))) {
      *err = "out of device memory (batched pools)";
      return -1;
    }
    cudaMemsetAsync(ctr, 0, 64, s);
    cudaMemsetAsync(e->b_arr.p, 0, T * 4, s);
    if (census) cudaMemsetAsync(census, 0, 8, s);
    BatchedParams p;
    p.codes = ptr<uint8_t>(e->codes);
    p.codes_len = e->codes.cap;
    p.offs = d_offs;
    p.ok = ptr<uint8_t>(e->ok);
    p.n_reads = n;
    p.n_reads_dev = nullptr;
    p.max_results = max_results;
    p.chain_ctr = ctr + 0;
    p.chain_ctr2 = ctr + 9;
    p.dir_split = e->tuning.split == 0 ? (uint32_t)e->tuning.dir_split : 0u;
    p.num_sms = (uint32_t)e->num_sms;
    p.batch_idle = (uint32_t)(e->tuning.batch_idle < 1 ? 1 : e->tuning.batch_idle);
    p.spill_head = ctr + 1;
    p.spill_tail = ctr + 2;
    p.spill = ptr<SpillEntry>(e->b_spill);
    p.spill_cap = e->b_spill_cap;
    p.res_total = ctr + 3;
    p.res = ptr<PendingHit>(e->b_res);
    p.res_cap = e->b_res_cap;
    p.rs_count = ptr<uint32_t>(e->b_arr);
    p.status = ctr + 4;
    p.census = census;
    cudaEventRecord(e->cev[0], s);
    launch_search_stage(e->X, p, e->tuning, e->num_sms, ctr, ptr<uint32_t>(e->b_long), long_cap,
                        wave ? ptr<SpillEntry>(e->b_blocks) : nullptr, wave ? e->b_spill_cap : 0u, e->dev_mid, false,
                        s);
    cudaEventRecord(e->cev[1], s);
    uint32_t h[5];
    HPG_CUDA(cudaMemcpyAsync(h, ctr, 20, cudaMemcpyDeviceToHost, s), "batched counters");
    HPG_CUDA(cudaStreamSynchronize(s), "batched search");
    status = h[4];
    res_total = h[3];
    if (!status) break;
    if (status & kStatusWaveAcct) {
      *err = "internal error: inconsistent work counts in the warp-cooperative search";
      return -1;
    }
    if (status & kStatusResFull) e->b_res_cap = (uint32_t)std::min<size_t>((size_t)res_total * 2 + 4096, 0xFFFFFFF0u);
    if (status & kStatusSpillFull) e->b_spill_cap = (uint32_t)std::min<size_t>((size_t)h[2] * 2 + 4096, 0xFFFFFFF0u);
  }
  if (status) {
    *err = "batched search pools kept overflowing";
    return -1;
  }
  if (census) {
    unsigned long long v = 0;
    HPG_CUDA(cudaMemcpy(&v, census, 8, cudaMemcpyDeviceToHost), "census");
    e->census_val += v;
  }
  // ordered finalize
  launch_scan(ptr<uint32_t>(e->b_arr), T, ptr<uint64_t>(e->b_seg), ptr<uint64_t>(e->scan_part), s);
  cudaMemsetAsync(e->hit_off.p, 0, T * 4, s);  // per-list cursors (hit_off is rewritten below)
  launch_scatter_hits(ptr<PendingHit>(e->b_res), ctr + 3, ptr<uint64_t>(e->b_seg), ptr<PendingHit>(e->b_sorted),
                      e->b_res_cap, ptr<uint32_t>(e->hit_off), s);
  launch_sort_truncate(ptr<PendingHit>(e->b_sorted), ptr<PendingHit>(e->b_res), ptr<uint64_t>(e->b_seg), (uint32_t)T,
                       max_results, ptr<uint32_t>(e->rs_count), ptr<uint8_t>(e->rs_trunc), e->num_sms, s);
  launch_scan(ptr<uint32_t>(e->rs_count), T, ptr<uint64_t>(e->hit_off), ptr<uint64_t>(e->scan_part), s);
  uint64_t h_tot = 0;
  HPG_CUDA(cudaMemcpyAsync(&h_tot, ptr<uint64_t>(e->hit_off) + T, 8, cudaMemcpyDeviceToHost, s), "hit count");
  HPG_CUDA(cudaStreamSynchronize(s), "hit scan");
  if (!ensure(e, e->hits, (h_tot + 1) * sizeof(hpg_hit_t)) || !ensure(e, e->rows, (h_tot + 1) * 4) ||
      !ensure(e, e->loc_off, (h_tot + 2) * 8) || !ensure(e, e->scan_part, scan_parts(h_tot) * 8)) {
    *err = "out of device memory (hits)";
    return -1;
  }
  launch_expand_hits(ptr<PendingHit>(e->b_sorted), ptr<uint64_t>(e->b_seg), ptr<uint64_t>(e->hit_off),
                     ptr<uint32_t>(e->rs_count), (uint32_t)T, ptr<hpg_hit_t>(e->hits), ptr<uint32_t>(e->rows), s);
  uint64_t l_tot = 0;
  if (!e->skip_locate) {
    launch_limit_rows(ptr<uint64_t>(e->hit_off), ptr<uint32_t>(e->rows), (uint32_t)T, e->locate_limit, nullptr,
                      ptr<uint8_t>(e->rs_trunc), s);
    launch_scan(ptr<uint32_t>(e->rows), h_tot, ptr<uint64_t>(e->loc_off), ptr<uint64_t>(e->scan_part), s);
    HPG_CUDA(cudaMemcpyAsync(&l_tot, ptr<uint64_t>(e->loc_off) + h_tot, 8, cudaMemcpyDeviceToHost, s), "loc count");
  }
  HPG_CUDA(cudaStreamSynchronize(s), "locate scan");
  cudaEventRecord(e->cev[2], s);
  if (l_tot > kMaxLocateRows) {
    *err = "too many located rows in one batched call (" + std::to_string(l_tot) + ", limit " +
           std::to_string(kMaxLocateRows) + "): split the batch or use the plain form";
    return -1;
  }
  if (!ensure(e, e->locs, (l_tot + 1) * sizeof(hpg_loc_t)) ||
      !ensure(e, e->b_rowhit, (l_tot + 1) * locate_row_item_bytes())) {
    *err = oom_message(("locate output, " + std::to_string(l_tot) + " rows of " + std::to_string(h_tot) + " hits").c_str(),
                       (l_tot + 1) * (sizeof(hpg_loc_t) + locate_row_item_bytes()));
    return -1;
  }
  if (census) cudaMemsetAsync(census, 0, 8, s);
  cudaMemsetAsync(ctr + 5, 0, 12, s);  // row claim counter and the two direction counters
  launch_locate_persistent(e->X, ptr<hpg_hit_t>(e->hits), ptr<uint64_t>(e->loc_off), (uint32_t)h_tot, l_tot, d_offs,
                           ptr<hpg_loc_t>(e->locs), e->b_rowhit.p, ctr + 5, census, e->num_sms, s);
  cudaEventRecord(e->cev[3], s);
  HPG_CUDA(cudaStreamSynchronize(s), "locate kernel");
  if (census) {
    unsigned long long v = 0;
    HPG_CUDA(cudaMemcpy(&v, census, 8, cudaMemcpyDeviceToHost), "census");
    e->census_val += v;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, e->cev[0], e->cev[1]);
  *t_search += ms;
  cudaEventElapsedTime(&e->drain_ms, e->dev_mid, e->cev[1]);
  cudaEventElapsedTime(&ms, e->cev[1], e->cev[2]);
  *t_final += ms;
  cudaEventElapsedTime(&ms, e->cev[2], e->cev[3]);
  *t_loc += ms;
  *n_hits_out = h_tot;
  *n_locs_out = l_tot;
  return 0;
}

}  // namespace

void engine_set_tuning(Engine* e, int min_blocks, int blocks_per_sm, int stack, int chunk) {
  // stack depth 0 selects the split (chain-only) form, -1 the lockstep form
  e->tuning.split = stack == 0 ? 1 : (stack < 0 ? 2 : 0);
  if (stack <= 0) stack = 2;
  e->tuning.min_blocks = min_blocks >= 16 ? 16 : (min_blocks >= 12 ? 12 : (min_blocks >= 10 ? 10 : 1));
  e->tuning.blocks_per_sm = blocks_per_sm;
  e->tuning.stack = stack <= 2 ? 2 : (stack <= 4 ? 4 : 8);
  e->tuning.chunk = chunk < 1 ? 1 : (chunk > 8 ? 8 : chunk);
}

void engine_set_dir_split(Engine* e, int mode) { e->tuning.dir_split = mode < 0 ? 0 : (mode > 2 ? 2 : mode); }
void engine_set_wave_group(Engine* e, int reads) {
  if (reads <= 0) {
    if (e->tuning.split == 3) e->tuning.split = 0;
    return;
  }
  e->tuning.split = 3;
  e->tuning.group = reads > 32 ? 32 : reads;
  // the warp-cooperative kernel is built for register bounds of 1, 8 and 12 blocks per SM
  e->tuning.min_blocks = e->tuning.min_blocks >= 12 ? 12 : (e->tuning.min_blocks >= 8 ? 8 : 1);
}
int engine_wave_group(Engine* e) { return e->tuning.split == 3 ? e->tuning.group : 0; }
void engine_set_idle_batch(Engine* e, int lanes) { e->tuning.batch_idle = lanes < 1 ? 1 : (lanes > 32 ? 32 : lanes); }
int engine_idle_batch(Engine* e) { return e->tuning.batch_idle; }
int engine_dir_split(Engine* e) { return e->tuning.dir_split; }
void engine_set_locate_limit(Engine* e, uint64_t max_rows) { e->locate_limit = max_rows; }
uint64_t engine_locate_limit(Engine* e) { return e->locate_limit; }

void engine_set_load_mode(Engine* e, int mode) { e->X.load_mode = (uint32_t)(mode < 0 ? 0 : (mode > 3 ? 3 : mode)); }
int engine_load_mode(Engine* e) { return (int)e->X.load_mode; }

void engine_get_tuning(Engine* e, int* out5) {
  out5[0] = e->tuning.block;
  out5[1] = batched_max_blocks_per_sm(e->tuning);
  out5[2] = e->tuning.split == 3 ? -2 : (e->tuning.split == 2 ? -1 : (e->tuning.split ? 0 : e->tuning.stack));
  out5[3] = e->tuning.split == 3 ? e->tuning.group : e->tuning.chunk;
  out5[4] = e->tuning.min_blocks;
}

// Autotuner: time the batched search on (a prefix of) the batch for every
// candidate setting and keep the fastest.  Writes up to max_rows rows of
// {min_blocks, blocks_per_sm, stack, chunk, search ms * 1000} to table.
int engine_autotune(Engine* e, const uint8_t* d_seqs, const uint64_t* d_offs, size_t n_reads, uint64_t total_bases,
                    uint32_t max_len, uint32_t max_results, int* table, int max_rows, int* rows_out,
                    std::string* err) {
  static const int cand_minb[] = {1, 10, 12, 16};  // 10: fused form only (the others take 1)
  static const int cand_stack[] = {-1, 0, 2, 4, 8};  // 0: split form, -1: lockstep form
  static const int cand_chunk[] = {1, 2, 4};
  BatchedTuning best = e->tuning;
  float best_ms = 1e30f;
  int rows = 0;
  DeviceResult r;
  // candidates run in the direct form (same kernels and grids; no capture per candidate)
  const bool graph_was = e->use_graph;
  e->use_graph = false;
  struct Restore {
    Engine* e;
    bool on;
    ~Restore() { e->use_graph = on; }
  } restore{e, graph_was};
  for (int mb : cand_minb)
    for (int st : cand_stack)
      for (int ch : cand_chunk) {
        engine_set_tuning(e, mb, 0, st, ch);
        float t = 0;
        for (int rep = 0; rep < 2; ++rep) {  // first run warms, second is timed
          if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases,
                                   max_len, max_results, &r, err) != 0)
            return -1;
          t = e->stage_ms[kStageSearch];
        }
        if (table && rows < max_rows) {
          int* row = table + 5 * rows;
          row[0] = mb;
          row[1] = batched_max_blocks_per_sm(e->tuning);
          row[2] = st;
          row[3] = ch;
          row[4] = (int)(t * 1000.0f);
        }
        ++rows;
        if (t < best_ms) {
          best_ms = t;
          best = e->tuning;
        }
      }
  // the warp-cooperative form: reads per warp group (lanes per read = 32 / group)
  // x register bound x one launch per index direction or one for both; rows
  // carry stack -2 and the group in the chains column
  for (int grp : {8, 16, 32})
    for (int mb : {8, 12})
      for (int ds : {0, 2}) {
        engine_set_tuning(e, mb, 0, 4, 1);
        e->tuning.split = 3;
        e->tuning.min_blocks = mb;
        e->tuning.group = grp;
        e->tuning.dir_split = ds;
        float t = 0;
        for (int rep = 0; rep < 2; ++rep) {
          if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases,
                                   max_len, max_results, &r, err) != 0)
            return -1;
          t = e->stage_ms[kStageSearch];
        }
        if (table && rows < max_rows) {
          int* row = table + 5 * rows;
          row[0] = mb;
          row[1] = batched_max_blocks_per_sm(e->tuning);
          row[2] = -2;
          row[3] = grp;
          row[4] = (int)(t * 1000.0f);
        }
        ++rows;
        if (t < best_ms) {
          best_ms = t;
          best = e->tuning;
        }
      }
  e->tuning = best;
  // then the block-load form, with the chosen setting
  uint32_t best_mode = e->X.load_mode;
  for (int mode = 0; mode < 4; ++mode) {
    e->X.load_mode = (uint32_t)mode;
    float t = 0;
    for (int rep = 0; rep < 2; ++rep) {
      if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases, max_len,
                               max_results, &r, err) != 0)
        return -1;
      t = e->stage_ms[kStageSearch];
    }
    if (table && rows < max_rows) {
      int* row = table + 5 * rows;
      row[0] = -1 - mode;  // load-mode rows are marked by a negative first column
      row[1] = batched_max_blocks_per_sm(e->tuning);
      row[2] = e->tuning.split == 3 ? -2 : (e->tuning.split == 2 ? -1 : (e->tuning.split ? 0 : e->tuning.stack));
      row[3] = e->tuning.split == 3 ? e->tuning.group : e->tuning.chunk;
      row[4] = (int)(t * 1000.0f);
    }
    ++rows;
    if (t < best_ms) {
      best_ms = t;
      best_mode = (uint32_t)mode;
    }
  }
  e->X.load_mode = best_mode;
  // then the direction split of the fused form (rows marked by -50 - mode);
  // one launch per direction is kept unless another mode is more than 2 %
  // faster: at equal speed it reads several times less DRAM (one direction's
  // blocks stay in L2), which leaves bandwidth to transfers and other work
  if (e->tuning.split == 0) {
    float t_on[3] = {0, 0, 0};
    for (int on = 0; on < 3; ++on) {
      e->tuning.dir_split = on;
      float t = 0;
      for (int rep = 0; rep < 2; ++rep) {
        if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases,
                                 max_len, max_results, &r, err) != 0)
          return -1;
        t = e->stage_ms[kStageSearch];
      }
      if (table && rows < max_rows) {
        int* row = table + 5 * rows;
        row[0] = -50 - on;
        row[1] = batched_max_blocks_per_sm(e->tuning);
        row[2] = e->tuning.stack;
        row[3] = e->tuning.chunk;
        row[4] = (int)(t * 1000.0f);
      }
      ++rows;
      t_on[on] = t;
    }
    int best_split = 0;
    for (int on = 1; on < 3; ++on)
      if (t_on[on] < t_on[best_split]) best_split = on;
    if (t_on[2] <= 1.02f * t_on[best_split]) best_split = 2;
    best_ms = t_on[best_split];
    e->tuning.dir_split = best_split;
  }
  // then the start-table length (rows marked by a first column of -100 - L)
  int best_kmer = (int)e->X.kmer_len;
  for (int L : {0, 8, 10, 11, 12}) {
    if (engine_set_kmer(e, L, err) != 0) return -1;
    float t = 0;
    for (int rep = 0; rep < 2; ++rep) {
      if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases, max_len,
                               max_results, &r, err) != 0)
        return -1;
      t = e->stage_ms[kStageSearch];
    }
    if (table && rows < max_rows) {
      int* row = table + 5 * rows;
      row[0] = -100 - L;
      row[1] = batched_max_blocks_per_sm(e->tuning);
      row[2] = e->tuning.split == 3 ? -2 : (e->tuning.split == 2 ? -1 : (e->tuning.split ? 0 : e->tuning.stack));
      row[3] = e->tuning.split == 3 ? e->tuning.group : e->tuning.chunk;
      row[4] = (int)(t * 1000.0f);
    }
    ++rows;
    if (t < best_ms) {
      best_ms = t;
      best_kmer = L;
    }
  }
  if (engine_set_kmer(e, best_kmer, err) != 0) return -1;
  // then the idle-lane batch (rows marked by -200 - batch): the fused kernel,
  // the chain-only kernel of the split form and every form's drain launch use it
  {
    int best_batch = e->tuning.batch_idle;
    for (int b : {1, 4, 8, 16}) {
      e->tuning.batch_idle = b;
      float t = 0;
      for (int rep = 0; rep < 2; ++rep) {
        if (engine_search_device(e, HPG_BWT_MODE_SEARCH1, kFormBatched, d_seqs, d_offs, n_reads, total_bases,
                                 max_len, max_results, &r, err) != 0)
          return -1;
        t = e->stage_ms[kStageSearch];
      }
      if (table && rows < max_rows) {
        int* row = table + 5 * rows;
        row[0] = -200 - b;
        row[1] = batched_max_blocks_per_sm(e->tuning);
        row[2] = e->tuning.stack;
        row[3] = e->tuning.chunk;
        row[4] = (int)(t * 1000.0f);
      }
      ++rows;
      if (t < best_ms) {
        best_ms = t;
        best_batch = b;
      }
    }
    e->tuning.batch_idle = best_batch;
  }
  if (rows_out) *rows_out = rows;
  return 0;
}

namespace {

// Batched form from the captured graph, then the walk-error check every form makes.
int finish_graph(Engine* e, const void* seqs, const uint64_t* offs, uint32_t n, uint64_t total,
                 uint32_t max_results, DeviceResult* out, std::string* err) {
  DeviceResult r;
  if (run_batched_graph(e, seqs, offs, n, total, max_results, &r, err) != 0) return -1;
  uint32_t derr = 0;
  HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
  if (derr) {
    cudaMemset(e->d_err, 0, 4);
    *err = "corrupt index: suffix-array walk did not reach a sampled row";
    return -1;
  }
  e->last = r;
  *out = r;
  return 0;
}

}  // namespace

int engine_set_kmer(Engine* e, int L, std::string* err) {
  if (L < 0 || L > 12) {
    *err = "start table length must be 0..12 symbols";
    return -1;
  }
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if ((uint32_t)L == e->X.kmer_len) return 0;
  HPG_CUDA(cudaStreamSynchronize(e->stream), "start table");
  for (uint2*& t : e->d_kmer) {
    cudaFree(t);
    t = nullptr;
  }
  e->X.kmer[0] = e->X.kmer[1] = nullptr;
  e->X.kmer_len = 0;
  if (L > 0) {
    const size_t bytes = ((size_t)1 << (2 * L)) * sizeof(uint2);
    for (int d = 0; d < 2; ++d) {
      if (cudaMalloc(&e->d_kmer[d], bytes) != cudaSuccess) {
        cudaGetLastError();
        *err = "out of device memory (start table)";
        return -1;
      }
      launch_build_kmer(e->X, (uint32_t)d, (uint32_t)L, e->d_kmer[d], e->stream);
    }
    HPG_CUDA(cudaStreamSynchronize(e->stream), "start table");
    e->X.kmer[0] = e->d_kmer[0];
    e->X.kmer[1] = e->d_kmer[1];
    e->X.kmer_len = (uint32_t)L;
  }
  return 0;
}

int engine_kmer(Engine* e) { return (int)e->X.kmer_len; }

void engine_set_graph(Engine* e, int on) { e->use_graph = on != 0; }
void engine_set_pipeline_chunk(Engine* e, size_t reads) { e->pipe_chunk = reads; }
int engine_graph(Engine* e) { return e->use_graph ? 1 : 0; }

int engine_search_device(Engine* e, int mode, int form, const uint8_t* d_seqs, const uint64_t* d_offs, size_t n_reads,
                         uint64_t total_bases, uint32_t max_len, uint32_t max_results, DeviceResult* out,
                         std::string* err) {
  if (mode != HPG_BWT_MODE_EXACT && mode != HPG_BWT_MODE_SEARCH1) {
    *err = "unknown search mode";
    return -1;
  }
  if (form != kFormPlain && form != kFormBatched) {
    *err = "unknown pipeline form";
    return -1;
  }
  if (form == kFormBatched && mode != HPG_BWT_MODE_SEARCH1) form = kFormPlain;  // exact search has no branches
  if (n_reads >= (1ull << 31)) {
    *err = "too many reads in one batch";
    return -1;
  }
  if (max_len > 32767) {
    *err = "reads longer than 32767 bases are not supported";
    return -1;
  }
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  cudaStream_t s = e->stream;
  const uint32_t n = (uint32_t)n_reads;
  const uint32_t len_cap = std::max<uint32_t>(max_len, 3);
  if (form == kFormBatched && e->use_graph) return finish_graph(e, d_seqs, d_offs, n, total_bases, max_results, out, err);

  if (!ensure(e, e->codes, total_bases + 16) || !ensure(e, e->ok, n + 16) || !ensure(e, e->rs_count, 8ull * n + 16) ||
      !ensure(e, e->rs_trunc, 2ull * n + 16) || !ensure(e, e->census, 16) || !ensure(e, e->ovf_count, 16)) {
    *err = "out of device memory (read buffers)";
    return -1;
  }
  // Sector census (bench only): counted per launch, summed on the host.
  unsigned long long* census = e->census_on ? ptr<unsigned long long>(e->census) : nullptr;
  e->census_val = 0;
  auto census_take = [&]() -> int {
    if (!census) return 0;
    unsigned long long v = 0;
    HPG_CUDA(cudaMemcpyAsync(&v, census, 8, cudaMemcpyDeviceToHost, s), "census");
    HPG_CUDA(cudaStreamSynchronize(s), "census");
    e->census_val += v;
    return 0;
  };

  // Chunk so that the plain form's vector scratch stays within ~8 GB.
  size_t chunk = e->chunk;
  if (chunk == 0) {
    const size_t per_read = (mode == HPG_BWT_MODE_SEARCH1) ? 2ull * 2 * len_cap * 8 : 0;
    chunk = per_read ? std::max<size_t>(1024, (8ull << 30) / per_read) : n_reads;
  }
  chunk = std::max<size_t>(1, std::min(chunk, std::max<size_t>(n_reads, 1)));

  cudaEventRecord(e->ev[0], s);
  launch_encode(d_seqs, total_bases, d_offs, n, e->d_table, ptr<uint8_t>(e->codes), ptr<uint8_t>(e->ok), s);
  cudaEventRecord(e->ev[1], s);

  size_t n_hits = 0, n_locs = 0;
  float t_search = 0, t_final = 0, t_loc = 0;
  cudaEvent_t a = e->cev[0], b = e->cev[1], c = e->cev[2], d = e->cev[3];
  e->drain_ms = 0;
  if (form == kFormBatched) {
    if (run_batched(e, d_seqs, d_offs, n, max_results, census, &n_hits, &n_locs, &t_search, &t_final, &t_loc, err) !=
        0)
      return -1;
    chunk = n_reads;  // skip the plain chunk loop
  }
  for (size_t r0 = (form == kFormBatched ? n_reads : 0); r0 < n_reads; r0 += chunk) {
    const uint32_t nr = (uint32_t)std::min(chunk, n_reads - r0);
    const size_t T = 2ull * nr;
    if (!ensure(e, e->slots, T * kSlotCap * sizeof(uint4)) || !ensure(e, e->hit_off, (T + 1) * 8) ||
        !ensure(e, e->scan_part, scan_parts(T) * 8)) {
      *err = "out of device memory (hit slots)";
      return -1;
    }
    if (mode == HPG_BWT_MODE_SEARCH1) {
      if (!ensure(e, e->vecs, 2ull * len_cap * T * sizeof(uint2))) {
        *err = "out of device memory (vector scratch)";
        return -1;
      }
      if (e->ovf_cap < T) {
        if (!ensure(e, e->ovf, T * sizeof(OvfEntry))) {
          *err = "out of device memory (overflow pool)";
          return -1;
        }
        e->ovf_cap = (uint32_t)std::min<size_t>(e->ovf.cap / sizeof(OvfEntry), 0xFFFFFFFFu);
      }
    }
    cudaEventRecord(a, s);
    for (int attempt = 0;; ++attempt) {
      if (census) cudaMemsetAsync(census, 0, 8, s);
      if (mode == HPG_BWT_MODE_EXACT) {
        launch_exact(e->X, ptr<uint8_t>(e->codes), d_offs, ptr<uint8_t>(e->ok), (uint32_t)r0, nr,
                     ptr<uint4>(e->slots), ptr<uint32_t>(e->rs_count), ptr<uint8_t>(e->rs_trunc), census, s);
        break;
      }
      cudaMemsetAsync(e->ovf_count.p, 0, 4, s);
      launch_plain_search1(e->X, ptr<uint8_t>(e->codes), d_offs, ptr<uint8_t>(e->ok), (uint32_t)r0, nr, max_results,
                           len_cap, ptr<uint2>(e->vecs), ptr<uint4>(e->slots), ptr<OvfEntry>(e->ovf), e->ovf_cap,
                           ptr<uint32_t>(e->ovf_count), ptr<uint32_t>(e->rs_count), ptr<uint8_t>(e->rs_trunc),
                           census, s);
      uint32_t used = 0;
      HPG_CUDA(cudaMemcpyAsync(&used, e->ovf_count.p, 4, cudaMemcpyDeviceToHost, s), "overflow count");
      HPG_CUDA(cudaStreamSynchronize(s), "search kernel");
      if (used <= e->ovf_cap) break;
      if (!ensure(e, e->ovf, (size_t)used * 2 * sizeof(OvfEntry))) {
        *err = "out of device memory (overflow pool)";
        return -1;
      }
      e->ovf_cap = (uint32_t)std::min<size_t>(e->ovf.cap / sizeof(OvfEntry), 0xFFFFFFFFu);
    }
    cudaEventRecord(b, s);
    if (census_take() != 0) return -1;
    // ordered hits of this chunk
    launch_scan(ptr<uint32_t>(e->rs_count) + 2 * r0, T, ptr<uint64_t>(e->hit_off), ptr<uint64_t>(e->scan_part), s);
    uint64_t h_tot = 0;
    HPG_CUDA(cudaMemcpyAsync(&h_tot, ptr<uint64_t>(e->hit_off) + T, 8, cudaMemcpyDeviceToHost, s), "hit count");
    HPG_CUDA(cudaStreamSynchronize(s), "hit scan");
    if (!ensure(e, e->hits, (n_hits + h_tot + 1) * sizeof(hpg_hit_t), true)) {
      *err = "out of device memory (hits)";
      return -1;
    }
    hpg_hit_t* hits = ptr<hpg_hit_t>(e->hits) + n_hits;
    launch_gather_hits(ptr<uint4>(e->slots), mode == HPG_BWT_MODE_SEARCH1 ? ptr<OvfEntry>(e->ovf) : nullptr,
                       ptr<uint32_t>(e->ovf_count), mode == HPG_BWT_MODE_SEARCH1 ? e->ovf_cap : 0,
                       ptr<uint32_t>(e->rs_count), ptr<uint64_t>(e->hit_off), (uint32_t)r0, nr, hits, s);
    // rows to locate
    if (!ensure(e, e->rows, (h_tot + 1) * 4) || !ensure(e, e->loc_off, (h_tot + 2) * 8) ||
        !ensure(e, e->scan_part, scan_parts(h_tot) * 8)) {
      *err = "out of device memory (locate offsets)";
      return -1;
    }
    launch_hit_rows(hits, (uint32_t)h_tot, ptr<uint32_t>(e->rows), s);
    launch_limit_rows(ptr<uint64_t>(e->hit_off), ptr<uint32_t>(e->rows), (uint32_t)T, e->locate_limit, nullptr,
                      ptr<uint8_t>(e->rs_trunc) + 2 * r0, s);
    launch_scan(ptr<uint32_t>(e->rows), h_tot, ptr<uint64_t>(e->loc_off), ptr<uint64_t>(e->scan_part), s);
    uint64_t l_tot = 0;
    HPG_CUDA(cudaMemcpyAsync(&l_tot, ptr<uint64_t>(e->loc_off) + h_tot, 8, cudaMemcpyDeviceToHost, s), "loc count");
    HPG_CUDA(cudaStreamSynchronize(s), "locate scan");
    if (census) cudaMemsetAsync(census, 0, 8, s);
    cudaEventRecord(c, s);
    if (!ensure(e, e->locs, (n_locs + l_tot + 1) * sizeof(hpg_loc_t), true)) {
      *err = oom_message(("locate output, " + std::to_string(n_locs + l_tot) + " rows").c_str(),
                         (n_locs + l_tot + 1) * sizeof(hpg_loc_t));
      return -1;
    }
    launch_locate(e->X, hits, ptr<uint64_t>(e->loc_off), (uint32_t)h_tot, l_tot, d_offs, (uint32_t)n_hits,
                  ptr<hpg_loc_t>(e->locs) + n_locs, census, s);
    cudaEventRecord(d, s);
    HPG_CUDA(cudaStreamSynchronize(s), "locate kernel");
    if (census_take() != 0) return -1;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    t_search += ms;
    cudaEventElapsedTime(&ms, b, c);
    t_final += ms;
    cudaEventElapsedTime(&ms, c, d);
    t_loc += ms;
    n_hits += h_tot;
    n_locs += l_tot;
  }
  cudaEventRecord(e->ev[kStageCount], s);
  HPG_CUDA(cudaStreamSynchronize(s), "pipeline");
  HPG_CUDA(cudaGetLastError(), "kernel launch");
  {
    uint32_t derr = 0;
    HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
    if (derr) {
      cudaMemset(e->d_err, 0, 4);
      *err = "corrupt index: suffix-array walk did not reach a sampled row";
      return -1;
    }
  }
  cudaEventElapsedTime(&e->stage_ms[kStageEncode], e->ev[0], e->ev[1]);
  e->stage_ms[kStageSearch] = t_search;
  e->stage_ms[kStageFinalize] = t_final;
  e->stage_ms[kStageLocate] = t_loc;
  DeviceResult r;
  r.n_reads = n_reads;
  r.n_hits = n_hits;
  r.hits = ptr<hpg_hit_t>(e->hits);
  r.n_locs = n_locs;
  r.locs = ptr<hpg_loc_t>(e->locs);
  r.rs_count = ptr<uint32_t>(e->rs_count);
  r.rs_truncated = ptr<uint8_t>(e->rs_trunc);
  e->last = r;
  *out = r;
  return 0;
}

int engine_copy_result(Engine* e, const DeviceResult& r, hpg_hit_t* hits, hpg_loc_t* locs, uint32_t* rs_count,
                       uint8_t* rs_truncated, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  cudaStream_t s = e->stream;
  if (hits && r.n_hits)
    HPG_CUDA(cudaMemcpyAsync(hits, r.hits, r.n_hits * sizeof(hpg_hit_t), cudaMemcpyDeviceToHost, s), "copy hits");
  if (locs && r.n_locs)
    HPG_CUDA(cudaMemcpyAsync(locs, r.locs, r.n_locs * sizeof(hpg_loc_t), cudaMemcpyDeviceToHost, s), "copy locs");
  if (rs_count && r.n_reads)
    HPG_CUDA(cudaMemcpyAsync(rs_count, r.rs_count, 2 * r.n_reads * 4, cudaMemcpyDeviceToHost, s), "copy counts");
  if (rs_truncated && r.n_reads)
    HPG_CUDA(cudaMemcpyAsync(rs_truncated, r.rs_truncated, 2 * r.n_reads, cudaMemcpyDeviceToHost, s), "copy flags");
  HPG_CUDA(cudaStreamSynchronize(s), "copy result");
  return 0;
}

namespace {

int host_result(Engine* e, const DeviceResult& r, size_t n_reads, hpg_result_set_t* out, std::string* err) {
  out->n_reads = n_reads;
  out->n_hits = r.n_hits;
  out->n_locs = r.n_locs;
  out->hits = (hpg_hit_t*)host_pool_alloc((r.n_hits + 1) * sizeof(hpg_hit_t));
  out->locs = (hpg_loc_t*)host_pool_alloc((r.n_locs + 1) * sizeof(hpg_loc_t));
  out->rs_count = (uint32_t*)host_pool_alloc((2 * n_reads + 1) * 4);
  out->rs_truncated = (uint8_t*)host_pool_alloc(2 * n_reads + 1);
  if (!out->hits || !out->locs || !out->rs_count || !out->rs_truncated) {
    *err = "out of host memory";
    return -1;
  }
  return engine_copy_result(e, r, out->hits, out->locs, out->rs_count, out->rs_truncated, err);
}

}  // namespace

int engine_search_host_keep(Engine* e, int mode, int form, const char* seqs, const uint64_t* offs, size_t n_reads,
                            uint32_t max_results, DeviceResult* r, std::string* err) {
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (n_reads && offs[n_reads] < offs[0]) {
    *err = "read offsets must be non-decreasing";
    return -1;
  }
  const uint64_t total = n_reads ? offs[n_reads] - offs[0] : 0;
  cudaStream_t s = e->stream;
  std::vector<uint64_t> rel;
  if (form == kFormBatched && mode == HPG_BWT_MODE_SEARCH1 && e->use_graph) {
    // the graph checks every read's offsets on the device (no host pass over them)
    if (n_reads >= (1ull << 31)) {
      *err = "too many reads in one batch";
      return -1;
    }
    if (total > (1ull << 40)) {
      *err = "batch too large";
      return -1;
    }
    const uint64_t* o = offs;
    if (n_reads && offs[0] != 0) {
      rel.resize(n_reads + 1);
      for (size_t i = 0; i <= n_reads; ++i) rel[i] = offs[i] - offs[0];
      o = rel.data();
    }
    static const uint64_t zero = 0;
    return finish_graph(e, seqs + (n_reads ? offs[0] : 0), n_reads ? o : &zero, (uint32_t)n_reads, total,
                        max_results, r, err);
  }
  uint32_t max_len = 0;
  for (size_t i = 0; i < n_reads; ++i) {
    if (offs[i + 1] < offs[i]) {
      *err = "read offsets must be non-decreasing";
      return -1;
    }
    const uint64_t L = offs[i + 1] - offs[i];
    if (L > 32767) {
      *err = "reads longer than 32767 bases are not supported";
      return -1;
    }
    max_len = std::max<uint32_t>(max_len, (uint32_t)L);
  }
  if (!ensure(e, e->seqs, total + 16) || !ensure(e, e->offs, (n_reads + 1) * 8)) {
    *err = "out of device memory (reads)";
    return -1;
  }
  rel.resize(n_reads + 1);
  for (size_t i = 0; i <= n_reads; ++i) rel[i] = offs[i] - offs[0];
  if (total) HPG_CUDA(cudaMemcpyAsync(e->seqs.p, seqs + offs[0], total, cudaMemcpyHostToDevice, s), "upload reads");
  HPG_CUDA(cudaMemcpyAsync(e->offs.p, rel.data(), (n_reads + 1) * 8, cudaMemcpyHostToDevice, s), "upload offsets");
  return engine_search_device(e, mode, form, ptr<uint8_t>(e->seqs), ptr<uint64_t>(e->offs), n_reads, total, max_len,
                              max_results, r, err);
}

int engine_search_host(Engine* e, int mode, int form, const char* seqs, const uint64_t* offs, size_t n_reads,
                       uint32_t max_results, hpg_result_set_t* out, std::string* err) {
  std::memset(out, 0, sizeof(*out));
  HPG_CUDA(cudaSetDevice(e->device), "cudaSetDevice");
  if (n_reads && offs[n_reads] < offs[0]) {
    *err = "read offsets must be non-decreasing";
    return -1;
  }
  // Pipelined on request only: on GB300 the copies slow the latency-bound
  // search by about as long as they take, so overlapping them gains nothing.
  const size_t pchunk = e->pipe_chunk;
  if (form == kFormBatched && mode == HPG_BWT_MODE_SEARCH1 && e->use_graph && pchunk && pchunk != SIZE_MAX &&
      n_reads >= 2 * pchunk && !e->census_on && n_reads < (1ull << 31) &&
      (n_reads ? offs[n_reads] - offs[0] : 0) <= (1ull << 40)) {
    const uint64_t total = n_reads ? offs[n_reads] - offs[0] : 0;
    if (run_graph_pipelined(e, seqs, offs, n_reads, total, max_results, out, err) != 0) {
      bwt_gpu_result_free(out);
      return -1;
    }
    uint32_t derr = 0;
    HPG_CUDA(cudaMemcpy(&derr, e->d_err, 4, cudaMemcpyDeviceToHost), "error word");
    if (derr) {
      cudaMemset(e->d_err, 0, 4);
      bwt_gpu_result_free(out);
      *err = "corrupt index: suffix-array walk did not reach a sampled row";
      return -1;
    }
    return 0;
  }
  DeviceResult r;
  if (engine_search_host_keep(e, mode, form, seqs, offs, n_reads, max_results, &r, err) != 0) return -1;
  return host_result(e, r, n_reads, out, err);
}

}  // namespace hpgbwt
