// api.cpp -- the drop-in C ABI: index lifetime, options and GPU batch search.
#include <cuda_runtime.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "engine.hpp"
#include "fm_device.cuh"
#include "kernels.cuh"
#include "hpg_bwt.h"
#include "index_format.hpp"
#include "serve.hpp"
#include "host_pool.hpp"

using namespace hpgbwt;

namespace hpgbwt {
DevIndex engine_dev_index(void* engine);
const uint8_t* engine_code_table(void* engine);
int gather_ceiling(int device, size_t bytes, uint32_t blocks, uint32_t steps, double* sectors_per_s,
                   std::string* err, uint32_t work);
}

namespace {

thread_local std::string g_last_error;

int fail(const std::string& msg) {
  g_last_error = msg;
  return -1;
}

Engine* engine_of(bwt_index_t* idx) { return idx ? static_cast<Engine*>(idx->gpu_) : nullptr; }

// The reference's exome (search/io.c:3-16,26-81) filled from the index file.
exome* make_exome(const Karyotype& k) {
  exome* ex = (exome*)std::calloc(1, sizeof(exome));
  const size_t n = k.name.size();
  ex->max_chromosomes = (int)(n + 1);
  ex->size = n;
  ex->chromosome = (char*)std::calloc((n + 1) * IDMAX, 1);
  ex->start = (uintmax_t*)std::calloc(n + 1, sizeof(uintmax_t));
  ex->end = (uintmax_t*)std::calloc(n + 1, sizeof(uintmax_t));
  ex->offset = (uintmax_t*)std::calloc(n + 1, sizeof(uintmax_t));
  for (size_t i = 0; i < n; ++i) {
    std::snprintf(ex->chromosome + i * IDMAX, IDMAX, "%s", k.name[i].c_str());
    ex->start[i] = k.start[i];
    ex->end[i] = k.end[i];
  }
  for (size_t i = 0; i <= n; ++i) ex->offset[i] = k.offset[i];
  return ex;
}

void free_exome(exome* ex) {
  if (!ex) return;
  std::free(ex->chromosome);
  std::free(ex->start);
  std::free(ex->end);
  std::free(ex->offset);
  std::free(ex);
}

// bwt_init_replace_table (bwt_commons.c:60-92).
void fill_config(bwt_config_t* c, const std::string& letters, bool inverse_sa) {
  std::memset(c, 0, sizeof(*c));
  c->nA = (uint8_t)letters.size();
  c->table = (uint8_t*)std::malloc(256);
  std::memset(c->table, 0xFF, 256);
  c->nucleotides = (char*)std::calloc(c->nA + 1, 1);
  c->reverse = (char*)std::calloc(c->nA + 1, 1);
  for (int i = 0; i < c->nA; ++i) {
    const char u = (char)std::toupper((unsigned char)letters[i]);
    c->nucleotides[i] = u;
    c->table[(unsigned char)u] = (uint8_t)i;
    c->table[(unsigned char)std::tolower((unsigned char)u)] = (uint8_t)i;
    if (u == 'A') c->AA = (uint8_t)i;
    else if (u == 'C') c->CC = (uint8_t)i;
    else if (u == 'G') c->GG = (uint8_t)i;
    else if (u == 'T') c->TT = (uint8_t)i;
  }
  c->reverse[c->AA] = (char)c->TT;
  c->reverse[c->CC] = (char)c->GG;
  c->reverse[c->GG] = (char)c->CC;
  c->reverse[c->TT] = (char)c->AA;
  c->inverse_sa = inverse_sa;
  c->duplicate_strand = false;  // always read as 0 (search/io.c:357-358)
}

}  // namespace

extern "C" {

const char* bwt_gpu_last_error(void) { return g_last_error.c_str(); }

bwt_index_t* bwt_index_open(const char* dirname, bool inverse_sa, int device, char* errbuf, size_t errlen) {
  auto report = [&](const std::string& m) -> bwt_index_t* {
    g_last_error = m;
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", m.c_str());
    return nullptr;
  };
  if (!dirname) return report("null index directory");
  HostIndex* h = new HostIndex();
  std::string e = read_host_index(dirname, inverse_sa, h);
  if (!e.empty()) {
    delete h;
    return report(e);
  }
  if (device < 0) {
    if (cudaGetDevice(&device) != cudaSuccess) {
      cudaGetLastError();
      device = 0;
    }
  }
  Engine* en = engine_create(*h, device, &e);
  if (!en) {
    delete h;
    return report(e);
  }
  bwt_index_t* idx = (bwt_index_t*)std::calloc(1, sizeof(bwt_index_t));
  idx->karyotype = make_exome(h->kar);
  fill_config(&idx->bwt_config, h->alphabet, inverse_sa);
  idx->dirname = strdup(dirname);
  idx->gpu_ = en;
  delete h;  // the GPU copy is authoritative; the karyotype lives in idx->karyotype
  return idx;
}

bwt_index_t* bwt_index_new(const char* dirname, bool inverse_sa) {
  char err[1024];
  bwt_index_t* idx = bwt_index_open(dirname, inverse_sa, -1, err, sizeof err);
  if (!idx) {
    std::fprintf(stderr, "bwt_index_new: %s\n", err);
    std::exit(EXIT_FAILURE);
  }
  return idx;
}

void bwt_index_free(bwt_index_t* index) {
  if (!index) return;
  engine_destroy(engine_of(index));
  free_exome(index->karyotype);
  std::free(index->bwt_config.table);
  std::free(index->bwt_config.nucleotides);
  std::free(index->bwt_config.reverse);
  std::free(index->dirname);
  std::free(index);
}

bwt_optarg_t* bwt_optarg_new(const size_t num_errors, const size_t num_threads, const int filter_read_mappings,
                             const int filter_seed_mappings) {
  bwt_optarg_t* o = (bwt_optarg_t*)std::malloc(sizeof(bwt_optarg_t));
  o->num_errors = num_errors;
  o->num_threads = num_threads;
  o->filter_read_mappings = filter_read_mappings;
  o->filter_seed_mappings = filter_seed_mappings;
  return o;
}

void bwt_optarg_free(bwt_optarg_t* optarg) { std::free(optarg); }

int bwt_gpu_search_batch(bwt_index_t* index, int mode, int form, const char* seqs, const uint64_t* offsets,
                         size_t n_reads, uint32_t max_results, hpg_result_set_t* out) {
  Engine* e = engine_of(index);
  if (!e || !out || (n_reads && (!seqs || !offsets))) return fail("bwt_gpu_search_batch: null argument");
  std::string err;
  if (engine_search_host(e, mode, form, seqs, offsets, n_reads, max_results, out, &err) != 0) return fail(err);
  return 0;
}

int bwt_gpu_block_search(bwt_index_t* index, const char* seqs, const uint64_t* offsets, size_t n_reads,
                         uint32_t max_results, hpg_result_set_t* out, hpg_block_anchor_t* anchors,
                         uint8_t* n_anchors) {
  Engine* e = engine_of(index);
  if (!e || !out || (n_reads && (!seqs || !offsets))) return fail("bwt_gpu_block_search: null argument");
  std::string err;
  if (engine_block_search_result(e, seqs, offsets, n_reads, max_results, out, anchors, n_anchors, &err) != 0) {
    bwt_gpu_result_free(out);
    return fail(err);
  }
  return 0;
}

float bwt_gpu_block_search_ms(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_block_ms(e) : 0.0f;
}

void bwt_gpu_result_free(hpg_result_set_t* out) {
  if (!out) return;
  host_pool_free(out->hits);
  host_pool_free(out->locs);
  host_pool_free(out->rs_count);
  host_pool_free(out->rs_truncated);
  std::memset(out, 0, sizeof(*out));
}

int bwt_gpu_search_device(bwt_index_t* index, int mode, int form, const uint8_t* d_seqs, const uint64_t* d_offsets,
                          size_t n_reads, uint64_t total_bases, uint32_t max_len, uint32_t max_results,
                          hpg_result_set_t* out) {
  Engine* e = engine_of(index);
  if (!e || !out) return fail("bwt_gpu_search_device: null argument");
  std::string err;
  DeviceResult r;
  if (engine_search_device(e, mode, form, d_seqs, d_offsets, n_reads, total_bases, max_len, max_results, &r, &err) !=
      0)
    return fail(err);
  out->n_reads = r.n_reads;
  out->n_hits = r.n_hits;
  out->hits = const_cast<hpg_hit_t*>(r.hits);
  out->n_locs = r.n_locs;
  out->locs = const_cast<hpg_loc_t*>(r.locs);
  out->rs_count = const_cast<uint32_t*>(r.rs_count);
  out->rs_truncated = const_cast<uint8_t*>(r.rs_truncated);
  return 0;
}

int bwt_gpu_copy_result(bwt_index_t* index, const hpg_result_set_t* dev, hpg_hit_t* hits, hpg_loc_t* locs,
                        uint32_t* rs_count, uint8_t* rs_truncated) {
  Engine* e = engine_of(index);
  if (!e || !dev) return fail("bwt_gpu_copy_result: null argument");
  DeviceResult r;
  r.n_reads = dev->n_reads;
  r.n_hits = dev->n_hits;
  r.hits = dev->hits;
  r.n_locs = dev->n_locs;
  r.locs = dev->locs;
  r.rs_count = dev->rs_count;
  r.rs_truncated = dev->rs_truncated;
  std::string err;
  if (engine_copy_result(e, r, hits, locs, rs_count, rs_truncated, &err) != 0) return fail(err);
  return 0;
}

void* bwt_gpu_stream(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_stream(e) : nullptr;
}

void bwt_gpu_stage_ms(bwt_index_t* index, float* out, int n) {
  Engine* e = engine_of(index);
  if (e && out) engine_stage_ms(e, out, n);
}

void bwt_gpu_set_census(bwt_index_t* index, int on) {
  Engine* e = engine_of(index);
  if (e) engine_set_census(e, on);
}

unsigned long long bwt_gpu_census(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_census(e) : 0ull;
}

unsigned long long bwt_gpu_launch_count(void) { return launch_count(); }

int bwt_gpu_gather_ceiling(int device, size_t bytes, uint32_t blocks, uint32_t steps, double* sectors_per_s) {
  std::string err;
  if (!sectors_per_s || gather_ceiling(device, bytes, blocks, steps, sectors_per_s, &err, 0) != 0)
    return fail(err.empty() ? "bwt_gpu_gather_ceiling: null argument" : err);
  return 0;
}

size_t bwt_gpu_index_bytes(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_index_bytes(e) : 0;
}

void bwt_gpu_set_tuning(bwt_index_t* index, int min_blocks, int blocks_per_sm, int stack_depth,
                        int chains_per_claim) {
  Engine* e = engine_of(index);
  if (e) engine_set_tuning(e, min_blocks, blocks_per_sm, stack_depth, chains_per_claim);
}

void bwt_gpu_get_tuning(bwt_index_t* index, int* out5) {
  Engine* e = engine_of(index);
  if (e && out5) engine_get_tuning(e, out5);
}

void bwt_gpu_set_load_mode(bwt_index_t* index, int mode) {
  Engine* e = engine_of(index);
  if (e) engine_set_load_mode(e, mode);
}

int bwt_gpu_load_mode(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_load_mode(e) : -1;
}

void bwt_gpu_set_graph(bwt_index_t* index, int on) {
  Engine* e = engine_of(index);
  if (e) engine_set_graph(e, on);
}

void bwt_gpu_set_direction_split(bwt_index_t* index, int mode) {
  Engine* e = engine_of(index);
  if (e) engine_set_dir_split(e, mode);
}

int bwt_gpu_direction_split(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_dir_split(e) : -1;
}

double bwt_gpu_map_device_seconds(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_map_device_seconds(e) : 0.0;
}

void bwt_gpu_set_wave_group(bwt_index_t* index, int reads) {
  Engine* e = engine_of(index);
  if (e) engine_set_wave_group(e, reads);
}

int bwt_gpu_wave_group(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_wave_group(e) : -1;
}

void bwt_gpu_set_idle_batch(bwt_index_t* index, int lanes) {
  Engine* e = engine_of(index);
  if (e) engine_set_idle_batch(e, lanes);
}

int bwt_gpu_idle_batch(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_idle_batch(e) : -1;
}

void bwt_gpu_set_locate_limit(bwt_index_t* index, uint64_t max_rows) {
  Engine* e = engine_of(index);
  if (e) engine_set_locate_limit(e, max_rows);
}

uint64_t bwt_gpu_locate_limit(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_locate_limit(e) : 0;
}

int bwt_gpu_set_start_table(bwt_index_t* index, int symbols) {
  Engine* e = engine_of(index);
  if (!e) return fail("bwt_gpu_set_start_table: null index");
  std::string err;
  if (engine_set_kmer(e, symbols, &err) != 0) return fail(err);
  return 0;
}

int bwt_gpu_start_table(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_kmer(e) : -1;
}

void bwt_gpu_set_pipeline_chunk(bwt_index_t* index, size_t reads) {
  Engine* e = engine_of(index);
  if (e) engine_set_pipeline_chunk(e, reads);
}

int bwt_gpu_graph(bwt_index_t* index) {
  Engine* e = engine_of(index);
  return e ? engine_graph(e) : -1;
}

int bwt_gpu_autotune(bwt_index_t* index, const uint8_t* d_seqs, const uint64_t* d_offsets, size_t n_reads,
                     uint64_t total_bases, uint32_t max_len, uint32_t max_results, int* table, int max_rows,
                     int* rows) {
  Engine* e = engine_of(index);
  if (!e) return fail("bwt_gpu_autotune: null index");
  std::string err;
  if (engine_autotune(e, d_seqs, d_offsets, n_reads, total_bases, max_len, max_results, table, max_rows, rows,
                      &err) != 0)
    return fail(err);
  return 0;
}

bwt_gpu_server_t* bwt_gpu_server_new(bwt_index_t* index, size_t max_batch_reads, uint64_t max_batch_bases,
                                     uint64_t hbm_budget_bytes, uint32_t max_results) {
  Engine* e = engine_of(index);
  if (!e) {
    fail("bwt_gpu_server_new: null index");
    return nullptr;
  }
  std::string err;
  Server* s = server_create(e, max_batch_reads, max_batch_bases, hbm_budget_bytes, max_results, &err);
  if (!s) fail(err);
  return reinterpret_cast<bwt_gpu_server_t*>(s);
}

int bwt_gpu_server_submit(bwt_gpu_server_t* server, const char* seqs, const uint64_t* offsets, size_t n_reads,
                          uint64_t* ticket) {
  if (!server || !ticket) return fail("bwt_gpu_server_submit: null argument");
  std::string err;
  if (server_submit(reinterpret_cast<Server*>(server), seqs, offsets, n_reads, ticket, &err) != 0) return fail(err);
  return 0;
}

int bwt_gpu_server_wait(bwt_gpu_server_t* server, uint64_t ticket, hpg_result_set_t* view, double* latency_ms,
                        int timeout_ms) {
  if (!server) return fail("bwt_gpu_server_wait: null server");
  std::string err;
  const int rc = server_wait(reinterpret_cast<Server*>(server), ticket, view, latency_ms, timeout_ms, &err);
  if (rc < 0) return fail(err);
  return rc;
}

int bwt_gpu_server_release(bwt_gpu_server_t* server, uint64_t ticket) {
  if (!server) return fail("bwt_gpu_server_release: null server");
  std::string err;
  if (server_release(reinterpret_cast<Server*>(server), ticket, &err) != 0) return fail(err);
  return 0;
}

void bwt_gpu_server_stats(bwt_gpu_server_t* server, double* out, int n) {
  if (server && out) server_stats(reinterpret_cast<Server*>(server), out, n);
}

void bwt_gpu_server_free(bwt_gpu_server_t* server) { server_destroy(reinterpret_cast<Server*>(server)); }

void bwt_gpu_set_chunk(bwt_index_t* index, size_t reads) {
  Engine* e = engine_of(index);
  if (e) engine_set_chunk(e, reads);
}

}  // extern "C"
