// seeds.cpp -- seeds (bwt_map_exact_seed, bwt_map_exact_seeds_seq) and
// candidate alignment locations (bwt_generate_cals) of hpg-libs' mapper
// (c/src/aligners/bwt/bwt.c), with every seed of a call searched and located
// in one GPU pass and the CALs built on the host.
//
// Device: engine_seed_search (map_device.cu) runs each seed on both strands;
// the rows the filter keeps go through engine_locate_rows.  Host: the seed
// plan, the regions, and the CAL merge of bwt.c:3631-3642, 3832-4031,
// 4378-4646 and 4652-4824, restated on std::list (the reference's linked
// lists: "insert" at the head, "insert_last" at the tail, iterator insert
// before the current item), then emitted as the reference's cal_t /
// seed_region_t records in the caller's hpg-libs containers.
#include <omp.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <list>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"
#include "hpg_bwt_api.h"

using namespace hpgbwt;

namespace {

[[noreturn]] void fatal(const std::string& what) {
  std::fprintf(stderr, "[hpgbwt] %s\n", what.c_str());
  std::exit(EXIT_FAILURE);
}

Engine* engine_for(bwt_index_t* idx) {
  Engine* e = idx ? static_cast<Engine*>(idx->gpu_) : nullptr;
  if (!e) fatal("bwt seeds: the index has no GPU context (load it with bwt_index_new)");
  return e;
}

constexpr int kMaxSeeds = 1000;  // seed ids per read (bwt.c:3640 passes 1000 as max_seeds)

// One seed of a read: bases [first, last] (both included); `valid` is false
// when the plan reaches outside the read (the reference reads past its buffer).
struct Seed {
  size_t first, last;
  int id;
  bool valid;
};

// The seed plan of bwt_map_exact_seeds_seq (bwt.c:3583-3625) and
// bwt_generate_cals (bwt.c:3863-3907), in the reference's size_t arithmetic.
std::vector<Seed> seed_plan(size_t len, size_t seed_size) {
  if (seed_size <= 10) seed_size = 16;
  const int pad = (int)(seed_size / 2);  // padding_left = padding_right
  const size_t extra = 16;               // the splice-junction seeds are 16 bases
  std::vector<Seed> out;
  int id = 0;
  auto add = [&](size_t first, size_t last) {
    out.push_back(Seed{first, last, id++, first <= last && last < len});
  };
  add((size_t)pad, (size_t)pad + extra - 1);
  const size_t num = len / seed_size;
  size_t off = 0;
  for (size_t i = 0; i < num; ++i, off += seed_size) add(off, off + seed_size - 1);
  if (len % seed_size > 0) add(len - seed_size, len - 1);
  if (len % seed_size != (size_t)pad) add(len - extra - (size_t)pad, len - (size_t)pad - 1);
  return out;
}

// The seed plan of bwt_map_exact_seeds_by_region (bwt.c:4033-4080): seeds of
// seed_size tiling [start_position, end_position) of the read, ids from 1, and
// the last seed_size bases of the window when its length is not a multiple.
std::vector<Seed> seed_plan_window(size_t read_len, int start_position, int end_position, int seed_size) {
  if (seed_size <= 10) seed_size = 16;
  const int len = end_position - start_position;
  std::vector<Seed> out;
  int id = 1;
  auto add = [&](long first, long last) {
    const bool ok = first >= 0 && first <= last && (size_t)last < read_len;
    out.push_back(Seed{ok ? (size_t)first : 0, ok ? (size_t)last : 0, id++, ok});
  };
  const int num = len / seed_size;
  long off = start_position;
  for (int i = 0; i < num; ++i, off += seed_size) add(off, off + seed_size - 1);
  if (len % seed_size > 0) add((long)end_position - seed_size, (long)end_position - 1);
  return out;
}

// A located seed (region_bwt_new's fields, bwt.c:1280).
struct Region {
  size_t chrom;  // 1-based
  int strand;    // 0 '+', 1 '-'
  size_t start, end;
  size_t seq_start, seq_end, seq_len;
  int id;
};

// Per read: ASCII bases and its seeds.
struct SeedJob {
  const char* seq;
  size_t len;
  std::vector<Seed> seeds;
};

// Regions of every seed of every job, in the reference's order (per seed:
// '+' rows by row, then '-' rows), bwt_map_exact_seed (bwt.c:1200-1294).
std::vector<std::vector<std::vector<Region>>> map_seeds(Engine* e, const std::vector<SeedJob>& jobs,
                                                        int filter_seed_mappings) {
  std::string seq;
  std::vector<uint64_t> offs{0};
  std::vector<uint32_t> spec;  // {read, first, last, 0}
  std::vector<std::pair<size_t, size_t>> where;  // (job, seed) of every searched seed
  for (size_t j = 0; j < jobs.size(); ++j) {
    seq.append(jobs[j].seq, jobs[j].len);
    offs.push_back(seq.size());
    for (size_t s = 0; s < jobs[j].seeds.size(); ++s) {
      const Seed& sd = jobs[j].seeds[s];
      if (!sd.valid) continue;
      spec.insert(spec.end(), {(uint32_t)j, (uint32_t)sd.first, (uint32_t)sd.last, 0u});
      where.emplace_back(j, s);
    }
  }
  std::string err;
  std::vector<uint32_t> kl(4 * where.size() + 4);
  if (!where.empty() && engine_seed_search(e, seq.data(), offs.data(), jobs.size(), spec.data(), where.size(),
                                           kl.data(), &err) != 0)
    fatal(err);
  // rows the reference locates: a strand adds its rows to the count and is
  // located unless the count passed the filter (bwt.c:1256-1268)
  struct RowOf {
    uint32_t w;  // index into `where`
    int type;    // 1 '+', 0 '-'
  };
  // the strands each seed locates (bit 1 '+', bit 0 '-') and its row count,
  // then the rows of every seed at its prefix-sum offset (seeds in parallel)
  const size_t W = where.size();
  std::vector<uint8_t> keep(W);
  std::vector<uint64_t> first_row(W + 1, 0);
#pragma omp parallel for schedule(static)
  for (size_t w = 0; w < W; ++w) {
    int actual = 0;
    uint8_t kept = 0;
    uint64_t n_rows = 0;
    for (int type = 1; type >= 0; --type) {
      const uint32_t k = kl[4 * w + (type ? 0 : 2)], l = kl[4 * w + (type ? 1 : 3)];
      actual += (int)((int64_t)l - (int64_t)k + 1);
      if (actual > filter_seed_mappings || k > l) continue;
      kept |= (uint8_t)(1u << type);
      n_rows += (uint64_t)l - k + 1;
    }
    keep[w] = kept;
    first_row[w + 1] = n_rows;
  }
  for (size_t w = 0; w < W; ++w) first_row[w + 1] += first_row[w];
  const size_t n_rows = first_row[W];
  std::vector<MapRow> rows(n_rows + 1);
  std::vector<RowOf> row_of(n_rows + 1);
#pragma omp parallel for schedule(static)
  for (size_t w = 0; w < W; ++w) {
    const Seed& sd = jobs[where[w].first].seeds[where[w].second];
    const uint32_t len = (uint32_t)(sd.last - sd.first);
    uint64_t at = first_row[w];
    for (int type = 1; type >= 0; --type) {
      if (!(keep[w] & (1u << type))) continue;
      const uint32_t k = kl[4 * w + (type ? 0 : 2)], l = kl[4 * w + (type ? 1 : 3)];
      for (uint64_t j = k; j <= l; ++j, ++at) {
        rows[at] = MapRow{(uint32_t)j, 0u, len};
        row_of[at] = RowOf{(uint32_t)w, type};
      }
    }
  }
  std::vector<hpg_loc_t> loc(n_rows + 1);
  if (n_rows && engine_locate_rows(e, rows.data(), n_rows, loc.data(), &err) != 0) fatal(err);
  // regions per job (jobs in parallel; a job's seeds, and so its rows, are contiguous)
  std::vector<size_t> job_first(jobs.size() + 1, W);
  for (size_t w = W; w-- > 0;) job_first[where[w].first] = w;
  for (size_t j = jobs.size(); j-- > 0;)
    if (job_first[j] > job_first[j + 1]) job_first[j] = job_first[j + 1];
  std::vector<std::vector<std::vector<Region>>> out(jobs.size());
#pragma omp parallel for schedule(dynamic, 256)
  for (size_t job = 0; job < jobs.size(); ++job) {
    out[job].resize(jobs[job].seeds.size());
    const size_t n = jobs[job].len;
    for (uint64_t r = first_row[job_first[job]]; r < first_row[job_first[job + 1]]; ++r) {
      const hpg_loc_t& q = loc[r];
      if (!q.valid) continue;
      const size_t s = where[row_of[r].w].second;
      const Seed& sd = jobs[job].seeds[s];
      const size_t len = sd.last - sd.first;
      const int type = row_of[r].type;
      Region g;
      g.chrom = (size_t)q.chrom + 1;
      g.strand = !type;
      g.start = (size_t)q.position + 1;
      g.end = g.start + len;
      g.seq_start = type ? sd.first : n - sd.last - 1;
      g.seq_end = type ? sd.last : n - sd.first - 1;
      g.seq_len = n;
      g.id = sd.id;
      out[job][s].push_back(g);
    }
  }
  return out;
}

region_t* to_region(const Region& g) {
  region_t* r = region_bwt_new(g.chrom, (short)g.strand, g.start, g.end, g.seq_start, g.seq_end, g.seq_len, g.id);
  if (!r) fatal("out of host memory");
  return r;
}

// ---- CAL merge (restated from bwt.c on std::list) -------------------------

struct SeedReg {
  int read_start, read_end;
  size_t genome_start, genome_end;
  int id;
};

struct ShortCal {
  size_t start, end, num_seeds;
  std::list<SeedReg> sr, dup;  // front = the linked list's first item
  std::vector<uint8_t> seen;   // seeds_ids_array (unsigned char counters), one per seed id of the read
};
using CalList = std::list<ShortCal>;

// short_cal_new (bwt.c:319-342); the reference's table has 1000 entries, of
// which a read uses its seed ids only (`ids`).
ShortCal new_short_cal(const Region& g, size_t ids) {
  if (g.id >= kMaxSeeds) fatal("seed id past the CAL seed table (1000 seeds per read)");
  ShortCal c;
  c.start = g.start;
  c.end = g.end;
  c.num_seeds = 1;
  c.seen.assign(ids, 0);
  c.seen[g.id] = 1;
  c.sr.push_front(SeedReg{(int)g.seq_start, (int)g.seq_end, g.start, g.end, g.id});
  return c;
}

// seed_region_select_linked_list (bwt.c:4378-4409): the first seed of an id
// joins the CAL's seeds; from the second on, the first moves to the
// duplicate list and every later one joins it.
void select_seed(ShortCal& c, const SeedReg& s) {
  uint8_t& seen = c.seen[s.id];
  if (!seen) {
    ++seen;
    c.sr.push_front(s);
    return;
  }
  if (seen == 1) {
    for (auto it = c.sr.begin(); it != c.sr.end(); ++it)
      if (it->id == s.id) {
        c.dup.push_front(*it);
        c.sr.erase(it);
        break;
      }
  }
  c.dup.push_front(s);
  ++seen;
}

// my_cp_list_append_linked_list (bwt.c:4652-4824): one region into the
// CAL list of its strand and chromosome, kept ordered by start; CALs within
// `dist` of each other merge.
void add_region(CalList& L, const Region& g, size_t dist, size_t ids) {
  if (L.empty()) {
    L.push_front(new_short_cal(g, ids));
    return;
  }
  const SeedReg s{(int)g.seq_start, (int)g.seq_end, g.start, g.end, g.id};
  bool grown = false;
  auto it = L.begin();
  for (; it != L.end(); ++it) {
    if (g.start < it->start) {
      if (g.end + dist < it->start) {  // a new CAL before this one
        L.insert(it, new_short_cal(g, ids));
      } else {  // this CAL now starts at the region
        it->start = g.start;
        it->num_seeds++;
        select_seed(*it, s);
        if (g.end > it->end) {
          it->end = g.end;
          grown = true;
        }
      }
      break;
    }
    if (g.end <= it->end) {  // inside this CAL
      it->num_seeds++;
      select_seed(*it, s);
      break;
    }
    if (it->end + dist >= g.start) {  // extends this CAL's end
      it->end = g.end;
      select_seed(*it, s);
      grown = true;
      it->num_seeds++;
      break;
    }
  }
  if (it == L.end()) {
    L.push_back(new_short_cal(g, ids));
    return;
  }
  if (!grown) return;
  // the grown CAL absorbs the following ones it now reaches; their duplicate
  // lists are dropped, their seeds move over only if they reach further
  auto nx = std::next(it);
  while (nx != L.end()) {
    if (it->end + dist < nx->start) break;
    if (it->end < nx->end) {
      it->end = nx->end;
      while (!nx->sr.empty()) {
        const SeedReg moved = nx->sr.front();
        nx->sr.pop_front();
        select_seed(*it, moved);
      }
    }
    nx = L.erase(nx);
  }
}

// append_seed_region_linked_list (bwt.c:4453-4646) without error lists: a
// CAL's seeds kept ordered by genome start, touching or overlapping seeds merged.
void append_seed(std::list<SeedReg>& L, const SeedReg& s) {
  if (L.empty()) {
    L.push_front(s);
    return;
  }
  bool grown = false;
  auto it = L.begin();
  for (; it != L.end(); ++it) {
    if (s.genome_start < it->genome_start) {
      if (s.genome_end + 1 < it->genome_start) {
        L.insert(it, s);
      } else {
        it->read_start = s.read_start;
        it->genome_start = s.genome_start;
        if (s.genome_end > it->genome_end) {
          it->read_end = s.read_end;
          it->genome_end = s.genome_end;
          grown = true;
        }
      }
      break;
    }
    if (s.genome_end <= it->genome_end) break;
    if (it->genome_end + 1 >= s.genome_start) {
      it->read_end = s.read_end;
      it->genome_end = s.genome_end;
      grown = true;
      break;
    }
  }
  if (it == L.end()) {
    L.push_back(s);
    return;
  }
  if (!grown) return;
  auto nx = std::next(it);
  while (nx != L.end()) {
    if (it->genome_end + 1 < nx->genome_start) break;
    if (it->genome_end + 1 < nx->genome_end) {
      it->read_end = nx->read_end;
      it->genome_end = nx->genome_end;
    }
    nx = L.erase(nx);
  }
}

seed_region_t* to_seed_region(const SeedReg& s, int id) {
  seed_region_t* r = seed_region_new(s.read_start, s.read_end, s.genome_start, s.genome_end, id, 0, 0);
  if (!r) fatal("out of host memory");
  return r;
}

linked_list_t* to_linked_list(const std::list<SeedReg>& L) {
  linked_list_t* out = linked_list_new(COLLECTION_MODE_ASYNCHRONIZED);
  if (!out) fatal("out of host memory");
  for (const SeedReg& s : L) linked_list_insert_last(to_seed_region(s, s.id), out);
  return out;
}

// bwt_generate_cals for one read (bwt.c:3832-4031), its regions given per seed.
void build_cals(const std::vector<std::vector<Region>>& regions, size_t read_length, size_t seed_size,
                const cal_optarg_t* cal_optarg, unsigned int nchromosomes, array_list_t* cal_list) {
  if (seed_size <= 10) seed_size = 16;
  const size_t nchrom = (size_t)nchromosomes + 1;
  std::vector<CalList> lists(2 * nchrom);  // [strand * nchrom + chromosome]
  const size_t ids = regions.size();  // seed ids of this read: 0 .. ids - 1
  for (const auto& seed_regions : regions)  // insert_seeds_and_merge: each seed's regions, last first
    for (auto g = seed_regions.rbegin(); g != seed_regions.rend(); ++g) {
      if (g->chrom >= nchrom) fatal("bwt_generate_cals: a seed mapped past nchromosomes");
      add_region(lists[(size_t)g->strand * nchrom + g->chrom], *g, read_length, ids);
    }
  const size_t min_cal_size = cal_optarg->min_cal_size;
  const int max_intron_size = (int)cal_optarg->max_intron_size;
  for (size_t j = 0; j < nchrom; ++j)
    for (size_t i = 0; i < 2; ++i) {
      CalList& L = lists[i * nchrom + j];
      for (auto c = L.begin(); c != L.end(); ++c) {
        if (c->end - c->start + 1 < min_cal_size) continue;
        std::list<SeedReg> merged;
        while (!c->sr.empty()) {
          const SeedReg s = c->sr.back();
          c->sr.pop_back();
          append_seed(merged, s);
        }
        linked_list_t* dup = to_linked_list(c->dup);
        c->dup.clear();
        cal_t* cal = cal_new(j, (short)i, c->start, c->end, c->num_seeds, to_linked_list(merged), dup);
        if (!cal) fatal("out of host memory");
        array_list_insert(cal, cal_list);
        if (merged.empty()) continue;
        const SeedReg first = merged.front(), last = merged.back();
        // seeds of the smaller CALs just before this one that lie before its
        // first seed in the read, and just after it beyond its last
        if ((size_t)first.read_start >= seed_size) {
          for (auto p = c; p != L.begin();) {
            --p;
            if (p->end - p->start + 1 >= min_cal_size || c->start - p->end >= (size_t)max_intron_size) break;
            for (const SeedReg& s : p->sr)
              if (s.read_end < first.read_start) array_list_insert(to_seed_region(s, 0), cal->candidates_seeds_start);
          }
        }
        if ((size_t)last.read_end < read_length - seed_size) {
          for (auto p = std::next(c); p != L.end(); ++p) {
            if (p->end - p->start + 1 >= min_cal_size || p->start - c->end >= (size_t)max_intron_size) break;
            for (const SeedReg& s : p->sr)
              if (s.read_start > last.read_end) array_list_insert(to_seed_region(s, 1), cal->candidates_seeds_end);
          }
        }
      }
    }
}

}  // namespace

extern "C" {

cal_optarg_t* cal_optarg_new(const size_t min_cal_size, const size_t max_cal_distance, const size_t num_seeds,
                             const size_t min_num_seeds_in_cal, const size_t seed_size, const size_t min_seed_size,
                             const size_t num_errors, const size_t max_intron_size, const size_t min_intron_size) {
  cal_optarg_t* o = static_cast<cal_optarg_t*>(std::calloc(1, sizeof(cal_optarg_t)));
  if (!o) return nullptr;
  o->min_cal_size = min_cal_size;
  o->max_cal_distance = max_cal_distance;
  o->num_seeds = num_seeds;
  o->min_num_seeds_in_cal = min_num_seeds_in_cal;
  o->seed_size = seed_size;
  o->min_seed_size = min_seed_size;
  o->num_errors = num_errors;
  o->max_intron_size = max_intron_size;
  o->min_intron_size = min_intron_size;
  return o;
}

void cal_optarg_free(cal_optarg_t* optarg) { std::free(optarg); }

seed_region_t* seed_region_new(int read_start, int read_end, size_t genome_start, size_t genome_end, int id,
                               int pos_err, int type_err) {
  seed_region_t* s = static_cast<seed_region_t*>(std::calloc(1, sizeof(seed_region_t)));
  if (!s) return nullptr;
  s->read_start = read_start;
  s->read_end = read_end;
  s->genome_start = genome_start;
  s->genome_end = genome_end;
  s->id = id;
  s->pos_err = pos_err;
  s->type_err = type_err;
  return s;
}

void seed_region_free(seed_region_t* s) {
  if (!s) return;
  std::free(s->info);
  if (s->errors_list) array_list_free(s->errors_list, std::free);
  std::free(s);
}

cal_t* cal_new(const size_t chromosome_id, const short int strand, const size_t start, const size_t end,
               const size_t num_seeds, linked_list_t* sr_list, linked_list_t* sr_duplicate_list) {
  cal_t* c = static_cast<cal_t*>(std::calloc(1, sizeof(cal_t)));
  if (!c) return nullptr;
  c->chromosome_id = chromosome_id;
  c->strand = strand;
  c->start = start;
  c->end = end;
  c->num_seeds = num_seeds;
  c->sr_list = sr_list;
  c->sr_duplicate_list = sr_duplicate_list;
  c->candidates_seeds_start = array_list_new(10, 1.25f, COLLECTION_MODE_ASYNCHRONIZED);
  c->candidates_seeds_end = array_list_new(10, 1.25f, COLLECTION_MODE_ASYNCHRONIZED);
  // the read span of the seeds: last seed's end - first seed's start (bwt.c:202-209)
  const seed_region_t* first = sr_list ? static_cast<const seed_region_t*>(linked_list_get_first(sr_list)) : nullptr;
  const seed_region_t* last = sr_list ? static_cast<const seed_region_t*>(linked_list_get_last(sr_list)) : nullptr;
  if (first && last) c->read_area += last->read_end - first->read_start;
  return c;
}

void cal_free(cal_t* c) {
  if (!c) return;
  auto free_seed = [](void* p) { seed_region_free(static_cast<seed_region_t*>(p)); };
  if (c->sr_list) linked_list_free(c->sr_list, free_seed);
  if (c->sr_duplicate_list) linked_list_free(c->sr_duplicate_list, free_seed);
  if (c->candidates_seeds_start) array_list_free(c->candidates_seeds_start, free_seed);
  if (c->candidates_seeds_end) array_list_free(c->candidates_seeds_end, free_seed);
  std::free(c);
}

region_t* region_bwt_new(const size_t chromosome_id, const short int strand, const size_t start, const size_t end,
                         const size_t seq_start, const size_t seq_end, const size_t seq_len, const int id) {
  region_t* r = static_cast<region_t*>(std::calloc(1, sizeof(region_t)));
  if (!r) return nullptr;
  r->chromosome_id = chromosome_id;
  r->strand = strand;
  r->start = start;
  r->end = end;
  r->seq_start = seq_start;
  r->seq_end = seq_end;
  r->seq_len = seq_len;
  r->id = id;
  return r;
}

void region_bwt_free(region_t* region) { std::free(region); }

size_t bwt_map_exact_seed(uint8_t* seq, size_t seq_len, size_t seq_start, size_t seq_end, bwt_optarg_t* bwt_optarg,
                          bwt_index_t* index, array_list_t* mapping_list, int id) {
  std::lock_guard<std::mutex> lk(map_api_mutex());
  Engine* e = engine_for(index);
  // the seed arrives as codes: back to bases through the index's alphabet
  const char* alphabet = index->bwt_config.nucleotides;
  const size_t na = alphabet ? std::strlen(alphabet) : 0;
  std::string ascii(seq_len, 'N');
  for (size_t i = 0; i < seq_len; ++i)
    if (seq[i] < na) ascii[i] = alphabet[seq[i]];
  SeedJob job{ascii.data(), seq_len, {Seed{seq_start, seq_end, id, seq_start <= seq_end && seq_end < seq_len}}};
  const auto regions = map_seeds(e, {job}, bwt_optarg->filter_seed_mappings);
  for (const Region& g : regions[0][0]) array_list_insert(to_region(g), mapping_list);
  return regions[0][0].size();
}

size_t bwt_map_exact_seeds_seq(int padding_left, int padding_right, char* seq, size_t seed_size, size_t min_seed_size,
                               bwt_optarg_t* bwt_optarg, bwt_index_t* index, array_list_t* mapping_list,
                               unsigned char step_id) {
  (void)padding_left;
  (void)padding_right;
  (void)min_seed_size;
  (void)step_id;
  std::lock_guard<std::mutex> lk(map_api_mutex());
  Engine* e = engine_for(index);
  const size_t len = std::strlen(seq);
  SeedJob job{seq, len, seed_plan(len, seed_size)};
  const auto regions = map_seeds(e, {job}, bwt_optarg->filter_seed_mappings);
  for (const auto& per_seed : regions[0])
    for (const Region& g : per_seed) array_list_insert(to_region(g), mapping_list);
  return array_list_size(mapping_list);
}

size_t bwt_map_exact_seeds_by_region(int start_position, int end_position, char* seq, int seed_size,
                                     int min_seed_size, bwt_optarg_t* bwt_optarg, bwt_index_t* index,
                                     array_list_t* mapping_list) {
  (void)min_seed_size;
  std::lock_guard<std::mutex> lk(map_api_mutex());
  Engine* e = engine_for(index);
  const size_t len = std::strlen(seq);
  SeedJob job{seq, len, seed_plan_window(len, start_position, end_position, seed_size)};
  const auto regions = map_seeds(e, {job}, bwt_optarg->filter_seed_mappings);
  for (const auto& per_seed : regions[0])
    for (const Region& g : per_seed) array_list_insert(to_region(g), mapping_list);
  return array_list_size(mapping_list);
}

size_t bwt_generate_cals(char* seq, size_t seed_size, bwt_optarg_t* bwt_optarg, cal_optarg_t* cal_optarg,
                         bwt_index_t* index, array_list_t* cal_list, unsigned int nchromosomes) {
  bwt_generate_cals_batch(&seq, 1, seed_size, bwt_optarg, cal_optarg, index, &cal_list, nchromosomes);
  return array_list_size(cal_list);
}

size_t bwt_generate_cals_batch(char** seqs, size_t num_reads, size_t seed_size, bwt_optarg_t* bwt_optarg,
                               cal_optarg_t* cal_optarg, bwt_index_t* index, array_list_t** cal_lists,
                               unsigned int nchromosomes) {
  std::vector<std::vector<std::vector<Region>>> regions;
  std::vector<SeedJob> jobs(num_reads);
  {
    std::lock_guard<std::mutex> lk(map_api_mutex());
    Engine* e = engine_for(index);
    for (size_t i = 0; i < num_reads; ++i) {
      const size_t len = std::strlen(seqs[i]);
      jobs[i] = SeedJob{seqs[i], len, seed_plan(len, seed_size)};
    }
    regions = map_seeds(e, jobs, bwt_optarg->filter_seed_mappings);
  }
  size_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (size_t i = 0; i < num_reads; ++i) {
    build_cals(regions[i], jobs[i].len, seed_size, cal_optarg, nchromosomes, cal_lists[i]);
    total += array_list_size(cal_lists[i]);
  }
  return total;
}

}  // extern "C"
