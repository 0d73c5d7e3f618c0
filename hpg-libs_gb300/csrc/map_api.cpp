// map_api.cpp -- the alignment-list entry points of c/src/aligners/bwt/bwt.c
// (bwt_map_exact_*, bwt_map_inexact_*), served by the GPU passes of the engine.
//
// Every call maps its reads as one batch: the search on the device (the exact
// pair of bwt_map_exact_seq, or BWSearch1 with hits only), then the host picks
// the suffix-array rows the reference would locate (interval cap, mapping
// filter), one device pass locates them, and the alignment records are built
// here with the reference's field values, order and quirks.  Anchors
// (bwt.c:1822-1869) take one more scan and locate pass for the reads that end
// without alignments in a list flagged 1.
#include <algorithm>
#include <charconv>
#include <chrono>
#include <memory>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"
#include "hpg_bwt_api.h"

using namespace hpgbwt;

namespace {

std::mutex& g_mu = map_api_mutex();

[[noreturn]] void fatal(const std::string& what) {
  // the reference's fatal path (bwt_commons.h:48-70): report and exit
  std::fprintf(stderr, "[hpgbwt] %s\n", what.c_str());
  std::exit(EXIT_FAILURE);
}

Engine* engine_for(bwt_index_t* idx) {
  Engine* e = idx ? static_cast<Engine*>(idx->gpu_) : nullptr;
  if (!e) fatal("bwt_map: the index has no GPU context (load it with bwt_index_new)");
  return e;
}

char* dup_bytes(const char* s, size_t n) {
  char* p = static_cast<char*>(std::malloc(n + 1));
  if (!p) fatal("out of host memory");
  if (n) std::memcpy(p, s, n);
  p[n] = '\0';
  return p;
}

char* dup_str(const char* s) { return dup_bytes(s, std::strlen(s)); }

double wall_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Time split of a call, printed to stderr when HPG_BWT_TIMING is set in the
// environment (a diagnostic for tuning the host side; silent otherwise).
struct Stopwatch {
  const char* what;
  bool on;
  double t;
  explicit Stopwatch(const char* w) : what(w), on(std::getenv("HPG_BWT_TIMING") != nullptr), t(wall_seconds()) {}
  void mark(const char* step) {
    if (!on) return;
    const double now = wall_seconds();
    std::fprintf(stderr, "[hpgbwt] %s: %s %.2f ms\n", what, step, (now - t) * 1e3);
    t = now;
  }
};

// "<len>M" (bwt.c:2125-2130) without printf.
char* cigar_match(size_t len) {
  char buf[24];
  const auto r = std::to_chars(buf, buf + sizeof buf - 2, (unsigned long)len);
  *r.ptr = 'M';
  return dup_bytes(buf, (size_t)(r.ptr - buf) + 1);
}

char* fmt(const char* f, unsigned long v) {
  char buf[48];
  std::snprintf(buf, sizeof buf, f, v);
  return dup_str(buf);
}

// Reads of one call, concatenated for the device passes.
struct Reads {
  std::string seq;
  std::vector<uint64_t> offs{0};
  void add(const char* s, size_t n) {
    seq.append(s, n);
    offs.push_back(seq.size());
  }
  size_t n() const { return offs.size() - 1; }
  size_t len(size_t i) const { return offs[i + 1] - offs[i]; }
};

// alignment_init_single_end (alignment.c:12-42) on a zeroed alignment_new().
alignment_t* new_alignment(char* qname, char* seq, char* qual, int strand, unsigned chrom, int pos, char* cigar,
                           int ncigar, int mapq, int mapped, int secondary) {
  alignment_t* a = alignment_new();
  if (!a) fatal("out of host memory");
  a->query_name = qname;
  a->sequence = seq;
  a->quality = qual;
  a->cigar = cigar;
  a->chromosome = chrom;
  a->position = pos;
  a->mate_position = -1;
  a->mate_chromosome = -1;
  a->template_length = 0;
  a->map_quality = mapq;
  a->num_cigar_operations = ncigar;
  a->is_paired_end = 0;
  a->is_paired_end_mapped = 0;
  a->is_seq_mapped = (uint8_t)mapped;
  a->is_mate_mapped = 0;
  a->seq_strand = (uint8_t)strand;
  a->mate_strand = 0;
  a->pair_num = 0;
  a->secondary_alignment = (uint8_t)secondary;
  a->fails_quality_check = 0;
  a->pc_optical_duplicate = 0;
  a->optional_fields = nullptr;
  a->optional_fields_length = 0;
  a->map_len = 0;
  a->alig_data = nullptr;
  return a;
}

// get_to_first_blank (commons/string_utils.c:400-428): skip a leading '@',
// stop at ' ' or '/' or after `length` bytes.
char* first_blank(const char* s, size_t length) {
  char* out = static_cast<char*>(std::malloc(length + 2));
  if (!out) fatal("out of host memory");
  size_t i = s[0] == '@' ? 1 : 0, o = 0;
  while (i < length && s[i] != ' ' && s[i] != '/') out[o++] = s[i++];
  out[o] = '\0';
  return out;
}

// ----------------------------------------------------------------- exact --

// bwt_map_exact_seq (bwt.c:889-981) for every read: alignments in the
// reference's order, '+' first.
std::vector<std::vector<alignment_t*>> exact_alignments(Engine* e, const Reads& R, const bwt_optarg_t* opt) {
  const size_t n = R.n();
  std::string err;
  std::vector<uint32_t> kl(4 * n + 4);
  if (engine_exact_api(e, R.seq.data(), R.offs.data(), n, kl.data(), &err) != 0) fatal(err);
  const size_t filter = (size_t)(long)opt->filter_read_mappings;
  const uint64_t top = engine_sa_top(e);
  struct Span {
    size_t k, l;
  };
  std::vector<Span> span(2 * n);
  std::vector<uint8_t> rc(n, 0);
  std::vector<MapRow> rows;
  for (size_t r = 0; r < n; ++r) {
    size_t k_aux = 0, l_aux = 0;
    for (int type = 1; type >= 0; --type) {
      const size_t k = type ? kl[4 * r] : kl[4 * r + 2], l = type ? kl[4 * r + 1] : kl[4 * r + 3];
      if (type == 0) rc[r] = (l_aux - k_aux + 1 < filter) ? 1 : 0;  // tested on the '+' interval (bwt.c:936)
      k_aux = k;
      l_aux = l;
      if (l_aux - k_aux + 1 >= filter) l_aux = k_aux + 1;  // bwt.c:945-947
      span[2 * r + (type ? 0 : 1)] = Span{k_aux, l_aux};
      for (size_t j = k_aux; j <= l_aux && j <= top; ++j)  // rows past the array are not read
        rows.push_back(MapRow{(uint32_t)j, 0u, (uint32_t)R.len(r)});
    }
  }
  std::vector<hpg_loc_t> loc(rows.size() + 1);
  if (engine_locate_rows(e, rows.data(), rows.size(), loc.data(), &err) != 0) fatal(err);
  std::vector<std::vector<alignment_t*>> out(n);
  size_t at = 0;
  for (size_t r = 0; r < n; ++r) {
    const size_t len = R.len(r);
    std::string strand_seq(R.seq.data() + R.offs[r], len);
    unsigned num = 0;
    for (int type = 1; type >= 0; --type) {
      if (type == 0 && rc[r]) seq_reverse_complementary(&strand_seq[0], (unsigned)len);
      const Span sp = span[2 * r + (type ? 0 : 1)];
      for (size_t j = sp.k; j <= sp.l && j <= top; ++j, ++at) {
        const hpg_loc_t& L = loc[at];
        if (!L.valid) continue;
        out[r].push_back(new_alignment(nullptr, dup_bytes(strand_seq.data(), len), nullptr, !type, L.chrom,
                                       (int)(unsigned)L.position, fmt("%lu=", (unsigned long)len), 1, 254, 1,
                                       num > 0));
        ++num;
      }
    }
  }
  return out;
}

void announce(size_t n) {  // bwt.c:894 prints one line per mapped sequence
  for (size_t i = 0; i < n; ++i) std::fputs("\tIn function ...\n", stdout);
}

// --------------------------------------------------------------- inexact --

struct InexactRead {
  const char* id;
  const char* seq;
  size_t len;
  const char* revcomp;  // may be null: computed here
  const char* quality;
};

// The output list of one read: the caller's array_list_t, or a fresh list
// (batch forms) whose items the caller collects.
struct OutList {
  array_list_t* list = nullptr;
  // a fresh list: first `cap` items in slots (a caller's flat array), any more in `fresh`
  void** slots = nullptr;
  uint32_t nslots = 0, cap = 0;
  std::vector<void*> fresh;
  int fresh_flag = 0;
  size_t size() { return list ? array_list_size(list) : nslots + fresh.size(); }
  void* get(size_t i) { return list ? array_list_get(i, list) : (i < nslots ? slots[i] : fresh[i - nslots]); }
  void insert(void* p) {
    if (list) array_list_insert(p, list);
    else if (nslots < cap) slots[nslots++] = p;
    else fresh.push_back(p);
  }
  int flag() { return list ? array_list_get_flag(list) : fresh_flag; }
  void set_flag(int f) {
    if (list) array_list_set_flag(f, list);
    else fresh_flag = f;
  }
};

// bwt_cigar_cpy (bwt.c:501-547): the read quality, reversed on the '-' strand.
void quality_copy(alignment_t* a, const char* quality) {
  const size_t n = std::strlen(quality);
  std::free(a->quality);
  a->quality = static_cast<char*>(std::malloc(n + 1));
  if (!a->quality) fatal("out of host memory");
  if (a->seq_strand == 0) {
    std::memcpy(a->quality, quality, n);
    a->quality[n] = '\0';
  } else {
    reverse_str(const_cast<char*>(quality), a->quality, n);
  }
}

// add_optional_fields (bwt.c:3065-3100): AS, NH and NM as 3-byte tags with
// 4-byte values; map quality becomes 255.
void optional_fields(alignment_t* a, size_t n_mappings, int read_length) {
  const int distance = a->map_quality;
  int as = (int)(read_length * 1 - distance * 0.4);
  as = as * 100 / read_length;
  char* f = static_cast<char*>(std::calloc(100, 1));
  if (!f) fatal("out of host memory");
  const uint32_t nh = (uint32_t)n_mappings;
  std::memcpy(f, "ASi", 3);
  std::memcpy(f + 3, &as, 4);
  std::memcpy(f + 7, "NHi", 3);
  std::memcpy(f + 10, &nh, 4);
  std::memcpy(f + 14, "NMi", 3);
  std::memcpy(f + 17, &distance, 4);
  a->map_quality = 255;
  std::free(a->optional_fields);
  a->optional_fields = reinterpret_cast<uint8_t*>(f);
  a->optional_fields_length = 21;
}

struct InexactOutcome {
  size_t added = 0;       // alignments this call put in the list
  bool anchors = false;   // list ended empty with flag 1
};

// The flat slot array of the last map_inexact call's fresh lists (the calls
// hold the entry points' lock, so one array serves them).
std::unique_ptr<void*[]> g_flat_slots;

// Alignments of one read into its list (bwt.c:1896-2289, without the
// anchors), from the records the device decided: which rows, in which order,
// with which flags (engine_inexact_records).  Only the records' allocation and
// their strings are made here.
InexactOutcome assemble_inexact(const InexactRead& rd, uint32_t n_rec, const MapRec* rec, uint8_t flags,
                                OutList& L) {
  InexactOutcome res;
  const size_t len = rd.len;
  if (len < 5) {  // bwt.c:1900-1917
    L.insert(new_alignment(nullptr, dup_bytes(rd.seq, len), fmt("%lu", 0), 0, (unsigned)-1, -1,
                           fmt("%luX", (unsigned long)len), 1, 0, 0, 0));
    res.added = 1;
    return res;
  }
  std::string rc_store;
  const char* minus_seq = rd.revcomp;
  for (uint32_t r = 0; r < n_rec; ++r) {
    const int strand = (int)(rec[r].chrom_strand >> 31);
    if (strand && !minus_seq) {  // the '-' strand's sequence (bwt.c:2003-2006)
      rc_store.assign(rd.seq, len);
      seq_reverse_complementary(&rc_store[0], (unsigned)len);
      minus_seq = rc_store.data();
    }
    L.insert(new_alignment(dup_str(rd.id), dup_bytes(strand ? minus_seq : rd.seq, len), nullptr, strand,
                           rec[r].chrom_strand & 0x7FFFFFFFu, rec[r].position, cigar_match(len), 1, 0,
                           1, r > 0));
  }
  if (flags & 1) L.set_flag(2);  // bwt.c:2180-2184
  if (flags & 2) static_cast<alignment_t*>(L.get(0))->secondary_alignment = 0;  // bwt.c:2234-2237
  res.added = n_rec;
  if (L.size() == 0) {
    res.anchors = L.flag() == 1;
  } else {
    for (size_t i = 0; i < L.size(); ++i) {
      alignment_t* a = static_cast<alignment_t*>(L.get(i));
      quality_copy(a, rd.quality);
      optional_fields(a, n_rec, (int)len);
    }
    L.set_flag(0);
  }
  return res;
}

// Maps reads into their lists; returns per read what was added.
std::vector<InexactOutcome> map_inexact(Engine* e, const std::vector<InexactRead>& rds, const bwt_optarg_t* opt,
                                        std::vector<OutList*>& lists) {
  const size_t n = rds.size();
  std::string err;
  Stopwatch sw("map_inexact");
  // 1. reads of 5+ bases, concatenated for the device
  std::vector<uint32_t> gidx(n, UINT32_MAX);
  std::vector<uint64_t> offs(1, 0);
  offs.reserve(n + 1);
  for (size_t i = 0; i < n; ++i)
    if (rds[i].len >= 5) {
      gidx[i] = (uint32_t)(offs.size() - 1);
      offs.push_back(offs.back() + rds[i].len);
    }
  const size_t m = offs.size() - 1;
  std::unique_ptr<char[]> seq(new char[offs.back() + 1]);
#pragma omp parallel for schedule(static) if (n > 4096)
  for (size_t i = 0; i < n; ++i)
    if (gidx[i] != UINT32_MAX) std::memcpy(seq.get() + offs[gidx[i]], rds[i].seq, rds[i].len);
  sw.mark("reads concatenated");
  // 2. the search, the rows, the merge and the order, on the device
  InexactRecords R;
  const double t0 = wall_seconds();
  if (engine_inexact_records(e, seq.get(), offs.data(), m, opt->filter_read_mappings, &R, &err) != 0) fatal(err);
  engine_note_map_device_seconds(e, wall_seconds() - t0);
  sw.mark("device pass");
  // 3. alignment records, read by read (fresh lists get their slots in one
  // flat array, sized from the records the device decided)
  std::vector<uint64_t> slot0(n + 1, 0);
  for (size_t i = 0; i < n; ++i)
    slot0[i + 1] = slot0[i] + (lists[i]->list ? 0 : (gidx[i] == UINT32_MAX ? 1 : R.n_rec[gidx[i]]));
  std::unique_ptr<void*[]> flat(new void*[slot0[n] + 1]);
  for (size_t i = 0; i < n; ++i)
    if (!lists[i]->list) {
      lists[i]->slots = flat.get() + slot0[i];
      lists[i]->cap = (uint32_t)(slot0[i + 1] - slot0[i]);
    }
  std::vector<InexactOutcome> out(n);
  // reads in parallel when each read's records go to a list of its own (a
  // caller's list named for two reads would take unlocked inserts from two threads)
  bool own_lists = true;
  {
    std::vector<const void*> seen;
    for (size_t i = 0; i < n; ++i)
      if (lists[i]->list) seen.push_back(lists[i]->list);
    std::sort(seen.begin(), seen.end());
    own_lists = std::adjacent_find(seen.begin(), seen.end()) == seen.end();
  }
#pragma omp parallel for schedule(dynamic, 256) if (own_lists && n > 256)
  for (size_t i = 0; i < n; ++i) {
    const uint32_t g = gidx[i];
    if (g == UINT32_MAX) {
      out[i] = assemble_inexact(rds[i], 0, nullptr, 0, *lists[i]);
      continue;
    }
    if (R.flags[g] & 4) fatal("too many rows to locate for one read");
    out[i] = assemble_inexact(rds[i], R.n_rec[g], R.rec.data() + R.rec_off[g], R.flags[g], *lists[i]);
  }
  sw.mark("records allocated");
  g_flat_slots = std::move(flat);
  std::vector<MapRow> rows;
  std::vector<hpg_loc_t> loc;
  // 4. anchors for reads left without alignments in a list flagged 1 (bwt.c:2243-2273)
  std::vector<uint32_t> need;
  Reads A;
  for (size_t i = 0; i < n; ++i)
    if (out[i].anchors) {
      need.push_back((uint32_t)A.n());
      A.add(rds[i].seq, rds[i].len);
    }
  if (need.empty()) return out;
  std::vector<uint32_t> ends(16 * need.size());
  if (engine_anchor_scan(e, A.seq.data(), A.offs.data(), A.n(), need.data(), need.size(), ends.data(), &err) != 0)
    fatal(err);
  struct Want {
    size_t read;
    int type, kind;
    uint32_t nt;
  };
  std::vector<Want> wants;
  rows.clear();
  size_t a = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!out[i].anchors) continue;
    for (int c = 0; c < 4; ++c) {  // '+' BACKWARD, '+' FORWARD, '-' BACKWARD, '-' FORWARD
      const uint32_t* v = &ends[16 * a + 4 * c];
      const uint32_t nt = v[0];
      const size_t k = v[1], l = v[2];
      const int kind = (c == 0 || c == 2) ? BACKWARD_ANCHOR : FORWARD_ANCHOR;
      if (nt == 0 || !(l - k < 50)) continue;  // at most 50 rows (bwt.c:1851)
      for (size_t j = k; j <= l; ++j) {
        rows.push_back(MapRow{(uint32_t)j, (uint32_t)kind, nt, 1});
        wants.push_back(Want{i, c < 2 ? 1 : 0, kind, nt});
      }
    }
    ++a;
  }
  loc.assign(rows.size() + 1, hpg_loc_t{});
  if (engine_locate_rows(e, rows.data(), rows.size(), loc.data(), &err) != 0) fatal(err);
  for (size_t w = 0; w < wants.size(); ++w) {
    if (!loc[w].valid) continue;
    const Want& W = wants[w];
    lists[W.read]->insert(bwt_anchor_new(!W.type, (int)loc[w].chrom, loc[w].position + 1,
                                         loc[w].position + W.nt, W.kind));
  }
  return out;
}

// ------------------------------------------------ inexact, block search --

// The cigar of one block-search result and its operation count
// (bwt.c:2513-2610); false for an error kind the reference skips.
bool block_cigar(int error, int pos, size_t len, int type, int dir, char* cigar, size_t cap, int* nops) {
  const unsigned long n = (unsigned long)len;
  const size_t last = len - 1;
  if (error == 0) {
    std::snprintf(cigar, cap, "%lu=", n);
    *nops = 1;
  } else if (error == HPG_BWT_MISMATCH) {
    if (pos == 0) {
      std::snprintf(cigar, cap, type ? "1S%luM" : "%luM1S", n - 1);
      *nops = 2;
    } else if ((size_t)pos == last) {
      std::snprintf(cigar, cap, type ? "%luM1S" : "1S%luM", n - 1);
      *nops = 2;
    } else {
      std::snprintf(cigar, cap, "%luM", n);
      *nops = 1;
    }
  } else if (error == HPG_BWT_INSERTION) {
    if (pos == 0) {
      std::snprintf(cigar, cap, type ? "1M1D%luM" : "%luM1D1M", n - 1);
    } else if ((size_t)pos == last) {
      std::snprintf(cigar, cap, type ? "%luM1D1M" : "1M1D%luM", n - 1);
    } else if (type) {
      if (dir) std::snprintf(cigar, cap, "%iM1D%luM", pos, n - (unsigned long)pos);
      else std::snprintf(cigar, cap, "%iM1D%luM", pos + 1, n - (unsigned long)pos - 1);
    } else {
      if (dir) std::snprintf(cigar, cap, "%luM1D%dM", n - (unsigned long)pos, pos);
      else std::snprintf(cigar, cap, "%luM1D%dM", n - (unsigned long)pos - 1, pos + 1);
    }
    *nops = 3;
  } else if (error == HPG_BWT_DELETION) {
    if (pos == 0) {
      std::snprintf(cigar, cap, type ? "1I%luM" : "%luM1I", n - 1);
      *nops = 2;
    } else if ((size_t)pos == last) {
      std::snprintf(cigar, cap, type ? "%luM1I" : "1I%luM", n - 1);
      *nops = 2;
    } else {
      if (type) std::snprintf(cigar, cap, "%dM1I%luM", pos, n - (unsigned long)pos - 1);
      else std::snprintf(cigar, cap, "%luM1I%dM", n - (unsigned long)pos - 1, pos);
      *nops = 3;
    }
  } else {
    return false;
  }
  return true;
}

// Per read after the block search: the results each type maps until the
// row filter is passed, and where their located rows start.
struct BlockPlan {
  int exceeded_type = -1;  // type whose results passed the filter (the loop stops there)
  size_t hit0[2] = {0, 0};  // first result of each type in the result array
  size_t nres[2] = {0, 0};  // results of each type that are mapped
  size_t row0[2] = {0, 0};  // first located row of each type
  size_t anchor_t = 0;      // item index of type 1 (type 0 is anchor_t + 1)
};

// Alignments of one read into its list (bwt.c:2313-2780, the anchors after).
InexactOutcome assemble_block(const InexactRead& rd, const BlockPlan& P, const BlockSearchOut& B, const hpg_loc_t* loc,
                              OutList& L) {
  InexactOutcome res;
  const size_t len = rd.len;
  if (len < 5) {  // bwt.c:2321-2337
    L.insert(new_alignment(nullptr, dup_bytes(rd.seq, len), fmt("%lu", 0), 0, (unsigned)-1, -1,
                           fmt("%luX", (unsigned long)len), 1, 0, 0, 0));
    res.added = 1;
    return res;
  }
  std::string rc_store;
  const char* strand_seq = rd.seq;
  size_t num = 0;
  for (int type = 1; type >= 0; --type) {
    const size_t t = P.anchor_t + (type ? 0 : 1);
    if (type == 0 && B.count[t]) {  // bwt.c:2477-2479
      if (rd.revcomp) {
        strand_seq = rd.revcomp;
      } else {
        rc_store.assign(rd.seq, len);
        seq_reverse_complementary(&rc_store[0], (unsigned)len);
        strand_seq = rc_store.data();
      }
    }
    std::vector<alignment_t*> tmp;
    size_t at = P.row0[type];
    for (size_t h = 0; h < P.nres[type]; ++h) {
      const hpg_hit_t& x = B.hits[P.hit0[type] + h];
      const int error = x.nm ? x.err_kind : 0;
      char cigar[96];
      int nops = 0;
      if (!block_cigar(error, x.err_pos, len, type, x.dir, cigar, sizeof cigar, &nops)) continue;
      for (int64_t j = x.k; j <= x.l; ++j, ++at) {
        const hpg_loc_t& q = loc[at];
        if (!q.valid) continue;
        tmp.push_back(new_alignment(nullptr, dup_bytes(strand_seq, len), fmt("%lu", 0), !type, q.chrom,
                                    (int)(q.position + 1), dup_str(cigar), nops, 254, 1, num > 0));
      }
    }
    if (P.exceeded_type == type) {  // bwt.c:2628-2633, 2655-2659 (its alignments were never made)
      L.set_flag(2);
      break;
    }
    // alignments closer than 10 bp on one chromosome (bwt.c:2661-2710)
    const int nm = (int)tmp.size();
    std::vector<uint8_t> del(nm, 0);
    for (int a1 = nm - 1; a1 >= 1; --a1) {
      if (del[a1]) continue;
      for (int a2 = a1 - 1; a2 >= 0; --a2) {
        const size_t dist = (size_t)std::abs(tmp[a1]->position - tmp[a2]->position);
        if (tmp[a1]->chromosome == tmp[a2]->chromosome && dist < 10 && !del[a2]) {
          if (tmp[a1]->num_cigar_operations < tmp[a2]->num_cigar_operations) del[a2] = 1;
          else del[a1] = 1;
        }
      }
    }
    bool primary_delete = false;
    for (int m = nm - 1; m >= 0; --m) {
      alignment_t* a = tmp[m];
      if (del[m]) {
        if (!a->secondary_alignment) primary_delete = true;
        alignment_free(a);
      } else {
        L.insert(a);
        a->secondary_alignment = num > 0;
        ++num;
      }
    }
    if (primary_delete) static_cast<alignment_t*>(L.get(0))->secondary_alignment = 0;
  }
  res.added = num;
  if (L.size() == 0) {
    res.anchors = L.flag() == 1;
  } else {  // bwt.c:2756-2772
    const size_t idlen = std::strlen(rd.id);
    for (size_t i = 0; i < L.size(); ++i) {
      alignment_t* a = static_cast<alignment_t*>(L.get(i));
      std::free(a->query_name);
      a->query_name = first_blank(rd.id, idlen);
      quality_copy(a, rd.quality);
      optional_fields(a, num, (int)len);
    }
    L.set_flag(0);
  }
  return res;
}

// bwt_map_inexact_read_2 (bwt.c:2313-2797) for every read; one block search
// and one locate pass for all of them, anchors in a third pass.
std::vector<InexactOutcome> map_block(Engine* e, const std::vector<InexactRead>& rds, const bwt_optarg_t* opt,
                                      std::vector<OutList*>& lists) {
  const size_t n = rds.size();
  std::string err;
  const int fr = opt->filter_read_mappings;
  // the reference's result lists hold filter_read_mappings results (bwt.c:2396-2400);
  // a negative filter is a failed allocation there
  if (fr < 0) fatal("bwt_map_inexact_read_2: filter_read_mappings is negative (result lists cannot be allocated)");
  const size_t filter = (size_t)fr;
  // 1. the block search for reads of 5+ bases
  Reads R;
  std::vector<uint32_t> gidx(n, UINT32_MAX);
  for (size_t i = 0; i < n; ++i)
    if (rds[i].len >= 5) {
      gidx[i] = (uint32_t)R.n();
      R.add(rds[i].seq, rds[i].len);
    }
  BlockSearchOut B;
  if (engine_block_search(e, R.seq.data(), R.offs.data(), R.n(), (uint32_t)fr, &B, &err) != 0) fatal(err);
  std::vector<uint64_t> item0(2 * R.n() + 1, 0);
  for (size_t t = 0; t < 2 * R.n(); ++t) item0[t + 1] = item0[t] + B.count[t];
  // 2. rows to locate: results in order until the rows passed the filter (bwt.c:2618-2634)
  std::vector<BlockPlan> plan(n);
  std::vector<MapRow> rows;
  for (size_t i = 0; i < n; ++i) {
    if (gidx[i] == UINT32_MAX) continue;
    BlockPlan& P = plan[i];
    const size_t g = gidx[i];
    P.anchor_t = 2 * g;
    size_t tot = 0;
    for (int type = 1; type >= 0; --type) {
      const size_t t = 2 * g + (type ? 0 : 1);
      P.hit0[type] = item0[t];
      P.row0[type] = rows.size();
      for (uint64_t h = item0[t]; h < item0[t + 1]; ++h) {
        const hpg_hit_t& x = B.hits[h];
        tot += (size_t)(x.l - x.k);
        if (tot > filter) {  // that type's alignments are dropped: nothing of it to locate
          P.exceeded_type = type;
          P.nres[type] = 0;
          rows.resize(P.row0[type]);
          break;
        }
        ++P.nres[type];
        const int error = x.nm ? x.err_kind : 0;
        uint32_t len_calc = (uint32_t)rds[i].len;
        if (error == HPG_BWT_DELETION) --len_calc;
        else if (error == HPG_BWT_INSERTION) ++len_calc;
        const uint32_t phys = (uint32_t)x.dir ^ (uint32_t)(type ? 0 : 1);  // direction = type ? dir : !dir
        for (int64_t j = x.k; j <= x.l; ++j) rows.push_back(MapRow{(uint32_t)j, phys, len_calc});
      }
      if (P.exceeded_type >= 0) break;
    }
  }
  std::vector<hpg_loc_t> loc(rows.size() + 1);
  if (engine_locate_rows(e, rows.data(), rows.size(), loc.data(), &err) != 0) fatal(err);
  // 3. alignment records, reads in parallel when each has a list of its own
  std::vector<InexactOutcome> out(n);
  bool own_lists = true;
  {
    std::vector<const void*> seen;
    for (size_t i = 0; i < n; ++i)
      if (lists[i]->list) seen.push_back(lists[i]->list);
    std::sort(seen.begin(), seen.end());
    own_lists = std::adjacent_find(seen.begin(), seen.end()) == seen.end();
  }
#pragma omp parallel for schedule(dynamic, 256) if (own_lists && n > 256)
  for (size_t i = 0; i < n; ++i) out[i] = assemble_block(rds[i], plan[i], B, loc.data(), *lists[i]);
  // 4. anchors of reads left without alignments in a list flagged 1 (bwt.c:2737-2754):
  //    the anchors BWSearchCPU left, '+' then '-', each located by
  //    __bwt_generate_anchor_list (bwt.c:1822-1869) when it spans at most 50 rows
  struct Want {
    size_t read;
    int type, kind;
    uint32_t nt;
  };
  std::vector<Want> wants;
  rows.clear();
  for (size_t i = 0; i < n; ++i) {
    if (!out[i].anchors || gidx[i] == UINT32_MAX) continue;
    const size_t len = rds[i].len;
    for (int type = 1; type >= 0; --type) {
      const size_t t = plan[i].anchor_t + (type ? 0 : 1);
      for (uint32_t a = 0; a < B.n_anchors[t]; ++a) {
        const hpg_block_anchor_t& x = B.anchors[2 * t + a];
        int kind;
        if ((size_t)(int64_t)x.end == len - 1) kind = type ? BACKWARD_ANCHOR : FORWARD_ANCHOR;
        else if (x.start == 0) kind = type ? FORWARD_ANCHOR : BACKWARD_ANCHOR;
        else continue;
        const uint32_t nt = (uint32_t)(x.end - x.start + 1);
        const size_t k = (size_t)x.k, l = (size_t)x.l;
        if (!(l - k < 50)) continue;
        for (size_t j = k; j <= l; ++j) {
          rows.push_back(MapRow{(uint32_t)j, (uint32_t)kind, nt, 1});
          wants.push_back(Want{i, type, kind, nt});
        }
      }
    }
  }
  if (wants.empty()) return out;
  loc.assign(rows.size() + 1, hpg_loc_t{});
  if (engine_locate_rows(e, rows.data(), rows.size(), loc.data(), &err) != 0) fatal(err);
  for (size_t w = 0; w < wants.size(); ++w) {
    if (!loc[w].valid) continue;
    const Want& W = wants[w];
    lists[W.read]->insert(bwt_anchor_new(!W.type, (int)loc[w].chrom, loc[w].position + 1,
                                         loc[w].position + W.nt, W.kind));
  }
  return out;
}

InexactRead read_of(const fastq_read_t* r) {
  return InexactRead{r->id, r->sequence, std::strlen(r->sequence), r->revcomp, r->quality};
}

}  // namespace

extern "C" {

bwt_anchor_t* bwt_anchor_new(int strand, int chromosome, size_t start, size_t end, int type) {
  bwt_anchor_t* a = static_cast<bwt_anchor_t*>(std::malloc(sizeof(bwt_anchor_t)));
  if (!a) fatal("out of host memory");
  a->strand = strand;
  a->chromosome = chromosome;
  a->start = start;
  a->end = end;
  a->type = type;
  return a;
}

void bwt_anchor_free(bwt_anchor_t* a) { std::free(a); }

void seq_reverse_complementary(char* seq, unsigned int len) {
  for (unsigned i = 0, j = len ? len - 1 : 0; len && i <= j; ++i, --j) {
    auto comp = [](char c) -> char {
      switch (c) {
        case 'A': case 'a': return 'T';
        case 'C': case 'c': return 'G';
        case 'G': case 'g': return 'C';
        case 'T': case 't': return 'A';
        default: return 'N';
      }
    };
    const char a = comp(seq[i]), b = comp(seq[j]);
    seq[i] = b;
    seq[j] = a;
    if (j == 0) break;
  }
}

char* reverse_str(char* src, char* dsp, size_t length) {
  for (size_t i = 0; i < length; ++i) dsp[i] = src[length - 1 - i];
  dsp[length] = '\0';
  return dsp;
}

size_t bwt_map_exact_seq(char* seq, bwt_optarg_t* opt, bwt_index_t* index, array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  announce(1);
  Reads R;
  R.add(seq, std::strlen(seq));
  auto al = exact_alignments(e, R, opt);
  for (alignment_t* a : al[0]) array_list_insert(a, mapping_list);
  return al[0].size();
}

size_t bwt_map_exact_read(fastq_read_t* read, bwt_optarg_t* opt, bwt_index_t* index, array_list_t* mapping_list) {
  const size_t padding = array_list_size(mapping_list);
  const size_t n = bwt_map_exact_seq(read->sequence, opt, index, mapping_list);
  const size_t qlen = std::strlen(read->quality) + 1;  // bwt.c:1014-1024, terminator included
  for (size_t i = 0; i < n; ++i) {
    alignment_t* m = static_cast<alignment_t*>(array_list_get(i + padding, mapping_list));
    if (!m) continue;
    m->query_name = first_blank(read->id, std::strlen(read->id) + 1);
    m->quality = static_cast<char*>(std::malloc(qlen + 1));
    if (!m->quality) fatal("out of host memory");
    if (m->seq_strand == 0) std::memcpy(m->quality, read->quality, qlen);
    else reverse_str(read->quality, m->quality, qlen);  // reverses the terminator to the front, as bwt.c does
    m->quality[qlen - 1] = '\0';
  }
  return n;
}

size_t bwt_map_exact_seqs(char** seqs, size_t num_reads, bwt_optarg_t* opt, bwt_index_t* index, char* out_status,
                          array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  announce(num_reads);
  Reads R;
  for (size_t i = 0; i < num_reads; ++i) R.add(seqs[i], std::strlen(seqs[i]));
  auto al = exact_alignments(e, R, opt);
  for (size_t i = 0; i < num_reads; ++i) {
    out_status[i] = al[i].empty() ? 0 : 1;
    for (alignment_t* a : al[i]) array_list_insert(a, mapping_list);
  }
  return array_list_size(mapping_list);
}

size_t bwt_map_exact_batch(fastq_batch_t* batch, bwt_optarg_t* opt, bwt_index_t* index,
                           fastq_batch_t* unmapped_batch, array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  const size_t n = batch->num_reads;
  announce(n);
  Reads R;
  for (size_t i = 0; i < n; ++i) {
    const char* s = batch->seq + batch->data_indices[i];
    R.add(s, std::strlen(s));
  }
  auto al = exact_alignments(e, R, opt);
  // bwt.c:1134-1172: names and qualities from the batch, unmapped reads copied out
  size_t u = 0;
  unmapped_batch->header_indices[0] = 0;
  unmapped_batch->data_indices[0] = 0;
  for (size_t i = 0; i < n; ++i) {
    const size_t hlen = (size_t)(batch->header_indices[i + 1] - batch->header_indices[i]);
    const size_t qlen = (size_t)(batch->data_indices[i + 1] - batch->data_indices[i]);
    if (!al[i].empty()) {
      for (alignment_t* m : al[i]) {
        m->query_name = first_blank(batch->header + batch->header_indices[i], hlen);
        m->quality = static_cast<char*>(std::malloc(qlen + 1));
        if (!m->quality) fatal("out of host memory");
        std::memcpy(m->quality, batch->quality + batch->data_indices[i], qlen);
        m->quality[qlen] = '\0';
        array_list_insert(m, mapping_list);
      }
    } else {
      ++u;
      std::memcpy(unmapped_batch->header + unmapped_batch->header_indices[u - 1],
                  batch->header + batch->header_indices[i], hlen);
      std::memcpy(unmapped_batch->seq + unmapped_batch->data_indices[u - 1], batch->seq + batch->data_indices[i],
                  qlen);
      std::memcpy(unmapped_batch->quality + unmapped_batch->data_indices[u - 1],
                  batch->quality + batch->data_indices[i], qlen);
      unmapped_batch->data_indices[u] = unmapped_batch->data_indices[u - 1] + (int)qlen;
      unmapped_batch->header_indices[u] = unmapped_batch->header_indices[u - 1] + (int)hlen;
    }
  }
  unmapped_batch->num_reads = u;
  return array_list_size(mapping_list);
}

size_t bwt_map_inexact_read(fastq_read_t* read, bwt_optarg_t* opt, bwt_index_t* index, array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  std::vector<InexactRead> rds{read_of(read)};
  OutList L;
  L.list = mapping_list;
  std::vector<OutList*> lists{&L};
  map_inexact(e, rds, opt, lists);
  if (rds[0].len < 5) return 1;  // bwt.c:1917
  return array_list_size(mapping_list);
}

size_t bwt_map_inexact_batch(fastq_batch_t* batch, bwt_optarg_t* opt, bwt_index_t* index,
                             fastq_batch_t* unmapped_batch, array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  const size_t n = batch->num_reads;
  Stopwatch sw("bwt_map_inexact_batch");
  std::vector<InexactRead> rds(n);
#pragma omp parallel for schedule(static) if (n > 4096)
  for (size_t i = 0; i < n; ++i) {
    const char* s = batch->seq + batch->data_indices[i];
    rds[i] = InexactRead{batch->header + batch->header_indices[i], s, std::strlen(s), nullptr,
                         batch->quality + batch->data_indices[i]};
  }
  sw.mark("reads");
  std::vector<OutList> L(n);
  std::vector<OutList*> lists(n);
  for (size_t i = 0; i < n; ++i) lists[i] = &L[i];
  map_inexact(e, rds, opt, lists);
  sw.mark("map_inexact");
  // the records into the caller's list, in read order; the unmapped reads'
  // slots in the unmapped batch (indices first, then the copies in parallel)
  std::vector<int64_t> slot(n, -1);
  size_t u = 0;
  unmapped_batch->header_indices[0] = 0;
  unmapped_batch->data_indices[0] = 0;
  for (size_t i = 0; i < n; ++i) {
    OutList& li = L[i];
    for (uint32_t j = 0; j < li.nslots; ++j) array_list_insert(li.slots[j], mapping_list);
    for (void* p : li.fresh) array_list_insert(p, mapping_list);
    // reads of 5+ bases get mapped records only; shorter ones one unmapped record
    const bool mapped = rds[i].len >= 5 && li.nslots + li.fresh.size() > 0;
    if (mapped) continue;
    const size_t hlen = (size_t)(batch->header_indices[i + 1] - batch->header_indices[i]);
    const size_t qlen = (size_t)(batch->data_indices[i + 1] - batch->data_indices[i]);
    slot[i] = (int64_t)u;
    ++u;
    unmapped_batch->data_indices[u] = unmapped_batch->data_indices[u - 1] + (int)qlen;
    unmapped_batch->header_indices[u] = unmapped_batch->header_indices[u - 1] + (int)hlen;
  }
#pragma omp parallel for schedule(static) if (n > 4096)
  for (size_t i = 0; i < n; ++i) {
    if (slot[i] < 0) continue;
    const size_t v = (size_t)slot[i];
    const size_t hlen = (size_t)(batch->header_indices[i + 1] - batch->header_indices[i]);
    const size_t qlen = (size_t)(batch->data_indices[i + 1] - batch->data_indices[i]);
    std::memcpy(unmapped_batch->header + unmapped_batch->header_indices[v], batch->header + batch->header_indices[i],
                hlen);
    std::memcpy(unmapped_batch->seq + unmapped_batch->data_indices[v], batch->seq + batch->data_indices[i], qlen);
    std::memcpy(unmapped_batch->quality + unmapped_batch->data_indices[v], batch->quality + batch->data_indices[i],
                qlen);
  }
  unmapped_batch->num_reads = u;
  g_flat_slots.reset();
  sw.mark("list and unmapped batch");
  return array_list_size(mapping_list);
}

size_t bwt_map_inexact_array_list(array_list_t* reads, bwt_optarg_t* opt, bwt_index_t* index, array_list_t** lists,
                                  size_t* num_unmapped, size_t* unmapped_indices) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  const size_t n = array_list_size(reads);
  std::vector<InexactRead> rds(n);
  std::vector<OutList> L(n);
  std::vector<OutList*> out(n);
  std::vector<size_t> before(n);
  for (size_t i = 0; i < n; ++i) {
    rds[i] = read_of(static_cast<fastq_read_t*>(array_list_get(i, reads)));
    L[i].list = lists[i];
    out[i] = &L[i];
    before[i] = array_list_size(lists[i]);
  }
  auto res = map_inexact(e, rds, opt, out);
  size_t total = 0;
  *num_unmapped = 0;
  for (size_t i = 0; i < n; ++i) {
    bool mapped = false;
    for (size_t j = before[i]; j < array_list_size(lists[i]) && j < before[i] + res[i].added; ++j)
      mapped = mapped || static_cast<alignment_t*>(array_list_get(j, lists[i]))->is_seq_mapped;
    total += res[i].added;
    if (!mapped) unmapped_indices[(*num_unmapped)++] = i;
  }
  return total;
}

size_t bwt_map_inexact_read_2(fastq_read_t* read, bwt_optarg_t* opt, bwt_index_t* index, array_list_t* mapping_list) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  std::vector<InexactRead> rds{read_of(read)};
  OutList L;
  L.list = mapping_list;
  std::vector<OutList*> lists{&L};
  map_block(e, rds, opt, lists);
  if (rds[0].len < 5) return 1;  // bwt.c:2337
  return array_list_size(mapping_list);
}

size_t bwt_map_inexact_array_list_2(array_list_t* reads, bwt_optarg_t* opt, bwt_index_t* index, array_list_t** lists,
                                    size_t* num_unmapped, size_t* unmapped_indices) {
  std::lock_guard<std::mutex> lk(g_mu);
  Engine* e = engine_for(index);
  const size_t n = array_list_size(reads);
  std::vector<InexactRead> rds(n);
  std::vector<OutList> L(n);
  std::vector<OutList*> out(n);
  std::vector<size_t> before(n);
  for (size_t i = 0; i < n; ++i) {
    rds[i] = read_of(static_cast<fastq_read_t*>(array_list_get(i, reads)));
    L[i].list = lists[i];
    out[i] = &L[i];
    before[i] = array_list_size(lists[i]);
  }
  auto res = map_block(e, rds, opt, out);
  size_t total = 0;
  *num_unmapped = 0;
  for (size_t i = 0; i < n; ++i) {
    bool mapped = false;
    for (size_t j = before[i]; j < array_list_size(lists[i]) && j < before[i] + res[i].added; ++j)
      mapped = mapped || static_cast<alignment_t*>(array_list_get(j, lists[i]))->is_seq_mapped;
    total += res[i].added;
    if (!mapped) unmapped_indices[(*num_unmapped)++] = i;
  }
  return total;
}

}  // extern "C"
