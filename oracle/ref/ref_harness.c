/*
 * TEST INFRASTRUCTURE ONLY -- the reference oracle harness.
 *
 * Links against the reference's own, unmodified sources (compiled from the
 * read-only reference tree by oracle/ref/Makefile into oracle/_ref/) and
 * drives them exactly the way c/src/aligners/bwt/bwt.c does, emitting the
 * flat records of include/hpg_bwt_records.h.  Only tests/ and the golden
 * fixture script load the resulting library; nothing in the product does.
 *
 *   ref_build_index   -> bwt_generate_index_files (bwt.c:744-819)
 *   ref_search        -> mode EXACT  : BWExactSearchBackward over backward ('+') and
 *                                      forward_rev ('-') (search/search.h:9-36)
 *                        mode SEARCH1: the four vector searches of bwt.c:1940-1950,
 *                                      BWSearch1VectorHelper per type (bwt.c:1989-2002)
 *                        then, for every hit, the locate loop of bwt.c:2158-2166.
 *   ref_block_search  -> BWSearchCPU per type as bwt_map_inexact_read_2 calls it
 *                        (bwt.c:2401-2470), its results located, and its anchors.
 *   ref_map_api       -> the alignment-list entry points themselves:
 *                        0 bwt_map_exact_read per read (bwt.c:994), fresh list each
 *                        1 bwt_map_exact_seqs over all reads, one thread (bwt.c:1040)
 *                        2 bwt_map_exact_batch over all reads (bwt.c:1097)
 *                        3 bwt_map_inexact_read per read (bwt.c:1879), fresh list with `flag`
 *                        5 bwt_map_inexact_read_2 per read (bwt.c:2313), fresh list with `flag`
 *                        serialised as described at ref_map_api.
 */
#include <ctype.h>
#include <fcntl.h>
#include <stdarg.h>
#include <unistd.h>

#include "bwt.h"
#include "hpg_bwt_records.h"

/* dbwt and bwt_map_exact_seq print progress on stdout; keep the test output clean. */
static int quiet_begin(void) {
  fflush(stdout);
  int saved = dup(1);
  int devnull = open("/dev/null", O_WRONLY);
  if (devnull >= 0) {
    dup2(devnull, 1);
    close(devnull);
  }
  return saved;
}

static void quiet_end(int saved) {
  fflush(stdout);
  if (saved >= 0) {
    dup2(saved, 1);
    close(saved);
  }
}

int ref_build_index(const char *fasta, const char *outdir, unsigned ratio) {
  int q = quiet_begin();
  bwt_generate_index_files((char *)fasta, (char *)outdir, ratio, false, "ACGT");
  /* save_exome_file (search/io.c:83-105) never closes its FILE, so the
   * "index" file would stay unflushed until the process exits. */
  fflush(NULL);
  quiet_end(q);
  return 0;
}

void *ref_index_load(const char *dir) { return bwt_index_new(dir, false); }

void ref_index_free(void *idx) { bwt_index_free((bwt_index_t *)idx); }

/* Growable output buffers. */
typedef struct {
  hpg_hit_t *hits;
  size_t n_hits, cap_hits;
  hpg_loc_t *locs;
  size_t n_locs, cap_locs;
} sink_t;

static void push_hit(sink_t *s, const hpg_hit_t *h) {
  if (s->n_hits == s->cap_hits) {
    s->cap_hits = s->cap_hits ? 2 * s->cap_hits : 1024;
    s->hits = (hpg_hit_t *)realloc(s->hits, s->cap_hits * sizeof(hpg_hit_t));
  }
  s->hits[s->n_hits++] = *h;
}

static void push_loc(sink_t *s, const hpg_loc_t *l) {
  if (s->n_locs == s->cap_locs) {
    s->cap_locs = s->cap_locs ? 2 * s->cap_locs : 1024;
    s->locs = (hpg_loc_t *)realloc(s->locs, s->cap_locs * sizeof(hpg_loc_t));
  }
  s->locs[s->n_locs++] = *l;
}

/* The locate loop of bwt.c:2158-2166 for one hit, with the same size_t
 * arithmetic; `direction` and `len_calc` as computed at bwt.c:2025-2036. */
static void locate_hit(bwt_index_t *index, sink_t *s, uint32_t hit_id, intmax_t k, intmax_t l,
                       size_t direction, size_t len_calc) {
  if (k > l) return;
  for (size_t j = (size_t)k; j <= (size_t)l; j++) {
    size_t key = direction ? size_SA(index->forward) - get_SA(j, index->forward) - len_calc - 1
                           : get_SA(j, index->backward);
    size_t idx = binsearch(index->karyotype->offset, index->karyotype->size, key);
    hpg_loc_t loc;
    memset(&loc, 0, sizeof(loc));
    loc.key = key;
    loc.hit = hit_id;
    if (key + len_calc <= index->karyotype->offset[idx]) {
      loc.valid = 1;
      loc.chrom = (uint32_t)(idx - 1);
      loc.position = index->karyotype->start[idx - 1] + (key - index->karyotype->offset[idx - 1]);
    }
    push_loc(s, &loc);
  }
}

static void fill_hit(hpg_hit_t *h, uint32_t read, int type, const result *r) {
  memset(h, 0, sizeof(*h));
  h->read = read;
  h->strand = (uint8_t)!type;
  h->dir = r->dir;
  h->nm = r->num_mismatches;
  if (r->num_mismatches) {
    h->err_kind = r->err_kind[0];
    h->err_base = r->err_base[0];
    h->err_pos = r->err_pos[0];
  }
  h->k = r->k;
  h->l = r->l;
}

/* Whether every character of a read is a letter of the index alphabet (either
 * case).  bwt_init_replace_table (bwt_commons.c:60-92) fills only those 2 x nA
 * entries of its malloc'ed table, so any other character gives an arbitrary
 * code, which can index past the C and O tables: such reads are not given to
 * the reference (the product maps them to no hits). */
static int in_alphabet(const bwt_index_t *index, const char *s, size_t len) {
  const char *nt = index->bwt_config.nucleotides;
  for (size_t i = 0; i < len; i++) {
    const int c = toupper((unsigned char)s[i]);
    int ok = 0;
    for (int a = 0; a < index->bwt_config.nA && !ok; a++) ok = (c == nt[a]);
    if (!ok) return 0;
  }
  return 1;
}

int ref_search(void *vidx, int mode, const char *seqs, const uint64_t *offsets, size_t n_reads,
               uint32_t max_results, hpg_result_set_t *out) {
  bwt_index_t *index = (bwt_index_t *)vidx;
  sink_t s;
  memset(&s, 0, sizeof(s));
  memset(out, 0, sizeof(*out));
  out->n_reads = n_reads;
  out->rs_count = (uint32_t *)calloc(2 * n_reads + 1, sizeof(uint32_t));
  out->rs_truncated = (uint8_t *)calloc(2 * n_reads + 1, 1);

  results_list r_list;
  new_results_list(&r_list, max_results ? max_results : 1);
  r_list.max_results = max_results; /* 0 is a legal (empty) capacity */

  for (size_t rd = 0; rd < n_reads; rd++) {
    size_t len = (size_t)(offsets[rd + 1] - offsets[rd]);
    const char *seq = seqs + offsets[rd];
    if (len < 3) continue; /* the helper reads outside its vectors below 3 bases */
    if (!in_alphabet(index, seq, len)) continue;
    uint8_t *code = (uint8_t *)malloc(len);
    encode_bases(code, (char *)seq, len, index->bwt_config.table);
    int16_t start = 0, end = (int16_t)(len - 1);

    if (mode == HPG_BWT_MODE_EXACT) {
      for (int type = 1; type >= 0; type--) {
        bwt_index *bi = type ? index->backward : index->forward_rev;
        result r;
        init_result(&r, 0);
        bound_result(&r, start, end);
        change_result(&r, 0, size_SA(bi) - 1, end);
        BWExactSearchBackward(code, bi, &r, NULL);
        if (r.k <= r.l) {
          hpg_hit_t h;
          r.num_mismatches = 0;
          fill_hit(&h, (uint32_t)rd, type, &r);
          uint32_t hid = (uint32_t)s.n_hits;
          push_hit(&s, &h);
          out->rs_count[2 * rd + !type]++;
          /* '+' rows live in backward's SA, '-' rows in forward's (direction 1). */
          locate_hit(index, &s, hid, r.k, r.l, type ? 0 : 1, len);
        }
      }
    } else {
      intmax_t *k0 = malloc(len * sizeof(intmax_t)), *l0 = malloc(len * sizeof(intmax_t));
      intmax_t *k1 = malloc(len * sizeof(intmax_t)), *l1 = malloc(len * sizeof(intmax_t));
      intmax_t *ki0 = malloc(len * sizeof(intmax_t)), *li0 = malloc(len * sizeof(intmax_t));
      intmax_t *ki1 = malloc(len * sizeof(intmax_t)), *li1 = malloc(len * sizeof(intmax_t));
      BWExactSearchVectorBackward(code, start, end, 0, size_SA(index->backward) - 1, k1, l1, index->backward);
      BWExactSearchVectorForward(code, start, end, 0, size_SA(index->forward) - 1, ki1, li1, index->forward);
      BWExactSearchVectorForward(code, start, end, 0, size_SA(index->backward_rev) - 1, k0, l0,
                                 index->backward_rev);
      BWExactSearchVectorBackward(code, start, end, 0, size_SA(index->forward_rev) - 1, ki0, li0,
                                  index->forward_rev);
      for (int type = 1; type >= 0; type--) {
        r_list.num_results = 0;
        r_list.read_index = 0;
        bool overflow;
        if (type == 1)
          overflow = BWSearch1VectorHelper(code, start, end, k1, l1, ki1, li1, index->backward,
                                           index->forward, &r_list, index->bwt_config.nA);
        else
          overflow = BWSearch1VectorHelper(code, start, end, ki0, li0, k0, l0, index->forward_rev,
                                           index->backward_rev, &r_list, index->bwt_config.nA);
        out->rs_truncated[2 * rd + !type] = overflow ? 1 : 0;
        out->rs_count[2 * rd + !type] = (uint32_t)r_list.num_results;
        for (size_t ii = 0; ii < r_list.num_results; ii++) {
          result *r = &r_list.list[ii];
          hpg_hit_t h;
          fill_hit(&h, (uint32_t)rd, type, r);
          uint32_t hid = (uint32_t)s.n_hits;
          push_hit(&s, &h);
          char error = r->num_mismatches ? r->err_kind[0] : 0;
          size_t direction = type ? r->dir : !r->dir;
          size_t len_calc = len;
          if (error == DELETION) len_calc--;
          else if (error == INSERTION) len_calc++;
          locate_hit(index, &s, hid, r->k, r->l, direction, len_calc);
        }
      }
      free(k0); free(l0); free(k1); free(l1);
      free(ki0); free(li0); free(ki1); free(li1);
    }
    free(code);
  }
  free(r_list.list);
  out->n_hits = s.n_hits;
  out->hits = s.hits;
  out->n_locs = s.n_locs;
  out->locs = s.locs;
  return 0;
}

/* The k-error block search as bwt_map_inexact_read_2 runs it (bwt.c:2401-2470):
 * BWSearchCPU per type with result lists of capacity max_results and anchor
 * lists of 2, then the locate loop of bwt.c:2640-2650 for every result of
 * rl_final (positions without that function's +1).  Anchors as
 * fmo_block_search: anchors[2 * (2 * read + strand) + a], a < n_anchors[..].
 * rs_truncated stays 0 (BWSearchCPU does not report refused results). */
int ref_block_search(void *vidx, const char *seqs, const uint64_t *offsets, size_t n_reads, uint32_t max_results,
                     hpg_result_set_t *out, hpg_block_anchor_t *anchors, uint8_t *n_anchors) {
  bwt_index_t *index = (bwt_index_t *)vidx;
  sink_t s;
  memset(&s, 0, sizeof(s));
  memset(out, 0, sizeof(*out));
  out->n_reads = n_reads;
  out->rs_count = (uint32_t *)calloc(2 * n_reads + 1, sizeof(uint32_t));
  out->rs_truncated = (uint8_t *)calloc(2 * n_reads + 1, 1);
  memset(n_anchors, 0, 2 * n_reads);
  results_list rl_prev, rl_next, rl_prev_i, rl_next_i, rl_final, rl_anch;
  results_list *lists[] = {&rl_prev, &rl_next, &rl_prev_i, &rl_next_i, &rl_final};
  for (int i = 0; i < 5; i++) {
    new_results_list(lists[i], max_results ? max_results : 1);
    lists[i]->max_results = max_results;
  }
  new_results_list(&rl_anch, 2);
  for (size_t rd = 0; rd < n_reads; rd++) {
    size_t len = (size_t)(offsets[rd + 1] - offsets[rd]);
    const char *seq = seqs + offsets[rd];
    if (len < 3 || len > 32767) continue;
    if (!in_alphabet(index, seq, len)) continue;
    uint8_t *code = (uint8_t *)malloc(len);
    encode_bases(code, (char *)seq, len, index->bwt_config.table);
    int frag = (int)(len / 2); /* bwt.c:2408-2412: len / (num_errors + 1), at least 30 */
    if (frag < 30) frag = 30;
    for (int type = 1; type >= 0; type--) {
      for (int i = 0; i < 5; i++) lists[i]->num_results = 0;
      rl_final.read_index = 0;
      if (type == 1)
        BWSearchCPU(code, len, index->backward, index->forward, &rl_prev, &rl_next, &rl_prev_i, &rl_next_i,
                    &rl_final, &rl_anch, (int16_t)frag, 1, index->bwt_config.nA);
      else
        BWSearchCPU(code, len, index->forward_rev, index->backward_rev, &rl_prev, &rl_next, &rl_prev_i,
                    &rl_next_i, &rl_final, &rl_anch, (int16_t)frag, 0, index->bwt_config.nA);
      const size_t t2 = 2 * rd + !type;
      out->rs_count[t2] = (uint32_t)rl_final.num_results;
      for (size_t ii = 0; ii < rl_final.num_results; ii++) {
        result *r = &rl_final.list[ii];
        hpg_hit_t h;
        fill_hit(&h, (uint32_t)rd, type, r);
        uint32_t hid = (uint32_t)s.n_hits;
        push_hit(&s, &h);
        char error = r->num_mismatches ? r->err_kind[0] : 0;
        size_t direction = type ? r->dir : !r->dir;
        size_t len_calc = len;
        if (error == DELETION) len_calc--;
        else if (error == INSERTION) len_calc++;
        locate_hit(index, &s, hid, r->k, r->l, direction, len_calc);
      }
      n_anchors[t2] = (uint8_t)rl_anch.num_results;
      for (size_t a = 0; a < rl_anch.num_results; a++) {
        hpg_block_anchor_t *o = &anchors[2 * t2 + a];
        memset(o, 0, sizeof(*o));
        o->k = rl_anch.list[a].k;
        o->l = rl_anch.list[a].l;
        o->start = rl_anch.list[a].start;
        o->end = rl_anch.list[a].end;
        o->pos = rl_anch.list[a].pos;
        o->dir = rl_anch.list[a].dir;
      }
    }
    free(code);
  }
  for (int i = 0; i < 5; i++) free(lists[i]->list);
  free(rl_anch.list);
  out->n_hits = s.n_hits;
  out->hits = s.hits;
  out->n_locs = s.n_locs;
  out->locs = s.locs;
  return 0;
}

void ref_result_free(hpg_result_set_t *out) {
  free(out->hits);
  free(out->locs);
  free(out->rs_count);
  free(out->rs_truncated);
  memset(out, 0, sizeof(*out));
}

/* ---- alignment lists, serialised (little endian) ----
 * per list:  u32 items, i32 list flag, u64 return value, u8 items-are-anchors,
 *            then per item an alignment or an anchor:
 * alignment: u32 chromosome, i32 position, i32 map_quality, i32 num_cigar_operations,
 *            u8 seq_strand, u8 is_seq_mapped, u8 secondary_alignment,
 *            i32 mate_position, i32 mate_chromosome, i32 template_length,
 *            str query_name, str sequence, str quality (at most the read's quality
 *            length: strand-0 qualities are not terminated, bwt.c:540), str cigar,
 *            i32 optional_fields_length + those bytes
 * anchor:    i32 strand, i32 chromosome, u64 start, u64 end, i32 type
 * str:       u32 length (0xFFFFFFFF for NULL) + bytes
 * api 1 appends u8 out_status per read; api 2 appends u32 unmapped reads and
 * per unmapped read str header, str seq, str quality (raw index ranges). */
typedef struct {
  uint8_t *p;
  size_t n, cap;
} blob_t;

static void put(blob_t *b, const void *v, size_t n) {
  if (b->n + n > b->cap) {
    b->cap = (b->n + n) * 2 + 1024;
    b->p = (uint8_t *)realloc(b->p, b->cap);
  }
  memcpy(b->p + b->n, v, n);
  b->n += n;
}
static void put_u8(blob_t *b, uint8_t v) { put(b, &v, 1); }
static void put_u32(blob_t *b, uint32_t v) { put(b, &v, 4); }
static void put_i32(blob_t *b, int32_t v) { put(b, &v, 4); }
static void put_u64(blob_t *b, uint64_t v) { put(b, &v, 8); }
static void put_str(blob_t *b, const char *s, size_t maxlen) {
  if (!s) {
    put_u32(b, 0xFFFFFFFFu);
    return;
  }
  size_t n = strnlen(s, maxlen);
  put_u32(b, (uint32_t)n);
  put(b, s, n);
}
static void put_raw(blob_t *b, const char *s, size_t n) {
  put_u32(b, (uint32_t)n);
  put(b, s, n);
}

static void put_list(blob_t *b, array_list_t *list, size_t ret, int anchors, size_t qmax) {
  size_t n = array_list_size(list);
  put_u32(b, (uint32_t)n);
  put_i32(b, array_list_get_flag(list));
  put_u64(b, ret);
  put_u8(b, (uint8_t)anchors);
  for (size_t i = 0; i < n; i++) {
    if (anchors) {
      bwt_anchor_t *a = (bwt_anchor_t *)array_list_get(i, list);
      put_i32(b, a->strand);
      put_i32(b, a->chromosome);
      put_u64(b, a->start);
      put_u64(b, a->end);
      put_i32(b, a->type);
    } else {
      alignment_t *a = (alignment_t *)array_list_get(i, list);
      put_u32(b, a->chromosome);
      put_i32(b, a->position);
      put_i32(b, a->map_quality);
      put_i32(b, a->num_cigar_operations);
      put_u8(b, a->seq_strand);
      put_u8(b, a->is_seq_mapped);
      put_u8(b, a->secondary_alignment);
      put_i32(b, a->mate_position);
      put_i32(b, a->mate_chromosome);
      put_i32(b, a->template_length);
      put_str(b, a->query_name, (size_t)-1);
      put_str(b, a->sequence, (size_t)-1);
      put_str(b, a->quality, qmax);
      put_str(b, a->cigar, (size_t)-1);
      put_i32(b, a->optional_fields_length);
      if (a->optional_fields_length > 0 && a->optional_fields) put(b, a->optional_fields, a->optional_fields_length);
    }
  }
}

static void free_list(array_list_t *list, int anchors) {
  size_t n = array_list_size(list);
  for (size_t i = 0; i < n; i++) {
    void *p = array_list_get(i, list);
    if (anchors) bwt_anchor_free((bwt_anchor_t *)p);
    else alignment_free((alignment_t *)p);
  }
  array_list_free(list, NULL);
}

/* Reads: sequences and qualities as NUL-terminated strings (seqs + offs[i],
 * length offs[i+1]-offs[i]-1), ids likewise with id_offs. */
int ref_map_api(void *vidx, int api, const char *seqs, const char *quals, const uint64_t *offs, const char *ids,
                const uint64_t *id_offs, size_t n, int filter, int flag, uint8_t **out, size_t *out_len) {
  bwt_index_t *index = (bwt_index_t *)vidx;
  bwt_optarg_t *opt = bwt_optarg_new(api == 3 || api == 5 ? 1 : 0, 1, filter, filter);
  blob_t b = {0};
  int q = quiet_begin(); /* bwt_map_exact_seq prints a line per read */
  if (api == 0 || api == 3 || api == 5) {
    for (size_t i = 0; i < n; i++) {
      fastq_read_t r;
      memset(&r, 0, sizeof(r));
      r.id = (char *)ids + id_offs[i];
      r.sequence = (char *)seqs + offs[i];
      r.quality = (char *)quals + offs[i];
      size_t len = offs[i + 1] - offs[i] - 1;
      char *rc = strdup(r.sequence);
      seq_reverse_complementary(rc, (unsigned)len);
      r.revcomp = rc;
      r.length = (int)len;
      array_list_t *list = array_list_new(16, 1.25f, COLLECTION_MODE_ASYNCHRONIZED);
      array_list_set_flag(api == 3 || api == 5 ? flag : 0, list);
      size_t ret = api == 0   ? bwt_map_exact_read(&r, opt, index, list)
                   : api == 3 ? bwt_map_inexact_read(&r, opt, index, list)
                              : bwt_map_inexact_read_2(&r, opt, index, list);
      int anchors = (api == 3 || api == 5) && len >= 5 && array_list_get_flag(list) == 1;
      put_list(&b, list, ret, anchors, len);
      free_list(list, anchors);
      free(rc);
    }
  } else if (api == 1) {
    char **ss = (char **)malloc(n * sizeof(char *) + 1);
    char *status = (char *)malloc(n + 1);
    for (size_t i = 0; i < n; i++) ss[i] = (char *)seqs + offs[i];
    array_list_t *list = array_list_new(16, 1.25f, COLLECTION_MODE_SYNCHRONIZED);
    size_t ret = bwt_map_exact_seqs(ss, n, opt, index, status, list);
    put_list(&b, list, ret, 0, (size_t)-1);
    for (size_t i = 0; i < n; i++) put_u8(&b, (uint8_t)status[i]);
    free_list(list, 0);
    free(ss);
    free(status);
  } else if (api == 2) {
    fastq_batch_t batch, unmapped;
    memset(&batch, 0, sizeof(batch));
    memset(&unmapped, 0, sizeof(unmapped));
    batch.num_reads = n;
    batch.header_indices = (int *)malloc((n + 1) * sizeof(int));
    batch.data_indices = (int *)malloc((n + 1) * sizeof(int));
    for (size_t i = 0; i <= n; i++) {
      batch.header_indices[i] = (int)id_offs[i];
      batch.data_indices[i] = (int)offs[i];
    }
    batch.header = (char *)ids;
    batch.seq = (char *)seqs;
    batch.quality = (char *)quals;
    unmapped.header_indices = (int *)calloc(n + 1, sizeof(int));
    unmapped.data_indices = (int *)calloc(n + 1, sizeof(int));
    unmapped.header = (char *)calloc(id_offs[n] + 1, 1);
    unmapped.seq = (char *)calloc(offs[n] + 1, 1);
    unmapped.quality = (char *)calloc(offs[n] + 1, 1);
    array_list_t *list = array_list_new(16, 1.25f, COLLECTION_MODE_SYNCHRONIZED);
    size_t ret = bwt_map_exact_batch(&batch, opt, index, &unmapped, list);
    put_list(&b, list, ret, 0, (size_t)-1);
    put_u32(&b, (uint32_t)unmapped.num_reads);
    for (size_t u = 0; u < unmapped.num_reads; u++) {
      put_raw(&b, unmapped.header + unmapped.header_indices[u],
              (size_t)(unmapped.header_indices[u + 1] - unmapped.header_indices[u]));
      put_raw(&b, unmapped.seq + unmapped.data_indices[u],
              (size_t)(unmapped.data_indices[u + 1] - unmapped.data_indices[u]));
      put_raw(&b, unmapped.quality + unmapped.data_indices[u],
              (size_t)(unmapped.data_indices[u + 1] - unmapped.data_indices[u]));
    }
    free_list(list, 0);
    free(batch.header_indices);
    free(batch.data_indices);
    free(unmapped.header_indices);
    free(unmapped.data_indices);
    free(unmapped.header);
    free(unmapped.seq);
    free(unmapped.quality);
  }
  quiet_end(q);
  bwt_optarg_free(opt);
  *out = b.p;
  *out_len = b.n;
  return 0;
}

/* Text lines of the seed and CAL records, the format tests/seed_lists.py
 * writes for the product's records. */
static void put_text(blob_t *b, const char *fmt, ...) {
  char line[256];
  va_list ap;
  va_start(ap, fmt);
  int n = vsnprintf(line, sizeof line, fmt, ap);
  va_end(ap);
  if (n > 0) put(b, line, (size_t)n < sizeof line ? (size_t)n : sizeof line - 1);
}

static void put_seed(blob_t *b, char tag, seed_region_t *s) {
  put_text(b, "%c %d %d %zu %zu %d\n", tag, s->read_start, s->read_end, s->genome_start, s->genome_end, s->id);
}

/* ref_seeds_cals: per read (seqs NUL-terminated at offs[i], as ref_map_api),
 *   mode 0: bwt_map_exact_seeds_seq (bwt.c:3577) into a fresh list:
 *           "R <returned> <size>" then "G chrom strand start end seq_start seq_end seq_len id" per region;
 *   mode 2: bwt_map_exact_seeds_by_region (bwt.c:4033) over the read window
 *           [min_cal_size, len - max_intron) (the two fields carry the window's offsets),
 *           written as mode 0;
 *   mode 1: bwt_generate_cals (bwt.c:3832) into a fresh list:
 *           "R <returned> <size>" then per CAL "C chrom strand start end num_seeds read_area" followed
 *           by its seeds: "S ..." (sr_list), "D ..." (sr_duplicate_list), "A ..." / "B ..."
 *           (candidates_seeds_start / _end), each "read_start read_end genome_start genome_end id".
 * Fields the reference leaves unset (region pos_err/type_err, the duplicates'
 * pos_err/type_err, cal flanks) are not written. */
int ref_seeds_cals(void *vidx, int mode, const char *seqs, const uint64_t *offs, size_t n, size_t seed_size,
                   int filter_seed, size_t min_cal_size, size_t max_intron, unsigned nchrom, uint8_t **out,
                   size_t *out_len) {
  bwt_index_t *index = (bwt_index_t *)vidx;
  bwt_optarg_t *opt = bwt_optarg_new(1, 1, 200, filter_seed);
  cal_optarg_t *copt = cal_optarg_new(min_cal_size, 0, 0, 0, seed_size, 0, 0, max_intron, 0);
  blob_t b = {0};
  for (size_t i = 0; i < n; i++) {
    char *seq = (char *)seqs + offs[i];
    array_list_t *list = array_list_new(16, 1.25f, COLLECTION_MODE_ASYNCHRONIZED);
    if (mode == 0 || mode == 2) {
      const size_t len = strlen(seq);
      size_t ret = mode == 0 ? bwt_map_exact_seeds_seq(0, 0, seq, seed_size, 0, opt, index, list, 0)
                             : bwt_map_exact_seeds_by_region((int)min_cal_size, (int)(len - max_intron), seq,
                                                             (int)seed_size, 0, opt, index, list);
      put_text(&b, "R %zu %zu\n", ret, array_list_size(list));
      for (size_t k = 0; k < array_list_size(list); k++) {
        region_t *r = (region_t *)array_list_get(k, list);
        put_text(&b, "G %zu %d %zu %zu %zu %zu %zu %d\n", r->chromosome_id, (int)r->strand, r->start, r->end,
                 r->seq_start, r->seq_end, r->seq_len, r->id);
      }
      array_list_free(list, (void *)region_bwt_free);
    } else {
      size_t ret = bwt_generate_cals(seq, seed_size, opt, copt, index, list, nchrom);
      put_text(&b, "R %zu %zu\n", ret, array_list_size(list));
      for (size_t k = 0; k < array_list_size(list); k++) {
        cal_t *c = (cal_t *)array_list_get(k, list);
        put_text(&b, "C %zu %d %zu %zu %zu %d\n", c->chromosome_id, (int)c->strand, c->start, c->end,
                 c->num_seeds, c->read_area);
        for (linked_list_item_t *it = c->sr_list ? c->sr_list->first : NULL; it; it = it->next)
          put_seed(&b, 'S', (seed_region_t *)it->item);
        for (linked_list_item_t *it = c->sr_duplicate_list ? c->sr_duplicate_list->first : NULL; it; it = it->next)
          put_seed(&b, 'D', (seed_region_t *)it->item);
        for (size_t a = 0; a < array_list_size(c->candidates_seeds_start); a++)
          put_seed(&b, 'A', (seed_region_t *)array_list_get(a, c->candidates_seeds_start));
        for (size_t a = 0; a < array_list_size(c->candidates_seeds_end); a++)
          put_seed(&b, 'B', (seed_region_t *)array_list_get(a, c->candidates_seeds_end));
      }
      array_list_free(list, (void *)cal_free);
    }
  }
  bwt_optarg_free(opt);
  cal_optarg_free(copt);
  *out = b.p;
  *out_len = b.n;
  return 0;
}

void ref_blob_free(uint8_t *p) { free(p); }
