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
 *   ref_map_inexact   -> bwt_map_inexact_read (bwt.c:1879) per read, flattened.
 *   ref_map_exact     -> bwt_map_exact_read (bwt.c:994) per read, flattened.
 */
#include <fcntl.h>
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

void ref_result_free(hpg_result_set_t *out) {
  free(out->hits);
  free(out->locs);
  free(out->rs_count);
  free(out->rs_truncated);
  memset(out, 0, sizeof(*out));
}
