/*
 * fm_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU oracle for the FM-index read
 * mapping hot path.
 *
 * A plain-C restatement of the reference's algorithms, used by tests/ as the
 * parity checker, by __graft_entry__.smoke() and by bench.py as the timed CPU
 * baseline ("port").  Nothing in the product links or calls it.  It is pinned
 * against the reference's own compiled sources (oracle/_ref, see
 * oracle/ref/Makefile) and against the committed golden fixtures in
 * tests/golden/.
 *
 * Followed, step by step:
 *   rank get_O ............................. search/csafm.h:166-181 (FM_COMP_64)
 *   BWT symbol get_B_from_O ................ search/csafm.h:183-206
 *   sampled-SA walk getScompValue .......... search/csafm.h:208-235
 *   BWiteration ............................ search/runtime.h:38-42
 *   complement views (backward_rev, ...) ... search/csafm.c:3-100, runtime.h:106-122
 *   BWExactSearchBackward/Forward .......... search/search.h:9-65
 *   BWExactSearchVectorBackward/Forward .... search/search.c:1407-1489
 *   BWSearch1VectorHelper .................. search/search.c:1491-1709
 *   add_result (truncation) ................ search/results.h:93-103
 *   per-read driver ........................ bwt.c:1940-2002
 *   k-error block search BWSearchCPU ....... search/search.c:1-646,1045-1405; search/search.h:9-155
 *     as bwt_map_inexact_read_2 drives it .. bwt.c:2401-2470 (one or two fragments)
 *   locate + karyotype ..................... bwt.c:2025-2036, 2158-2166; search/io.h:43-64
 *   index files ............................ search/csafm.c:121-250, search/io.c:26-81,336-362
 */
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/hpg_bwt_records.h"

/* ---------------------------------------------------------------- index -- */

typedef struct {
  uint32_t siz, m;
  uint32_t *desp;  /* [4][m] */
  uint64_t *count; /* [4][m] */
} fmo_occ_t;

typedef struct {
  uint32_t siz, n, ratio;
  uint32_t *v;
} fmo_samp_t;

typedef struct {
  const fmo_occ_t *O;
  const fmo_samp_t *S;
  uint32_t C[4], C1[4];
  uint8_t map[4]; /* query code -> physical table row (identity or complement) */
} fmo_view_t;

typedef struct {
  uint8_t code_of[256]; /* 0xFF outside the alphabet */
  uint8_t comp[4];
  fmo_occ_t O, Oi;
  fmo_samp_t S, Si;
  uint32_t C[4], C1[4];
  size_t kar_size;
  uint64_t *kar_start, *kar_offset; /* offset has kar_size+1 entries */
  fmo_view_t bw, fw, bw_rev, fw_rev;
} fmo_index_t;

static int read_exact(FILE *f, void *p, size_t sz, size_t n) { return fread(p, sz, n, f) == n; }

static FILE *open_in(const char *dir, const char *name, const char *mode) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  return fopen(path, mode);
}

static int load_vec4(const char *dir, const char *name, uint32_t out[4]) {
  FILE *f = open_in(dir, name, "rb");
  uint32_t n = 0;
  int ok = f && read_exact(f, &n, 4, 1) && n == 4 && read_exact(f, out, 4, 4);
  if (f) fclose(f);
  return ok;
}

static int load_samp(const char *dir, const char *name, fmo_samp_t *s) {
  FILE *f = open_in(dir, name, "rb");
  int ok = f && read_exact(f, &s->siz, 4, 1) && read_exact(f, &s->n, 4, 1) && read_exact(f, &s->ratio, 4, 1);
  if (ok) {
    s->v = (uint32_t *)malloc((size_t)s->n * 4 + 4);
    ok = read_exact(f, s->v, 4, s->n) && s->ratio > 0;
  }
  if (f) fclose(f);
  return ok;
}

static int load_occ(const char *dir, const char *name, fmo_occ_t *o) {
  char fn[256];
  uint32_t nd = 0, nc = 0, mc = 0;
  snprintf(fn, sizeof fn, "%s.desp", name);
  FILE *f = open_in(dir, fn, "rb");
  int ok = f && read_exact(f, &o->siz, 4, 1) && read_exact(f, &nd, 4, 1) && read_exact(f, &o->m, 4, 1) && nd == 4;
  if (ok) {
    o->desp = (uint32_t *)malloc((size_t)4 * o->m * 4);
    ok = read_exact(f, o->desp, 4, (size_t)4 * o->m);
  }
  if (f) fclose(f);
  if (!ok) return 0;
  snprintf(fn, sizeof fn, "%s.count", name);
  f = open_in(dir, fn, "rb");
  ok = f && read_exact(f, &nc, 4, 1) && read_exact(f, &mc, 4, 1) && nc == 4 && mc == o->m;
  if (ok) {
    o->count = (uint64_t *)malloc((size_t)4 * o->m * 8);
    ok = read_exact(f, o->count, 8, (size_t)4 * o->m);
  }
  if (f) fclose(f);
  return ok;
}

static void make_view(fmo_index_t *ix, fmo_view_t *v, const fmo_occ_t *O, const fmo_samp_t *S, int comp) {
  v->O = O;
  v->S = S;
  for (int b = 0; b < 4; b++) {
    uint8_t p = comp ? ix->comp[b] : (uint8_t)b;
    v->map[b] = p;
    v->C[b] = ix->C[p];
    v->C1[b] = ix->C1[p];
  }
}

void fmo_index_free(fmo_index_t *ix) {
  if (!ix) return;
  free(ix->O.desp); free(ix->O.count); free(ix->Oi.desp); free(ix->Oi.count);
  free(ix->S.v); free(ix->Si.v);
  free(ix->kar_start); free(ix->kar_offset);
  free(ix);
}

fmo_index_t *fmo_index_load(const char *dir) {
  fmo_index_t *ix = (fmo_index_t *)calloc(1, sizeof(fmo_index_t));
  char alpha[256] = {0};
  FILE *f = open_in(dir, "config.txt", "r");
  if (!f || !fgets(alpha, sizeof alpha, f)) {
    if (f) fclose(f);
    free(ix);
    return NULL;
  }
  fclose(f);
  size_t al = strlen(alpha);
  if (al && alpha[al - 1] == '\n') alpha[--al] = 0;
  if (al != 4) { free(ix); return NULL; }
  memset(ix->code_of, 0xFF, sizeof ix->code_of);
  int idx[4] = {-1, -1, -1, -1}; /* positions of A, C, G, T */
  for (int i = 0; i < 4; i++) {
    char u = alpha[i] & ~0x20;
    ix->code_of[(unsigned char)u] = (uint8_t)i;
    ix->code_of[(unsigned char)(u | 0x20)] = (uint8_t)i;
    const char *p = strchr("ACGT", u);
    if (!p) { free(ix); return NULL; }
    idx[p - "ACGT"] = i;
  }
  ix->comp[idx[0]] = (uint8_t)idx[3]; ix->comp[idx[3]] = (uint8_t)idx[0];
  ix->comp[idx[1]] = (uint8_t)idx[2]; ix->comp[idx[2]] = (uint8_t)idx[1];

  if (!load_vec4(dir, "C.vec", ix->C) || !load_vec4(dir, "C1.vec", ix->C1) || !load_occ(dir, "O", &ix->O) ||
      !load_occ(dir, "Oi", &ix->Oi) || !load_samp(dir, "S.vec", &ix->S) || !load_samp(dir, "Si.vec", &ix->Si)) {
    fmo_index_free(ix);
    return NULL;
  }
  /* karyotype: ">name start end" lines, offset[i+1] = offset[i] + end-start+1 */
  f = open_in(dir, "index", "r");
  if (!f) { fmo_index_free(ix); return NULL; }
  size_t cap = 64;
  ix->kar_start = (uint64_t *)malloc(cap * 8);
  ix->kar_offset = (uint64_t *)malloc((cap + 1) * 8);
  ix->kar_offset[0] = 0;
  char line[8192];
  while (fgets(line, sizeof line, f)) {
    if (line[0] != '>') continue;
    char *sp = strchr(line, ' ');
    unsigned long long s = 0, e = 0;
    if (!sp || sscanf(sp, " %llu %llu", &s, &e) != 2) continue;
    if (ix->kar_size == cap) {
      cap *= 2;
      ix->kar_start = (uint64_t *)realloc(ix->kar_start, cap * 8);
      ix->kar_offset = (uint64_t *)realloc(ix->kar_offset, (cap + 1) * 8);
    }
    ix->kar_start[ix->kar_size] = s;
    ix->kar_offset[ix->kar_size + 1] = ix->kar_offset[ix->kar_size] + (e - s + 1);
    ix->kar_size++;
  }
  fclose(f);
  make_view(ix, &ix->bw, &ix->O, &ix->S, 0);
  make_view(ix, &ix->fw, &ix->Oi, &ix->Si, 0);
  make_view(ix, &ix->bw_rev, &ix->O, &ix->S, 1);
  make_view(ix, &ix->fw_rev, &ix->Oi, &ix->Si, 1);
  return ix;
}

/* ------------------------------------------------------------ rank / LF -- */

/* Occ of physical symbol p in columns 0..m (= BWT rows 0..m-1). */
static inline uint32_t occ(const fmo_occ_t *O, uint8_t p, uint32_t m) {
  uint32_t q = m >> 6, r = m & 63;
  uint64_t w = O->count[(size_t)p * O->m + q] << (63 - r);
  return O->desp[(size_t)p * O->m + q] + (uint32_t)__builtin_popcountll(w);
}

/* One backward-extension step by query symbol b over a (possibly complement) view. */
static inline void step(const fmo_view_t *v, uint8_t b, int64_t *k, int64_t *l) {
  uint8_t p = v->map[b];
  uint32_t nk = v->C1[b] + occ(v->O, p, (uint32_t)*k);
  uint32_t nl = v->C[b] + occ(v->O, p, (uint32_t)(*l + 1));
  *k = nk;
  *l = nl;
}

/* BWT symbol of row i, or 0xFF for the '$' row. */
static inline uint8_t bwt_symbol(const fmo_occ_t *O, uint32_t i) {
  uint32_t m = i + 1, q = m >> 6, r = m & 63;
  for (uint8_t p = 0; p < 4; p++)
    if ((O->count[(size_t)p * O->m + q] >> r) & 1) return p;
  return 0xFF;
}

/* SA value of row m by the sampled walk; uses the physical table. */
static uint32_t sa_value(const fmo_index_t *ix, const fmo_occ_t *O, const fmo_samp_t *S, uint32_t m) {
  uint32_t i = m, j = 0;
  while (i % S->ratio) {
    uint8_t b = bwt_symbol(O, i);
    i = (b == 0xFF) ? 0 : ix->C[b] + occ(O, b, i + 1);
    j++;
  }
  return (uint32_t)((S->v[i / S->ratio] + j) % (O->siz - 1));
}

/* ------------------------------------------------------------- results -- */

typedef struct {
  hpg_hit_t *hits;
  size_t n_hits, cap_hits;
  hpg_loc_t *locs;
  size_t n_locs, cap_locs;
} sink_t;

static void sink_hit(sink_t *s, const hpg_hit_t *h) {
  if (s->n_hits == s->cap_hits) {
    s->cap_hits = s->cap_hits ? 2 * s->cap_hits : 256;
    s->hits = (hpg_hit_t *)realloc(s->hits, s->cap_hits * sizeof(hpg_hit_t));
  }
  s->hits[s->n_hits++] = *h;
}

static void sink_loc(sink_t *s, const hpg_loc_t *l) {
  if (s->n_locs == s->cap_locs) {
    s->cap_locs = s->cap_locs ? 2 * s->cap_locs : 256;
    s->locs = (hpg_loc_t *)realloc(s->locs, s->cap_locs * sizeof(hpg_loc_t));
  }
  s->locs[s->n_locs++] = *l;
}

/* The reference helper keeps one mutable `result` and appends copies of it. */
typedef struct {
  uint8_t dir, nm, kind, base;
  int16_t err_pos, pos;
  int64_t k, l;
} cursor_t;

typedef struct {
  hpg_hit_t *buf;
  uint32_t n, cap;
  uint32_t read;
  uint8_t strand;
} list_t;

/* Appends like add_result; returns 1 when the list is already full. */
static int list_add(list_t *L, const cursor_t *c) {
  if (L->n >= L->cap) return 1;
  hpg_hit_t *h = &L->buf[L->n++];
  memset(h, 0, sizeof *h);
  h->read = L->read;
  h->strand = L->strand;
  h->dir = c->dir;
  h->nm = c->nm;
  if (c->nm) {
    h->err_kind = c->kind;
    h->err_base = c->base;
    h->err_pos = c->err_pos;
  }
  h->k = c->k;
  h->l = c->l;
  return 0;
}

/* ------------------------------------------------------------- searches -- */

static void exact_backward(const uint8_t *W, const fmo_view_t *v, cursor_t *c, int16_t start) {
  int64_t k = c->k, l = c->l;
  int16_t i;
  for (i = c->pos; i >= start; i--) {
    step(v, W[i], &k, &l);
    if (k > l) break;
  }
  c->k = k;
  c->l = l;
  c->pos = i;
}

static void exact_forward(const uint8_t *W, const fmo_view_t *v, cursor_t *c, int16_t end) {
  int64_t k = c->k, l = c->l;
  int16_t i;
  for (i = c->pos; i <= end; i++) {
    step(v, W[i], &k, &l);
    if (k > l) break;
  }
  c->k = k;
  c->l = l;
  c->pos = i;
}

/* Interval of W[j..end] in vk/vl[j]; after a failure the failed pair repeats. */
static void vector_backward(const uint8_t *W, int16_t start, int16_t end, int64_t k, int64_t l, int64_t *vk,
                            int64_t *vl, const fmo_view_t *v) {
  int16_t i = end, j = end - start;
  for (; i >= start; i--, j--) {
    step(v, W[i], &k, &l);
    vk[j] = k;
    vl[j] = l;
    if (k > l) { i--; j--; break; }
  }
  for (; i >= start; i--, j--) { vk[j] = k; vl[j] = l; }
}

/* Interval of W[start..start+j] in vk/vl[j]. */
static void vector_forward(const uint8_t *W, int16_t start, int16_t end, int64_t k, int64_t l, int64_t *vk,
                           int64_t *vl, const fmo_view_t *v) {
  int16_t i = start, j = 0;
  for (; i <= end; i++, j++) {
    step(v, W[i], &k, &l);
    vk[j] = k;
    vl[j] = l;
    if (k > l) { i++; j++; break; }
  }
  for (; i <= end; i++, j++) { vk[j] = k; vl[j] = l; }
}

/* BWSearch1VectorHelper: one exact hit, then deletion / mismatch / insertion
 * branches wherever the interval size changes.  Returns 1 on overflow. */
static int search1_helper(const uint8_t *W, int16_t start, int16_t end, const int64_t *vk, const int64_t *vl,
                          const int64_t *vki, const int64_t *vli, const fmo_view_t *B, const fmo_view_t *F,
                          list_t *L) {
  int16_t n = end - start, half = n / 2, i, j;
  int64_t res, res_last, k, l, ka, la;
  cursor_t c;
  memset(&c, 0, sizeof c);
  c.dir = 0;

  if (vk[0] <= vl[0]) {
    c.k = vk[0]; c.l = vl[0]; c.pos = -1;
    if (list_add(L, &c)) return 1;
  }
  c.nm = 1; c.kind = HPG_BWT_MATCH; c.base = 0xFF; c.err_pos = start;

  res = vl[0] - vk[0];
  res_last = res;
  k = vk[1]; l = vl[1];
  res = l - k;
  if (res != res_last) {
    /* first base of the read is extra: the rest is already searched */
    c.k = k; c.l = l; c.pos = -1;
    c.kind = HPG_BWT_DELETION; c.base = 0xFF; c.err_pos = start;
    if (list_add(L, &c)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      ka = k; la = l;
      step(B, b, &ka, &la);
      if (ka > la) continue;
      uint8_t bw = W[start];
      if (b != bw) {
        c.k = ka; c.l = la; c.pos = -1;
        c.kind = HPG_BWT_MISMATCH; c.base = b; /* err_pos kept */
        if (list_add(L, &c)) return 1;
      }
      step(B, bw, &ka, &la);
      if (ka <= la) {
        /* the reference stores kind 3, base INSERTION(3), position b here */
        c.k = ka; c.l = la; c.pos = -1;
        c.kind = 3; c.base = HPG_BWT_INSERTION; c.err_pos = b;
        if (list_add(L, &c)) return 1;
      }
    }
  }

  for (i = start + 2, j = 2; j <= half; i++, j++) {
    res_last = res;
    k = vk[j]; l = vl[j];
    res = l - k;
    if (res == res_last) continue;
    c.k = k; c.l = l; c.pos = i - 2;
    c.kind = HPG_BWT_DELETION; c.base = 0xFF; c.err_pos = i - 1;
    exact_backward(W, B, &c, start);
    if (c.k <= c.l && list_add(L, &c)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      ka = k; la = l;
      step(B, b, &ka, &la);
      if (ka > la) continue;
      c.k = ka; c.l = la; c.pos = i - 1;
      c.kind = HPG_BWT_INSERTION; c.base = b;
      exact_backward(W, B, &c, start);
      if (c.k <= c.l && list_add(L, &c)) return 1;
      if (b != W[i - 1]) {
        c.k = ka; c.l = la; c.pos = i - 2;
        c.kind = HPG_BWT_MISMATCH;
        exact_backward(W, B, &c, start);
        if (c.k <= c.l && list_add(L, &c)) return 1;
      }
    }
  }

  half--;
  res = vli[n] - vki[n];
  c.dir = 1;
  res_last = res;
  k = vki[n - 1]; l = vli[n - 1];
  res = l - k;
  if (res != res_last) {
    c.k = k; c.l = l; c.pos = -1;
    c.kind = HPG_BWT_DELETION; c.base = 0xFF; c.err_pos = end;
    if (list_add(L, &c)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      ka = k; la = l;
      step(F, b, &ka, &la);
      if (ka > la) continue;
      uint8_t bw = W[end];
      if (b != bw) {
        c.k = ka; c.l = la; c.pos = -1;
        c.kind = HPG_BWT_MISMATCH; c.base = b;
        if (list_add(L, &c)) return 1;
      }
      step(F, bw, &ka, &la);
      if (ka <= la) {
        c.k = ka; c.l = la; c.pos = -1;
        c.kind = HPG_BWT_INSERTION; c.base = b;
        if (list_add(L, &c)) return 1;
      }
    }
  }

  for (i = end - 2, j = n - 2; j >= half; i--, j--) {
    res_last = res;
    k = vki[j]; l = vli[j];
    res = l - k;
    if (res == res_last) continue;
    c.k = k; c.l = l; c.pos = i + 2;
    c.kind = HPG_BWT_DELETION; c.base = 0xFF; c.err_pos = i + 1;
    exact_forward(W, F, &c, end);
    if (c.k <= c.l && list_add(L, &c)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      ka = k; la = l;
      step(F, b, &ka, &la);
      if (ka > la) continue;
      c.k = ka; c.l = la; c.pos = i + 1;
      c.kind = HPG_BWT_INSERTION; c.base = b;
      exact_forward(W, F, &c, end);
      if (c.k <= c.l && list_add(L, &c)) return 1;
      if (b != W[i + 1]) {
        c.k = ka; c.l = la; c.pos = i + 2;
        c.kind = HPG_BWT_MISMATCH;
        exact_forward(W, F, &c, end);
        if (c.k <= c.l && list_add(L, &c)) return 1;
      }
    }
  }
  return 0;
}

/* -------------------------------------------------------------- locate -- */

static size_t kar_search(const fmo_index_t *ix, uint64_t key) {
  size_t lo = 0, size = ix->kar_size;
  const uint64_t *p = ix->kar_offset;
  while (size > 0) { /* first offset > key among offset[0..size) */
    size_t w = size / 2;
    if (p[lo + w] <= key) { lo += w + 1; size -= w + 1; }
    else size = w;
  }
  return lo;
}

/* Locate every row of hit `hid`; phys_fw selects the forward (reversed-text) SA. */
static void locate(const fmo_index_t *ix, sink_t *s, uint32_t hid, int64_t k, int64_t l, int phys_fw,
                   uint64_t len_calc) {
  if (k > l) return;
  for (uint64_t j = (uint64_t)k; j <= (uint64_t)l; j++) {
    uint64_t key;
    if (phys_fw)
      key = (uint64_t)(ix->Si.siz - sa_value(ix, &ix->Oi, &ix->Si, (uint32_t)j)) - len_calc - 1;
    else
      key = sa_value(ix, &ix->O, &ix->S, (uint32_t)j);
    size_t id = kar_search(ix, key);
    hpg_loc_t loc;
    memset(&loc, 0, sizeof loc);
    loc.key = key;
    loc.hit = hid;
    if (key + len_calc <= ix->kar_offset[id]) {
      loc.valid = 1;
      loc.chrom = (uint32_t)(id - 1);
      loc.position = ix->kar_start[id - 1] + (key - ix->kar_offset[id - 1]);
    }
    sink_loc(s, &loc);
  }
}

/* ------------------------------------------------ k-error block search -- */
/*
 * BWSearchCPU (search/search.c:1171-1405) as bwt_map_inexact_read_2 drives it
 * (bwt.c:2413-2470): fragment size max(len / 2, 30), hence one or two
 * fragments and at most one error.  Three or more fragments (a caller of
 * BWSearchCPU with a smaller fragment size) add the partial branch passes
 * and change_direction (search/search.h:157-198), which reads the inverse
 * suffix array (R/Ri, loaded by bwt_index_new with inverse_sa); no entry
 * point of bwt.c reaches them, and this restatement refuses them.
 *
 * Results live in lists with the reference's capacity rule (add_result,
 * search/results.h:93-103): a full list refuses the result and the function
 * that tried returns at once ("true").  A list entry is updated in place, as
 * the reference updates the `result` it iterates over.
 */

typedef struct {
  uint8_t dir, nm, kind, base;
  int16_t err_pos, start, pos, end;
  int64_t k, l;
} bres_t; /* the fields of `result` this search touches (one error at most) */

typedef struct {
  bres_t *v;
  uint32_t n, cap;
  int refused; /* a result was refused (reported in rs_truncated bit 0) */
} blist_t;

static int blist_add(blist_t *L, const bres_t *r) {
  if (L->n >= L->cap) {
    L->refused = 1;
    return 1;
  }
  L->v[L->n++] = *r;
  return 0;
}

/* BWExactSearchForward/Backward with an anchor (search/search.h:9-65). */
static void block_exact_forward(const uint8_t *W, const fmo_view_t *v, bres_t *r, bres_t *a) {
  int64_t k = 0, l = 0, k2 = r->k, l2 = r->l;
  int16_t i;
  for (i = r->pos; i <= r->end; i++) {
    step(v, W[i], &k2, &l2);
    if (k2 > l2) break;
    k = k2;
    l = l2;
  }
  memset(a, 0, sizeof *a);
  a->dir = 1;
  a->start = r->pos;
  a->end = (int16_t)(i - 1);
  a->k = k;
  a->l = l;
  a->pos = i;
  r->k = k2;
  r->l = l2;
  r->pos = i;
}

static void block_exact_backward(const uint8_t *W, const fmo_view_t *v, bres_t *r, bres_t *a) {
  int64_t k = 0, l = 0, k2 = r->k, l2 = r->l;
  int16_t i;
  for (i = r->pos; i >= r->start; i--) {
    step(v, W[i], &k2, &l2);
    if (k2 > l2) break;
    k = k2;
    l = l2;
  }
  memset(a, 0, sizeof *a);
  a->dir = 0;
  a->start = (int16_t)(i + 1);
  a->end = r->pos;
  a->k = k;
  a->l = l;
  a->pos = i;
  r->k = k2;
  r->l = l2;
  r->pos = i;
}

/* calculateDBackward / calculateDForward (search/search.c:1045-1169): per
 * position, how many restarts of a greedy exact walk the rest of the read
 * needs -- the lower bound on errors left.  Byte arithmetic as the reference's
 * (uint8_t counter, int8_t total). */
static void block_d_backward(uint8_t *D, const uint8_t *W, int16_t nW, const fmo_view_t *bw, const fmo_view_t *fw,
                             const bres_t *r, int64_t top) {
  uint8_t z = 0;
  int8_t last;
  int64_t k = r->k, l = r->l;
  for (int16_t i = r->pos; i >= 0; i--) {
    step(bw, W[i], &k, &l);
    if (k > l) {
      k = 0;
      l = top;
      z++;
    }
    D[i] = z;
  }
  if (r->end == nW - 1) {
    last = (int8_t)D[0];
  } else {
    k = 0;
    l = top;
    for (int16_t i = (int16_t)(r->end + 1); i < nW; i++) {
      step(fw, W[i], &k, &l);
      if (k > l) {
        k = 0;
        l = top;
        z++;
      }
      D[i] = z;
    }
    last = (int8_t)D[nW - 1];
    for (int16_t i = (int16_t)(r->end + 1); i < nW; i++) D[i] = (uint8_t)(last - D[i]);
  }
  for (int16_t i = r->pos; i >= 0; i--) D[i] = (uint8_t)(last - D[i]);
}

static void block_d_forward(uint8_t *D, const uint8_t *W, int16_t nW, const fmo_view_t *bw, const fmo_view_t *fw,
                            const bres_t *r, int64_t top) {
  uint8_t z = 0;
  int8_t last;
  int64_t k = r->k, l = r->l;
  for (int16_t i = r->pos; i < nW; i++) {
    step(fw, W[i], &k, &l);
    if (k > l) {
      k = 0;
      l = top;
      z++;
    }
    D[i] = z;
  }
  if (r->start == 0) {
    last = (int8_t)D[nW - 1];
  } else {
    k = 0;
    l = top;
    for (int16_t i = (int16_t)(r->start - 1); i >= 0; i--) {
      step(bw, W[i], &k, &l);
      if (k > l) {
        k = 0;
        l = top;
        z++;
      }
      D[i] = z;
    }
    last = (int8_t)D[0];
    for (int16_t i = (int16_t)(r->start - 1); i >= 0; i--) D[i] = (uint8_t)(last - D[i]);
  }
  for (int16_t i = r->pos; i < nW; i++) D[i] = (uint8_t)(last - D[i]);
}

/* BWExactPartialResultsBackward/Forward (search/search.c:471-646): walk each
 * result to the end of the block rule's range; every step whose interval
 * size changes while the error bound D allows one more error is a branch
 * point (rl_next); a walk that covers the rest of the read survives
 * (rl_next_i). */
static int block_partial_backward(const uint8_t *W, const uint8_t *D, uint8_t max_errors, const fmo_view_t *v,
                                  blist_t *prev, blist_t *next, blist_t *next_i, int16_t bs, int16_t last_block) {
  for (uint32_t ii = 0; ii < prev->n; ii++) {
    bres_t *r = &prev->v[ii];
    const int16_t start = r->start, pos = r->pos;
    int64_t k = 0, l = 0, k_next = r->k, l_next = r->l;
    int64_t results, results_next = l_next - k_next;
    const int16_t cb = (int16_t)(pos / bs);
    const uint8_t bound = (uint8_t)(max_errors - r->nm);
    int16_t lbp;
    int complete;
    if (cb < last_block || pos == start - 1) {
      lbp = start;
      complete = 1;
    } else if (cb > last_block) {
      lbp = (int16_t)(((pos + 1) % bs) ? (cb - 1) * bs : cb * bs);
      complete = 0;
    } else if ((pos + 1) % bs) {
      lbp = start;
      complete = 1;
    } else {
      lbp = (int16_t)(cb * bs);
      complete = 0;
    }
    for (int16_t i = pos; i >= lbp; i--) {
      k = k_next;
      l = l_next;
      if (k > l) break;
      step(v, W[i], &k_next, &l_next);
      results = results_next;
      results_next = l_next - k_next;
      if (results == results_next || bound < D[i]) continue;
      r->k = k;
      r->l = l;
      r->pos = i;
      if (blist_add(next, r)) return 1;
    }
    if (complete && k_next <= l_next) {
      r->k = k_next;
      r->l = l_next;
      r->pos = (int16_t)(start - 1);
      if (blist_add(next_i, r)) return 1;
    }
  }
  prev->n = 0;
  return 0;
}

static int block_partial_forward(const uint8_t *W, const uint8_t *D, uint8_t max_errors, const fmo_view_t *v,
                                 blist_t *prev, blist_t *next, blist_t *next_i, int16_t bs, int16_t last_block) {
  for (uint32_t ii = 0; ii < prev->n; ii++) {
    bres_t *r = &prev->v[ii];
    const int16_t pos = r->pos, end = r->end;
    int64_t k = 0, l = 0, k_next = r->k, l_next = r->l;
    int64_t results, results_next = l_next - k_next;
    const int16_t cb = (int16_t)(pos / bs);
    const uint8_t bound = (uint8_t)(max_errors - r->nm);
    int16_t lbp;
    int complete;
    if (cb > last_block || pos == end + 1) {
      lbp = end;
      complete = 1;
    } else if (cb < last_block) {
      lbp = (int16_t)((pos % bs) ? (cb + 2) * bs - 1 : (cb + 1) * bs - 1);
      complete = 0;
    } else if (pos % bs) {
      lbp = end;
      complete = 1;
    } else {
      lbp = (int16_t)((cb + 1) * bs - 1);
      complete = 0;
    }
    for (int16_t i = pos; i <= lbp; i++) {
      k = k_next;
      l = l_next;
      if (k > l) break;
      step(v, W[i], &k_next, &l_next);
      results = results_next;
      results_next = l_next - k_next;
      if (results == results_next || bound < D[i]) continue;
      r->k = k;
      r->l = l;
      r->pos = i;
      if (blist_add(next, r)) return 1;
    }
    if (complete && k_next <= l_next) {
      r->k = k_next;
      r->l = l_next;
      r->pos = (int16_t)(end + 1);
      if (blist_add(next_i, r)) return 1;
    }
  }
  prev->n = 0;
  return 0;
}

/* BWExactFinalResultBackward/Forward (search/search.h:67-155): extend one
 * result over the rest of its range unless the block rule skips it. */
static int block_final_backward(const uint8_t *W, const fmo_view_t *v, bres_t *r, blist_t *fin, int16_t bs,
                                int16_t last_block) {
  const int16_t start = r->start, pos = r->pos;
  const int16_t cb = (int16_t)(pos / bs);
  if (!(cb < last_block || pos == start - 1)) {
    if (cb > last_block) return 0;
    if (!((pos + 1) % bs)) return 0;
  }
  int64_t k = r->k, l = r->l;
  for (int16_t i = pos; i >= start; i--) {
    step(v, W[i], &k, &l);
    if (k > l) break;
  }
  if (k <= l) {
    r->k = k;
    r->l = l;
    r->pos = (int16_t)(start - 1);
    return blist_add(fin, r);
  }
  return 0;
}

static int block_final_forward(const uint8_t *W, const fmo_view_t *v, bres_t *r, blist_t *fin, int16_t bs,
                               int16_t last_block) {
  const int16_t pos = r->pos, end = r->end;
  const int16_t cb = (int16_t)(pos / bs);
  if (!(cb > last_block || pos == end + 1)) {
    if (cb < last_block) return 0;
    if (!(pos % bs)) return 0;
  }
  int64_t k = r->k, l = r->l;
  for (int16_t i = pos; i <= end; i++) {
    step(v, W[i], &k, &l);
    if (k > l) break;
  }
  if (k <= l) {
    r->k = k;
    r->l = l;
    r->pos = (int16_t)(end + 1);
    return blist_add(fin, r);
  }
  return 0;
}

/* BWBranchFinalResultsBackward/Forward (search/search.c:116-469), for
 * results without an earlier error (the only ones one error allows): a
 * deletion, then per base an insertion and a mismatch.  The mismatch starts
 * from the interval the insertion's extension left in the result when that
 * extension survived, as the reference's does (it resets only `pos`). */
static int block_branch_backward(const uint8_t *W, const fmo_view_t *v, blist_t *prev, blist_t *fin, int16_t bs,
                                 int16_t last_block) {
  for (uint32_t ii = 0; ii < prev->n; ii++) {
    bres_t *r = &prev->v[ii];
    if (r->dir != 0) continue;
    const int16_t pos = r->pos;
    if (pos < r->start) {
      if (block_final_backward(W, v, r, fin, bs, last_block)) return 1;
      continue;
    }
    if (r->nm) return -1; /* two errors: not reachable with two fragments */
    const int64_t k = r->k, l = r->l;
    r->nm = 1;
    r->kind = HPG_BWT_DELETION;
    r->base = 0xFF;
    r->err_pos = pos;
    r->pos = (int16_t)(pos - 1);
    if (block_final_backward(W, v, r, fin, bs, last_block)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      int64_t ka = k, la = l;
      step(v, b, &ka, &la);
      if (ka > la) continue;
      if (b != W[pos]) {
        r->k = ka;
        r->l = la;
        r->pos = pos;
        r->kind = HPG_BWT_INSERTION;
        r->base = b;
        if (block_final_backward(W, v, r, fin, bs, last_block)) return 1;
        r->pos = (int16_t)(pos - 1);
        r->kind = HPG_BWT_MISMATCH;
        if (block_final_backward(W, v, r, fin, bs, last_block)) return 1;
      }
    }
  }
  prev->n = 0;
  return 0;
}

static int block_branch_forward(const uint8_t *W, const fmo_view_t *v, blist_t *prev, blist_t *fin, int16_t bs,
                                int16_t last_block) {
  for (uint32_t ii = 0; ii < prev->n; ii++) {
    bres_t *r = &prev->v[ii];
    if (r->dir != 1) continue;
    const int16_t pos = r->pos;
    if (pos > r->end) {
      if (blist_add(fin, r)) return 1;
      continue;
    }
    if (r->nm) return -1;
    const int64_t k = r->k, l = r->l;
    r->nm = 1;
    r->kind = HPG_BWT_DELETION;
    r->base = 0xFF;
    r->err_pos = pos;
    r->pos = (int16_t)(pos + 1);
    if (block_final_forward(W, v, r, fin, bs, last_block)) return 1;
    for (uint8_t b = 0; b < 4; b++) {
      int64_t ka = k, la = l;
      step(v, b, &ka, &la);
      if (ka > la) continue;
      if (b != W[pos]) {
        r->k = ka;
        r->l = la;
        r->pos = pos;
        r->kind = HPG_BWT_INSERTION;
        r->base = b;
        if (block_final_forward(W, v, r, fin, bs, last_block)) return 1;
        r->pos = (int16_t)(pos + 1);
        r->kind = HPG_BWT_MISMATCH;
        if (block_final_forward(W, v, r, fin, bs, last_block)) return 1;
      }
    }
  }
  prev->n = 0;
  return 0;
}

/* BWSearchCPU for one or two fragments.  L: prev, next, final, anchors. */
static void block_search(const uint8_t *W, int16_t nW, const fmo_view_t *bw, const fmo_view_t *fw, blist_t *L,
                         int16_t fragsize, int type, uint8_t *D, int64_t top) {
  blist_t *prev = &L[0], *next = &L[1], *fin = &L[2], *anch = &L[3];
  const int16_t fragments = (int16_t)((uint64_t)nW / (uint64_t)fragsize);
  int16_t half = (int16_t)(fragments / 2);
  if (fragments % 2) half++;
  anch->n = 0;
  bres_t r, a;
  memset(&r, 0, sizeof r);
  if (fragments <= 1) {
    r.k = 0;
    r.l = top;
    r.start = 0;
    r.end = (int16_t)(nW - 1);
    if (type == 0) {
      r.dir = 1;
      r.pos = 0;
      block_exact_forward(W, fw, &r, &a);
    } else {
      r.dir = 0;
      r.pos = (int16_t)(nW - 1);
      block_exact_backward(W, bw, &r, &a);
    }
    if (blist_add(anch, &a)) return;
    if (r.k <= r.l) blist_add(fin, &r);
    return;
  }
  if (fragments > 2) return; /* needs the inverse suffix array (header note) */

  /* block 0, forward over the first fragment, then the rest of the read */
  prev->n = next->n = 0;
  r.dir = 1;
  r.k = 0;
  r.l = top;
  r.pos = 0;
  r.start = 0;
  r.end = (int16_t)(fragsize - 1);
  block_exact_forward(W, fw, &r, &a);
  if (blist_add(anch, &a)) return;
  r.end = (int16_t)(nW - 1);
  if (r.k <= r.l) {
    block_d_forward(D, W, nW, bw, fw, &r, top);
    if (blist_add(prev, &r)) return;
    /* err_count = fragments - 1 = 1: one partial pass, then the final branches */
    if (!block_partial_forward(W, D, (uint8_t)(fragments - 1), fw, prev, next, fin, fragsize, (int16_t)(half - 1)))
      block_branch_forward(W, fw, next, fin, fragsize, (int16_t)(half - 1));
  }

  /* last block, backward over the last fragment, then the rest of the read */
  prev->n = next->n = 0;
  memset(&r, 0, sizeof r);
  r.dir = 0;
  r.k = 0;
  r.l = top;
  r.pos = (int16_t)(nW - 1);
  r.start = (int16_t)(fragsize * (fragments - 1));
  r.end = (int16_t)(nW - 1);
  block_exact_backward(W, bw, &r, &a);
  if (blist_add(anch, &a)) return;
  r.start = 0;
  if (r.k <= r.l) {
    block_d_backward(D, W, nW, bw, fw, &r, top);
    if (blist_add(prev, &r)) return;
    if (!block_partial_backward(W, D, (uint8_t)(fragments - 1), bw, prev, next, fin, fragsize, 0))
      block_branch_backward(W, bw, next, fin, fragsize, 0);
  }
}

/* ------------------------------------------------------------ per read -- */

/* Rows of a list's kept hits, and whether a locate limit leaves them unlocated
 * (the product's bwt_gpu_set_locate_limit: lists over the limit keep their hits,
 * get no located rows and bit 1 of their truncation flag). */
static int over_limit(const hpg_hit_t *h, uint32_t n, uint64_t limit) {
  if (!limit) return 0;
  uint64_t rows = 0;
  for (uint32_t t = 0; t < n; t++)
    if (h[t].k <= h[t].l) rows += (uint64_t)(h[t].l - h[t].k + 1);
  return rows > limit;
}

static void one_read(const fmo_index_t *ix, int mode, uint32_t rd, const char *seq, size_t len, uint32_t max_results,
                     uint64_t limit, sink_t *s, hpg_hit_t *lbuf, uint8_t *code, int64_t *vecs, bres_t *bbuf,
                     uint32_t *rs_count, uint8_t *rs_trunc, hpg_block_anchor_t *anchors, uint8_t *n_anchors) {
  if (len < 3 || len > 32767) return;
  for (size_t i = 0; i < len; i++) {
    code[i] = ix->code_of[(unsigned char)seq[i]];
    if (code[i] == 0xFF) return; /* outside the alphabet: unmappable */
  }
  int16_t start = 0, end = (int16_t)(len - 1);
  int64_t top = (int64_t)ix->S.siz - 1;

  if (mode == HPG_BWT_MODE_EXACT) {
    for (int type = 1; type >= 0; type--) {
      const fmo_view_t *v = type ? &ix->bw : &ix->fw_rev;
      cursor_t c;
      memset(&c, 0, sizeof c);
      c.k = 0; c.l = top; c.pos = end;
      exact_backward((const uint8_t *)code, v, &c, start);
      if (c.k <= c.l) {
        hpg_hit_t h;
        memset(&h, 0, sizeof h);
        h.read = rd; h.strand = (uint8_t)!type; h.k = c.k; h.l = c.l;
        uint32_t hid = (uint32_t)s->n_hits;
        sink_hit(s, &h);
        rs_count[2 * (size_t)rd + !type] = 1;
        if (over_limit(&h, 1, limit)) {
          rs_trunc[2 * (size_t)rd + !type] |= 2;
          continue;
        }
        locate(ix, s, hid, c.k, c.l, type ? 0 : 1, len);
      }
    }
    return;
  }

  if (mode == HPG_BWT_MODE_BLOCK) {
    /* bwt_map_inexact_read_2 (bwt.c:2401-2470): fragment size len / 2, at
     * least 30; lists of capacity filter_read_mappings, anchors of 2 */
    int16_t frag = (int16_t)(len / 2);
    if (frag < 30) frag = 30;
    for (int type = 1; type >= 0; type--) {
      const size_t t2 = 2 * (size_t)rd + !type;
      blist_t L[4] = {{bbuf, 0, max_results, 0},
                      {bbuf + (size_t)max_results + 1, 0, max_results, 0},
                      {bbuf + 2 * ((size_t)max_results + 1), 0, max_results, 0},
                      {bbuf + 3 * ((size_t)max_results + 1), 0, 2, 0}};
      if (type)
        block_search(code, (int16_t)len, &ix->bw, &ix->fw, L, frag, type, (uint8_t *)vecs, top);
      else
        block_search(code, (int16_t)len, &ix->fw_rev, &ix->bw_rev, L, frag, type, (uint8_t *)vecs, top);
      const blist_t *fin = &L[2], *anch = &L[3];
      for (uint32_t t = 0; t < fin->n; t++) {
        const bres_t *b = &fin->v[t];
        hpg_hit_t *h = &lbuf[t];
        memset(h, 0, sizeof *h);
        h->read = rd;
        h->strand = (uint8_t)!type;
        h->dir = b->dir;
        h->nm = b->nm;
        if (b->nm) {
          h->err_kind = b->kind;
          h->err_base = b->base;
          h->err_pos = b->err_pos;
        }
        h->k = b->k;
        h->l = b->l;
      }
      const int skip = over_limit(lbuf, fin->n, limit);
      const int refused = L[0].refused | L[1].refused | L[2].refused | L[3].refused;
      rs_trunc[t2] = (uint8_t)(refused | (skip ? 2 : 0));
      rs_count[t2] = fin->n;
      if (n_anchors) {
        n_anchors[t2] = (uint8_t)anch->n;
        for (uint32_t a = 0; a < anch->n; a++) {
          hpg_block_anchor_t *o = &anchors[2 * t2 + a];
          memset(o, 0, sizeof *o);
          o->k = anch->v[a].k;
          o->l = anch->v[a].l;
          o->start = anch->v[a].start;
          o->end = anch->v[a].end;
          o->pos = anch->v[a].pos;
          o->dir = anch->v[a].dir;
        }
      }
      for (uint32_t t = 0; t < fin->n; t++) {
        const hpg_hit_t *h = &lbuf[t];
        uint32_t hid = (uint32_t)s->n_hits;
        sink_hit(s, h);
        if (skip) continue;
        uint8_t err = h->nm ? h->err_kind : 0;
        int direction = type ? h->dir : !h->dir;
        uint64_t len_calc = len;
        if (err == HPG_BWT_DELETION) len_calc--;
        else if (err == HPG_BWT_INSERTION) len_calc++;
        locate(ix, s, hid, h->k, h->l, direction, len_calc);
      }
    }
    return;
  }

  int64_t *k1 = vecs, *l1 = k1 + len, *ki1 = l1 + len, *li1 = ki1 + len;
  int64_t *k0 = li1 + len, *l0 = k0 + len, *ki0 = l0 + len, *li0 = ki0 + len;
  vector_backward(code, start, end, 0, top, k1, l1, &ix->bw);
  vector_forward(code, start, end, 0, top, ki1, li1, &ix->fw);
  vector_forward(code, start, end, 0, top, k0, l0, &ix->bw_rev);
  vector_backward(code, start, end, 0, top, ki0, li0, &ix->fw_rev);
  for (int type = 1; type >= 0; type--) {
    list_t L = {lbuf, 0, max_results, rd, (uint8_t)!type};
    int over = type ? search1_helper(code, start, end, k1, l1, ki1, li1, &ix->bw, &ix->fw, &L)
                    : search1_helper(code, start, end, ki0, li0, k0, l0, &ix->fw_rev, &ix->bw_rev, &L);
    const int skip = over_limit(lbuf, L.n, limit);
    rs_trunc[2 * (size_t)rd + !type] = (uint8_t)(over | (skip ? 2 : 0));
    rs_count[2 * (size_t)rd + !type] = L.n;
    for (uint32_t t = 0; t < L.n; t++) {
      const hpg_hit_t *h = &lbuf[t];
      uint32_t hid = (uint32_t)s->n_hits;
      sink_hit(s, h);
      if (skip) continue;
      uint8_t err = h->nm ? h->err_kind : 0;
      int direction = type ? h->dir : !h->dir;
      uint64_t len_calc = len;
      if (err == HPG_BWT_DELETION) len_calc--;
      else if (err == HPG_BWT_INSERTION) len_calc++;
      locate(ix, s, hid, h->k, h->l, direction, len_calc);
    }
  }
}

/* Batch driver: reads are split into chunks processed by `threads` OpenMP
 * threads (dynamic schedule, as bwt.c:1134), then merged in read order. */
static int search_impl(const fmo_index_t *ix, int mode, const char *seqs, const uint64_t *offsets, size_t n_reads,
                       uint32_t max_results, uint64_t locate_limit, int threads, hpg_result_set_t *out,
                       hpg_block_anchor_t *anchors, uint8_t *n_anchors) {
  memset(out, 0, sizeof *out);
  out->n_reads = n_reads;
  out->rs_count = (uint32_t *)calloc(2 * n_reads + 1, sizeof(uint32_t));
  out->rs_truncated = (uint8_t *)calloc(2 * n_reads + 1, 1);
  if (threads < 1) threads = 1;
  size_t maxlen = 3;
  for (size_t r = 0; r < n_reads; r++) {
    size_t len = (size_t)(offsets[r + 1] - offsets[r]);
    if (len > maxlen) maxlen = len;
  }
  if (maxlen > 32767) maxlen = 32767;
  size_t nchunks = n_reads ? (n_reads + 255) / 256 : 0;
  sink_t *sinks = (sink_t *)calloc(nchunks + 1, sizeof(sink_t));
#pragma omp parallel num_threads(threads)
  {
    hpg_hit_t *lbuf = (hpg_hit_t *)malloc(((size_t)max_results + 1) * sizeof(hpg_hit_t));
    uint8_t *code = (uint8_t *)malloc(maxlen + 1);
    int64_t *vecs = (int64_t *)malloc(8 * (maxlen + 1) * sizeof(int64_t));
    bres_t *bbuf = mode == HPG_BWT_MODE_BLOCK ? (bres_t *)malloc((3 * ((size_t)max_results + 1) + 2) * sizeof(bres_t))
                                              : NULL;
#pragma omp for schedule(dynamic, 1)
    for (size_t ch = 0; ch < nchunks; ch++) {
      size_t r0 = ch * 256, r1 = r0 + 256 < n_reads ? r0 + 256 : n_reads;
      for (size_t r = r0; r < r1; r++)
        one_read(ix, mode, (uint32_t)r, seqs + offsets[r], (size_t)(offsets[r + 1] - offsets[r]), max_results,
                 locate_limit, &sinks[ch], lbuf, code, vecs, bbuf, out->rs_count, out->rs_truncated, anchors,
                 n_anchors);
    }
    free(bbuf);
    free(lbuf);
    free(code);
    free(vecs);
  }
  size_t nh = 0, nl = 0;
  for (size_t ch = 0; ch < nchunks; ch++) {
    nh += sinks[ch].n_hits;
    nl += sinks[ch].n_locs;
  }
  out->hits = (hpg_hit_t *)malloc((nh + 1) * sizeof(hpg_hit_t));
  out->locs = (hpg_loc_t *)malloc((nl + 1) * sizeof(hpg_loc_t));
  size_t hb = 0, lb = 0;
  for (size_t ch = 0; ch < nchunks; ch++) {
    sink_t *s = &sinks[ch];
    if (s->n_hits) memcpy(out->hits + hb, s->hits, s->n_hits * sizeof(hpg_hit_t));
    for (size_t t = 0; t < s->n_locs; t++) {
      out->locs[lb + t] = s->locs[t];
      out->locs[lb + t].hit += (uint32_t)hb;
    }
    hb += s->n_hits;
    lb += s->n_locs;
    free(s->hits);
    free(s->locs);
  }
  free(sinks);
  out->n_hits = nh;
  out->n_locs = nl;
  return 0;
}

int fmo_search_limit(const fmo_index_t *ix, int mode, const char *seqs, const uint64_t *offsets, size_t n_reads,
                     uint32_t max_results, uint64_t locate_limit, int threads, hpg_result_set_t *out) {
  return search_impl(ix, mode, seqs, offsets, n_reads, max_results, locate_limit, threads, out, NULL, NULL);
}

/* The k-error block search with its anchors: anchors[2 * (2 * read + strand)
 * + a] for a < n_anchors[2 * read + strand] (arrays of 4 n and 2 n entries,
 * n_anchors zeroed here). */
int fmo_block_search(const fmo_index_t *ix, const char *seqs, const uint64_t *offsets, size_t n_reads,
                     uint32_t max_results, uint64_t locate_limit, int threads, hpg_result_set_t *out,
                     hpg_block_anchor_t *anchors, uint8_t *n_anchors) {
  if (n_anchors) memset(n_anchors, 0, 2 * n_reads);
  return search_impl(ix, HPG_BWT_MODE_BLOCK, seqs, offsets, n_reads, max_results, locate_limit, threads, out,
                     anchors, n_anchors);
}

int fmo_search(const fmo_index_t *ix, int mode, const char *seqs, const uint64_t *offsets, size_t n_reads,
               uint32_t max_results, int threads, hpg_result_set_t *out) {
  return fmo_search_limit(ix, mode, seqs, offsets, n_reads, max_results, 0, threads, out);
}

void fmo_result_free(hpg_result_set_t *out) {
  free(out->hits);
  free(out->locs);
  free(out->rs_count);
  free(out->rs_truncated);
  memset(out, 0, sizeof *out);
}

int fmo_max_threads(void) { return omp_get_max_threads(); }
