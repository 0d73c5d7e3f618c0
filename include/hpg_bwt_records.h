/*
 * hpg_bwt_records.h -- flat, canonical result records of the FM-index read
 * mapping hot path (exact backward search, BWSearch1 1-error backtracking,
 * sampled-SA locate).
 *
 * These plain-C records are what the GPU batch entry points return, and what
 * the CPU oracles emit for parity checks.  They carry exactly the fields of
 * the reference's `result` (c/src/aligners/bwt/search/results.h:13-21) that
 * decide the mapping output, plus the per-row locate values of
 * c/src/aligners/bwt/bwt.c:2158-2166.
 *
 * Ordering contract:
 *   hits  : by read, then strand ('+' = type 1 first, as bwt.c:1989), then the
 *           order in which BWSearch1VectorHelper appends to its results_list
 *           (search/search.c:1491-1709).  Truncation at max_results keeps the
 *           first max_results hits of that order (search/results.h:93-103).
 *   locs  : by hit, then suffix-array row ascending (bwt.c:2158).
 */
#ifndef HPG_BWT_RECORDS_H
#define HPG_BWT_RECORDS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Search modes of the batch entry points. */
#define HPG_BWT_MODE_EXACT   0 /* BWExactSearchBackward on both strands: '+' over backward,
                                  '-' over forward_rev (search/search.h:9-36). */
#define HPG_BWT_MODE_SEARCH1 1 /* 4 vector searches + BWSearch1VectorHelper per strand,
                                  as bwt.c:1940-2002. */
#define HPG_BWT_MODE_BLOCK   2 /* k-error block search BWSearchCPU per strand with the
                                  fragment size of bwt_map_inexact_read_2 (bwt.c:2413-2470;
                                  search/search.c:1171-1405): max(len / 2, 30), so one
                                  error; hits in rl_final order. bwt_gpu_block_search. */

/* Error kinds (c/src/aligners/bwt/bwt_commons.h:15-18). DELETION means one
 * extra base in the read, INSERTION one base missing from it. */
#define HPG_BWT_MATCH     0
#define HPG_BWT_DELETION  1
#define HPG_BWT_MISMATCH  2
#define HPG_BWT_INSERTION 3

/* Strand codes: the reference's `type` 1 ('+') is strand 0, type 0 ('-') is 1. */
#define HPG_BWT_STRAND_PLUS  0
#define HPG_BWT_STRAND_MINUS 1

typedef struct {
  uint32_t read;     /* read index within the batch */
  uint8_t strand;    /* HPG_BWT_STRAND_* (= !type) */
  uint8_t dir;       /* result.dir: 0 backward half, 1 forward half */
  uint8_t nm;        /* result.num_mismatches (0 or 1) */
  uint8_t err_kind;  /* err_kind[0]; 0 when nm == 0 (the reference leaves it unset) */
  uint8_t err_base;  /* err_base[0]; 0 when nm == 0 */
  uint8_t pad0;
  int16_t err_pos;   /* err_pos[0];  0 when nm == 0 */
  uint32_t pad1;
  int64_t k, l;      /* suffix-array interval; k > l (empty) is possible */
} hpg_hit_t;         /* 32 bytes */

typedef struct {
  uint64_t key;      /* text offset from the sampled-SA walk (size_t arithmetic, bwt.c:2159-2161) */
  uint64_t position; /* start[idx-1] + key - offset[idx-1] (bwt.c:2166); 0 when !valid */
  uint32_t hit;      /* index of the owning hit */
  uint32_t chrom;    /* idx - 1 from binsearch (search/io.h:43-64); 0 when !valid */
  uint32_t valid;    /* key + len_calc <= offset[idx] (bwt.c:2164) */
  uint32_t pad;
} hpg_loc_t;         /* 32 bytes */

/* Anchor of the k-error block search: the `result` one block's exact search
 * leaves in rl_anchor (BWExactSearchBackward/Forward with r_anchor,
 * search/search.h:9-65, called from BWSearchCPU, search/search.c:1171-1405):
 * the last non-empty interval before the first failing base and the read span
 * it matched.  At most two per (read, strand), in the order BWSearchCPU adds
 * them (the first block's forward search, then the last block's backward one). */
typedef struct {
  int64_t k, l;      /* 0, 0 when the block's first base already failed */
  int16_t start;     /* matched span start..end; end = start - 1 when empty */
  int16_t end;
  int16_t pos;       /* where the search stopped */
  uint8_t dir;       /* 0 backward search, 1 forward search */
  uint8_t pad;
} hpg_block_anchor_t; /* 24 bytes */

typedef struct {
  size_t n_reads;
  size_t n_hits;
  hpg_hit_t *hits;
  size_t n_locs;
  hpg_loc_t *locs;
  uint32_t *rs_count;    /* [2*n_reads] hits kept per (read, strand) */
  uint8_t *rs_truncated; /* [2*n_reads] bit 0: the helper overflowed max_results;
                          bit 1: rows not located (over the locate limit) */
} hpg_result_set_t;

#ifdef __cplusplus
}
#endif

#endif /* HPG_BWT_RECORDS_H */
