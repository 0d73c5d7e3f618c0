/*
 * hpg_bwt_api.h -- the alignment-list entry points of hpg-libs' FM-index mapper
 * (c/src/aligners/bwt/bwt.h), served from the GPU.
 *
 * A caller built against hpg-libs keeps its own containers and bioformats
 * (array_list_t, alignment_t, fastq_read_t, fastq_batch_t): the types below
 * have the same layout and are skipped when the hpg-libs headers were
 * included first (their include guards).  The library creates alignments with
 * alignment_new() and appends them with array_list_insert(), resolved at load
 * time to the caller's hpg-libs; processes without hpg-libs get the
 * library's own definitions of those container functions (same behaviour).
 *
 * Searches run as one GPU batch per call (a per-read call is a batch of one):
 * exact backward search or BWSearch1 on the device, then the SA rows the
 * reference would locate, then the alignment records on the host, following
 * bwt.c's rules and observable quirks (listed per function).
 */
#ifndef HPG_BWT_API_H
#define HPG_BWT_API_H

#include <pthread.h>
#include <stddef.h>
#include <stdint.h>

#include "hpg_bwt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- hpg-libs types (c/src/containers/array_list.h:29-43,
 * c/src/bioformats/bam/alignment.h:39-69, c/src/bioformats/fastq/fastq_read.h:27-42,
 * c/src/bioformats/fastq/fastq_batch.h:24-34, c/src/aligners/bwt/bwt.h:173-179) ---- */
#ifndef ARRAY_LIST_H
#define ARRAY_LIST_H
#ifndef COLLECTION_MODE_SYNCHRONIZED
#define COLLECTION_MODE_SYNCHRONIZED 1
#define COLLECTION_MODE_ASYNCHRONIZED 2
#endif
typedef struct array_list {
  size_t capacity;
  size_t size;
  float realloc_factor;
  int mode;
  int flag;
  int (*compare_fn)(const void *, const void *);
  pthread_mutex_t lock;
  pthread_cond_t condition;
  void **items;
} array_list_t;
array_list_t *array_list_new(size_t initial_capacity, float realloc_factor, int SYNC_MODE);
void array_list_free(array_list_t *array_list_p, void (*data_callback)(void *));
int array_list_insert(void *item_p, array_list_t *array_list_p);
size_t array_list_size(array_list_t *array_list_p);
void *array_list_get(size_t index, array_list_t *array_list_p);
void *array_list_remove_at(size_t index, array_list_t *array_list_p);
int array_list_clear(array_list_t *array_list_p, void (*data_callback)(void *));
void array_list_set_flag(int flag, array_list_t *array_list_p);
int array_list_get_flag(array_list_t *array_list_p);
#endif

#ifndef ALIGNMENTS_H
#define ALIGNMENTS_H
typedef struct alignment {
  int optional_fields_length;
  unsigned int chromosome;
  int position;
  int mate_position;
  int mate_chromosome;
  int template_length;
  int map_quality;
  int mapq;
  int num_cigar_operations;
  int map_len;
  uint8_t is_paired_end;
  uint8_t is_paired_end_mapped;
  uint8_t is_seq_mapped;
  uint8_t is_mate_mapped;
  uint8_t seq_strand;
  uint8_t mate_strand;
  uint8_t pair_num;
  uint8_t secondary_alignment;
  uint8_t fails_quality_check;
  uint8_t pc_optical_duplicate;
  char *query_name;
  char *sequence;
  char *quality;
  char *cigar;
  uint8_t *optional_fields;
  void *alig_data;
} alignment_t;
alignment_t *alignment_new(void);
void alignment_free(alignment_t *alignment_p);
#endif

#ifndef FASTQ_READ_H
#define FASTQ_READ_H
typedef struct fastq_read {
  char *id;
  char *sequence;
  char *revcomp;
  char *quality;
  char *rev_quality;
  char *adapter;
  char *adapter_revcomp;
  char *adapter_quality;
  int length;
  int adapter_length;
  int adapter_strand;
} fastq_read_t;
#endif

#ifndef FASTQ_BATCH_H
#define FASTQ_BATCH_H
typedef struct fastq_batch {
  unsigned long num_reads;
  unsigned long data_indices_size;
  unsigned long data_size;
  int source_id;
  int *header_indices;
  char *header;
  int *data_indices;
  char *seq;
  char *quality;
} fastq_batch_t;
#endif

#ifndef HPG_BWT_ANCHOR_DEFINED
#define HPG_BWT_ANCHOR_DEFINED
#define BACKWARD_ANCHOR 0
#define FORWARD_ANCHOR 1
typedef struct bwt_anchor {
  int strand;
  int chromosome;
  size_t start;
  size_t end;
  int type;
} bwt_anchor_t;
#endif

/* ---- hpg-libs linked list (c/src/containers/linked_list.h:35-60) ---- */
#ifndef LINKED_LIST_H
#define LINKED_LIST_H
typedef struct linked_list_item {
  void *item;
  struct linked_list_item *prev;
  struct linked_list_item *next;
} linked_list_item_t;
typedef struct linked_list {
  size_t size;
  int mode;
  int flag;
  int (*compare_fn)(const void *, const void *);
  pthread_mutex_t lock;
  pthread_cond_t condition;
  linked_list_item_t *first;
  linked_list_item_t *last;
} linked_list_t;
linked_list_t *linked_list_new(int SYNC_MODE);
void linked_list_free(linked_list_t *linked_list_p, void (*data_callback)(void *));
int linked_list_insert(void *item_p, linked_list_t *linked_list_p);
int linked_list_insert_last(void *item_p, linked_list_t *linked_list_p);
size_t linked_list_size(linked_list_t *linked_list_p);
void *linked_list_get_first(linked_list_t *linked_list_p);
void *linked_list_get_last(linked_list_t *linked_list_p);
typedef struct linked_list_iterator {
  linked_list_t *linked_list_p;
  linked_list_item_t *curr_pos;
} linked_list_iterator_t;
linked_list_iterator_t *linked_list_iterator_new(linked_list_t *linked_list_p);
void linked_list_iterator_free(linked_list_iterator_t *iterator_p);
void *linked_list_iterator_curr(linked_list_iterator_t *iterator_p);
void *linked_list_iterator_next(linked_list_iterator_t *iterator_p);
#endif

/* ---- seeds and candidate alignment locations (bwt.h:56-66,93-111,123-142,185-198) ---- */
#ifndef HPG_BWT_CAL_TYPES_DEFINED
#define HPG_BWT_CAL_TYPES_DEFINED
typedef struct cal_optarg {
  size_t min_cal_size;
  size_t max_cal_distance;
  size_t num_seeds;
  size_t min_num_seeds_in_cal;
  size_t seed_size;
  size_t min_seed_size;
  size_t num_errors;
  size_t max_intron_size;
  size_t min_intron_size;
} cal_optarg_t;

typedef struct seed_region {
  int read_start;
  int read_end;
  size_t genome_start;
  size_t genome_end;
  int id;
  int fusion_left;
  int fusion_right;
  int strand;
  int chromosome_id;
  int num_mismatches;
  int pos_err;
  int type_err;
  array_list_t *errors_list;
  void *info;
} seed_region_t;

typedef struct cal {
  size_t chromosome_id;
  short int strand;
  size_t start;
  size_t end;
  size_t num_seeds;
  int read_area;
  int l_flank;
  int r_flank;
  int fill_gaps;
  int num_targets;
  int type_seeds;
  int num_mismatches;
  linked_list_t *sr_list;
  linked_list_t *sr_duplicate_list;
  array_list_t *candidates_seeds_start;
  array_list_t *candidates_seeds_end;
  void *info;
} cal_t;

typedef struct region {
  size_t chromosome_id;
  short int strand;
  size_t start;
  size_t end;
  size_t seq_start;
  size_t seq_end;
  size_t seq_len;
  int id;
  int pos_err;
  int type_err;
} region_t;
#endif

/* bwt.c:128-156, 174-212, 239-249, 282-313, 385-409 */
cal_optarg_t *cal_optarg_new(const size_t min_cal_size, const size_t max_cal_distance, const size_t num_seeds,
                             const size_t min_num_seeds_in_cal, const size_t seed_size, const size_t min_seed_size,
                             const size_t num_errors, const size_t max_intron_size, const size_t min_intron_size);
void cal_optarg_free(cal_optarg_t *optarg);
cal_t *cal_new(const size_t chromosome_id, const short int strand, const size_t start, const size_t end,
               const size_t num_seeds, linked_list_t *sr_list, linked_list_t *sr_duplicate_list);
void cal_free(cal_t *cal);
seed_region_t *seed_region_new(int read_start, int read_end, size_t genome_start, size_t genome_end, int id,
                               int pos_err, int type_err);
void seed_region_free(seed_region_t *seed_region);
region_t *region_bwt_new(const size_t chromosome_id, const short int strand, const size_t start, const size_t end,
                         const size_t seq_start, const size_t seq_end, const size_t seq_len, const int id);
void region_bwt_free(region_t *region);

/* ---- seeds (bwt.c:1200-1294, 3577-3630) ----
 * bwt_map_exact_seed: the codes seq[seq_start .. seq_end] (both ends
 * included) searched exactly on the '+' strand (backward over the backward
 * index) and the '-' strand (the complemented seed forward over the same
 * index, i.e. its reverse complement); the '+' rows, then the '-' rows, are
 * located on the backward suffix array unless the rows counted so far exceed
 * filter_seed_mappings (a strand over the filter adds nothing, and the count
 * carries to the next strand).  Every row inside one chromosome becomes a
 * region_t appended to mapping_list: chromosome 1-based, strand 0 '+' / 1 '-',
 * genome start 1-based and end = start + (seq_end - seq_start), read span on
 * the strand searched, seq_len, the seed id.  pos_err and type_err are 0 (the
 * reference leaves them unset).  Seeds that reach past the read (the reference
 * reads beyond its buffer there) map nothing.  Returns the regions added.
 * bwt_map_exact_seeds_seq: the reference's seed plan over an ASCII read (seed
 * size 16 when <= 10; a 16-base seed at seed_size/2, consecutive seeds, the
 * last seed_size bases when the length is not a multiple, a 16-base seed
 * ending seed_size/2 before the end), all seeds in one GPU pass; returns the
 * list's size.  padding_*, min_seed_size and step_id are ignored, as in the
 * reference. */
size_t bwt_map_exact_seed(uint8_t *seq, size_t seq_len, size_t seq_start, size_t seq_end, bwt_optarg_t *bwt_optarg,
                          bwt_index_t *index, array_list_t *mapping_list, int id);
size_t bwt_map_exact_seeds_seq(int padding_left, int padding_right, char *seq, size_t seed_size,
                               size_t min_seed_size, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                               array_list_t *mapping_list, unsigned char step_id);
/* bwt_map_exact_seeds_by_region (bwt.c:4033-4080): the seeds of seed_size
 * (16 when <= 10) tiling the read window [start_position, end_position), ids
 * from 1, plus the window's last seed_size bases when its length is not a
 * multiple, each mapped as bwt_map_exact_seed does; returns the list's size.
 * min_seed_size is ignored, as in the reference. */
size_t bwt_map_exact_seeds_by_region(int start_position, int end_position, char *seq, int seed_size,
                                     int min_seed_size, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                                     array_list_t *mapping_list);

/* ---- candidate alignment locations (bwt.c:3631-3642, 3832-4031, 4378-4646, 4652-4824) ----
 * bwt_generate_cals: the seed plan of bwt_map_exact_seeds_seq; each seed's
 * regions, last first, merged into per-(strand, chromosome) lists of short
 * CALs within max_cal_distance = the read length (my_cp_list_append_linked_list,
 * seeds of one id after the first kept in a duplicate list); then, per
 * chromosome 0..nchromosomes and strand, every short CAL of at least
 * min_cal_size bases becomes a cal_t appended to cal_list, its seeds merged
 * by genome position (append_seed_region_linked_list), with the seeds of the
 * smaller neighbouring CALs within max_intron_size that lie before its first
 * seed (candidates_seeds_start, id 0) or after its last (candidates_seeds_end,
 * id 1).  Returns the list's size.
 * bwt_generate_cals_batch (no reference counterpart): the same for
 * seqs[0..num_reads) into cal_lists[i], with the seeds of every read in one
 * GPU pass and the CALs built on the host threads. */
size_t bwt_generate_cals(char *seq, size_t seed_size, bwt_optarg_t *bwt_optarg, cal_optarg_t *cal_optarg,
                         bwt_index_t *index, array_list_t *cal_list, unsigned int nchromosomes);
size_t bwt_generate_cals_batch(char **seqs, size_t num_reads, size_t seed_size, bwt_optarg_t *bwt_optarg,
                               cal_optarg_t *cal_optarg, bwt_index_t *index, array_list_t **cal_lists,
                               unsigned int nchromosomes);

/* bwt.h:181-182 */
bwt_anchor_t *bwt_anchor_new(int strand, int chromosome, size_t start, size_t end, int type);
void bwt_anchor_free(bwt_anchor_t *bwt_anchor);
/* bwt.h:326,330: reverse complement in place (non-ACGT -> 'N'); reverse `length` bytes into dsp and
 * terminate it at dsp[length]. */
void seq_reverse_complementary(char *seq, unsigned int len);
char *reverse_str(char *src, char *dsp, size_t length);

/* ---- exact mapping (bwt.c:889-1163) ----
 * Per read: '+' is BWExactSearchBackward over the backward index; '-' is
 * BWExactSearchForward over forward_rev (so it rarely finds the reverse
 * strand), both located on the backward suffix array; an interval of at least
 * filter_read_mappings rows is cut to its first two rows; every valid row
 * becomes an alignment with cigar "<len>=", map quality 254, the first one
 * primary.  bwt_map_exact_seq prints "\tIn function ...\n" per read, like the
 * reference.  bwt_map_exact_seqs appends in read order (the reference's order
 * depends on its OpenMP schedule; with one thread they agree). */
size_t bwt_map_exact_seq(char *seq, bwt_optarg_t *bwt_optarg, bwt_index_t *index, array_list_t *mapping_list);
size_t bwt_map_exact_read(fastq_read_t *read, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                          array_list_t *mapping_list);
size_t bwt_map_exact_seqs(char **seqs, size_t num_reads, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                          char *out_status, array_list_t *mapping_list);
size_t bwt_map_exact_batch(fastq_batch_t *batch, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                           fastq_batch_t *unmapped_batch, array_list_t *mapping_list);

/* ---- inexact mapping (bwt.c:1879-2310) ----
 * BWSearch1 on both strands with filter_read_mappings as the result-list
 * capacity; only the exact hits become alignments (cigar "<len>M", 0-based
 * positions); a strand whose hits span more than filter_read_mappings rows
 * drops every alignment of the call from that strand on and sets the list
 * flag to 2; alignments closer than 10 bp on one chromosome are merged; the
 * read quality and the AS/NH/NM optional fields are added; reads shorter than
 * 5 bases get one unmapped record.  When the list ends empty with flag 1, the
 * longest exact prefix/suffix matches of the four vector searches are located
 * as bwt_anchor_t items (at most 50 rows each). */
size_t bwt_map_inexact_read(fastq_read_t *read, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                            array_list_t *mapping_list);
/* Batch forms declared by bwt.h:362-366,519-524 (their reference bodies are
 * commented out): every read is mapped as bwt_map_inexact_read maps it into a
 * fresh list.  _batch appends the alignments in read order and copies reads
 * without any to unmapped_batch; _array_list maps reads[i] (fastq_read_t *)
 * into lists[i] (whose flag the caller sets, 1 asking for anchors) and lists
 * the reads that got no alignment in unmapped_indices. */
size_t bwt_map_inexact_batch(fastq_batch_t *batch, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                             fastq_batch_t *unmapped_batch, array_list_t *mapping_list);
size_t bwt_map_inexact_array_list(array_list_t *reads, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                                  array_list_t **lists, size_t *num_unmapped, size_t *unmapped_indices);

/* ---- inexact mapping by the k-error block search (bwt.h:559, bwt.c:2313-2797) ----
 * BWSearchCPU on both strands with fragments of max(len / 2, 30) bases (one
 * error), result lists of capacity filter_read_mappings; every result becomes
 * alignments: cigar "<len>=" for exact results, soft clips or M/I/D for
 * one-error ones (bwt.c:2513-2610), 1-based positions, map quality 254 (NM
 * 254 after the optional fields), the query name's first word.  Rows are
 * counted over both strands as l - k per result; past filter_read_mappings
 * the strand's alignments are dropped, the '-' strand is not searched after
 * the '+' one passed, and the list flag becomes 2 (0 again when alignments
 * remain).  Alignments closer than 10 bp on one chromosome are merged.  When
 * the list ends empty with flag 1, the block anchors that touch a read end are
 * located as bwt_anchor_t items (at most 50 rows each).  Reads shorter than 5
 * bases get one unmapped record.  A negative filter_read_mappings exits, as
 * the reference's list allocation does. */
size_t bwt_map_inexact_read_2(fastq_read_t *read, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                              array_list_t *mapping_list);
/* No counterpart in the reference: reads[i] (fastq_read_t *) mapped as
 * bwt_map_inexact_read_2 maps it into lists[i], all reads in one GPU pass;
 * unmapped_indices lists the reads that got no alignment. */
size_t bwt_map_inexact_array_list_2(array_list_t *reads, bwt_optarg_t *bwt_optarg, bwt_index_t *index,
                                    array_list_t **lists, size_t *num_unmapped, size_t *unmapped_indices);

#ifdef __cplusplus
}
#endif

#endif /* HPG_BWT_API_H */
